"""Seeded cases of the adjoint and tangent-linear tests (test infrastructure)."""
import dataclasses

import numpy as np

from cuteflow_gb300 import cases


def with_wave(c, amp=0.25, seed=3):
    """A still-water case with a Gaussian hump on the free surface (waves in a few steps)."""
    rng = np.random.default_rng(seed)
    xc, yc = cases.cell_centroids(c.x, c.y, c.tri)
    x0 = xc.min() + (xc.max() - xc.min()) * rng.uniform(0.3, 0.7)
    y0 = yc.min() + (yc.max() - yc.min()) * rng.uniform(0.3, 0.7)
    r2 = ((xc - x0) ** 2 + (yc - y0) ** 2) / (0.15 * (xc.max() - xc.min())) ** 2
    U0 = c.U0.copy()
    wet = U0[:, 0] > 0.05
    U0[wet, 0] += amp * np.exp(-r2[wet])
    U0[wet, 1] += 0.05 * U0[wet, 0] * rng.standard_normal(wet.sum())
    U0[wet, 2] += 0.05 * U0[wet, 0] * rng.standard_normal(wet.sum())
    return dataclasses.replace(c, U0=U0)


def generic(c, seed):
    """Depth and velocity noise on every clearly wet element.  A state exactly at rest, or with
    a free surface flat to the last bit, sits on kinks and jumps of the scheme (s* = 0 selects
    a region, r = dupw / (dloc + eps) of the WAF limiter is undefined at dloc = 0), where
    central differences do not measure a derivative."""
    rng = np.random.default_rng(seed)
    U0 = c.U0.copy()
    wet = U0[:, 0] > 0.05
    U0[wet, 0] *= 1.0 + 0.02 * rng.standard_normal(wet.sum())
    U0[wet, 1] = U0[wet, 0] * 0.1 * rng.standard_normal(wet.sum())
    U0[wet, 2] = U0[wet, 0] * 0.1 * rng.standard_normal(wet.sum())
    return dataclasses.replace(c, U0=U0)


def make(kind):
    if kind == "hllc_dam":
        c = cases.circular_dam_break(20, 20, iflux=1)
        c.manning = np.linspace(0.02, 0.05, c.nelt)
        return generic(c, 1), {}
    if kind == "riadh_dam":
        c = cases.circular_dam_break(18, 16, iflux=2)
        c.manning = np.linspace(0.05, 0.02, c.nelt)
        return generic(c, 2), {"fricimplic": 2}
    if kind == "waf_flood":
        c = cases.flooding(26, 12, seed=12, lx=520.0, ly=240.0, iflux=3, nbumps=2)
        c.params["debitglob"] = [8.0 * 240.0]
        c.params["ilimiteur"] = 3
        return generic(with_wave(c), 3), {}
    if kind == "waf_explicit":
        c = cases.flooding(22, 10, seed=13, lx=440.0, ly=200.0, iflux=3, nbumps=0)
        c.params["debitglob"] = [6.0 * 200.0]
        c.params["ilimiteur"] = 2
        return generic(with_wave(c, seed=4), 4), {"fricimplic": 0}
    if kind == "hllc_flood":
        c = cases.flooding(26, 12, seed=11, lx=520.0, ly=240.0, iflux=1, nbumps=2)
        c.params["debitglob"] = [8.0 * 240.0]
        return generic(with_wave(c, seed=5), 5), {}
    if kind == "waf_superbee":
        c = cases.flooding(26, 12, seed=12, lx=520.0, ly=240.0, iflux=3, nbumps=2)
        c.params["debitglob"] = [8.0 * 240.0]
        c.params["ilimiteur"] = 1
        return generic(with_wave(c, seed=6), 6), {}
    if kind == "waf_conservative":
        c = cases.flooding(26, 12, seed=12, lx=520.0, ly=240.0, iflux=3, nbumps=2)
        c.params["debitglob"] = [8.0 * 240.0]
        c.params["ilimiteur"] = 4
        return generic(with_wave(c, seed=7), 7), {"flux_mode": 1}
    if kind == "riadh_transm":
        c = cases.flooding(24, 12, seed=11, lx=480.0, ly=240.0, iflux=2, nbumps=1)
        return generic(with_wave(c, seed=8), 8), {"inlet": 1, "outlet": 2}
    raise KeyError(kind)





def objective(eta, UN, w_eta, w_state):
    return float(np.sum(w_eta * eta) + np.sum(w_state * UN))


def times(dt, t0=0.0):
    """Start time of every step: t_{k+1} = t_k + dt_k, as the step accumulates it."""
    t = np.empty(len(dt))
    acc = t0
    for k, d in enumerate(dt):
        t[k] = acc
        acc = acc + d
    return t


def oracle_run(O, c, params, U0, n, dt, t, gauges, zm):
    case = dataclasses.replace(c, manning=n, params={**c.params, **params, "is_override_manning": 0})
    U = U0.copy()
    eta = np.empty((len(dt), len(gauges)))
    for k in range(len(dt)):
        r = O.run(case, 1, U0=U, t0=t[k], dt_replay=dt[k:k + 1])
        U = r["U"]
        eta[k] = U[gauges, 0] + zm[gauges]
    return eta, U


KINDS = ["hllc_dam", "riadh_dam", "waf_flood", "waf_explicit", "hllc_flood"]
# cases where the run is smooth along the test directions (central differences are valid)
FD_KINDS = ["hllc_dam", "riadh_dam", "waf_flood", "hllc_flood"]
ALL_KINDS = KINDS + ["waf_superbee", "waf_conservative", "riadh_transm"]
