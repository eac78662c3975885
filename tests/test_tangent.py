"""The step differentiated in forward mode on the CPU (tests/flux_harness.cpp: the GPU step's
templated arithmetic on Dual numbers, replaying a dt sequence) against the CPU oracle: its
value lane is the oracle's replayed run bit for bit, and its tangent is the central difference
of the oracle's replayed run where the run is smooth in the direction taken.  The GPU adjoint
is checked against this tangent (tests/test_gpu_adjoint.py)."""
import numpy as np
import pytest

import adjoint_cases as AC
import harness as H

N = 25


def _direction(c, seed):
    rng = np.random.default_rng(seed)
    wet = c.U0[:, 0] > 0.05
    dU = np.zeros_like(c.U0)
    dU[wet, 0] = 0.01 * rng.uniform(-1.0, 1.0, wet.sum())
    dU[wet, 1:] = 0.01 * rng.uniform(-1.0, 1.0, (wet.sum(), 2))
    dn = c.manning * rng.uniform(-1.0, 1.0, c.nelt)
    return dU, dn


def _gauges(c, seed=7, G=7):
    rng = np.random.default_rng(seed)
    return rng.choice(np.flatnonzero(c.U0[:, 0] > 0.05), G, replace=False)


@pytest.mark.parametrize("kind", AC.ALL_KINDS)
def test_tangent_value_lane_is_the_oracle(oracle, kind):
    c, extra = AC.make(kind)
    dt = oracle.run(c, N, params=extra)["dt_hist"][:N]
    t = AC.times(dt)
    g = _gauges(c)
    zm = oracle.setup(c)[2]
    dU, dn = _direction(c, 1)
    eta, _, U, _ = H.tangent(c, extra, c.U0, dU, c.manning, dn, dt, t, g)
    eta_o, U_o = AC.oracle_run(oracle, c, extra, c.U0, c.manning, dt, t, g, zm)
    assert np.array_equal(U, U_o) and np.array_equal(eta, eta_o)


@pytest.mark.parametrize("kind", AC.FD_KINDS)
def test_tangent_is_the_central_difference(oracle, kind):
    c, extra = AC.make(kind)
    dt = oracle.run(c, N, params=extra)["dt_hist"][:N]
    t = AC.times(dt)
    g = _gauges(c)
    zm = oracle.setup(c)[2]
    rng = np.random.default_rng(3)
    w_eta = rng.standard_normal((N, len(g)))
    w_state = 0.01 * rng.standard_normal((c.nelt, 3))
    dU, dn = _direction(c, 2)
    _, deta, _, dUN = H.tangent(c, extra, c.U0, dU, c.manning, dn, dt, t, g)
    tl = float(np.sum(w_eta * deta) + np.sum(w_state * dUN))
    eps = 1e-6
    Jp = AC.objective(*AC.oracle_run(oracle, c, extra, c.U0 + eps * dU, c.manning + eps * dn, dt, t, g, zm),
                      w_eta, w_state)
    Jm = AC.objective(*AC.oracle_run(oracle, c, extra, c.U0 - eps * dU, c.manning - eps * dn, dt, t, g, zm),
                      w_eta, w_state)
    fd = (Jp - Jm) / (2 * eps)
    assert abs(fd - tl) <= 1e-5 * abs(tl), (fd, tl)
