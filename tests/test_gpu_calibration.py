"""The Manning calibration workload's gradient at its stated size against central differences.

Case (cases.calibration()): 500x200 quads = 200,000 triangles with the circular dam break's flat bed
and walls, first-order HLLC, a true Manning field piecewise constant over 12 seeded Voronoi zones,
40 seeded gauges whose free-surface elevation is observed every 10 s of simulated time, 3000 steps.
The objective is J = sum over the observations of (eta - eta_obs)^2, the gradient is taken at the
calibration's initial guess n = 0.035 by the discrete adjoint, and every finite difference replays
the recorded dt sequence (the adjoint holds dt fixed).

  - every one of the 12 zones has a non-zero gradient;
  - the 12 zone gradients agree with central differences of the GPU forward, step 1e-6 relative
    (1e-6 * 0.035 on every element of the zone), to 1e-5 relative;
  - 20 seeded random elements agree with central differences of the GPU forward to 1e-5 relative
    where the gradient is resolvable (|g| above 1e-8 in absolute terms, against zone gradients of
    order 1-500), and to 1e-8 absolute elsewhere (elements whose influence on the gauges is below
    FP64 resolution).  The element step is 1e-5 relative: a 1e-6 relative change of one element's
    n of 200,000 moves the gauge elevations by ~1e-12 relative, ~5000 units in the last place, so
    central differences at that step resolve the derivative only to ~2e-5 (measured on this case:
    at most 2.5e-5; at 1e-5 at most 3.4e-6);
  - the zone of the largest gradient (step 1e-6) and the two elements of the largest gradients
    among the 20 (step 1e-5) agree with central differences of the CPU oracle's forward (the
    restatement of the reference step, replaying the same dt sequence) to 1e-5 relative.
"""
import numpy as np
import pytest

from cuteflow_gb300 import cases

pytestmark = pytest.mark.gpu

STEPS = 3000
OBS_EVERY = 10.0
N0 = 0.035


@pytest.fixture(scope="module")
def calib(gpu_lib):
    from cuteflow_gb300 import Solver
    from cuteflow_gb300.adjoint import Adjoint
    c, zones, nz, gauges = cases.calibration()
    s = Solver(c)
    adj = Adjoint(s, STEPS, gauges, 0, budget_bytes=64 << 30)
    s.set_manning(c.manning)
    s.set_state(c.U0)
    eta_obs, _ = adj.forward()
    dt_t, t_t = adj.dt_history()
    obs = cases.observation_steps(t_t, dt_t, OBS_EVERY)
    n0 = np.full(c.nelt, N0)
    s.set_manning(n0)
    s.set_state(c.U0)
    eta0, _ = adj.forward()
    dt, t = adj.dt_history()
    r = eta0[obs] - eta_obs[obs]
    w = np.zeros_like(eta0)
    w[obs] = 2.0 * r
    _, gn = adj.backward(w)
    gz = np.array([gn[zones == z].sum() for z in range(nz.size)])
    rng = np.random.default_rng(17)
    elems = rng.choice(c.nelt, 20, replace=False)

    def dJ_gpu(n_plus, n_minus):
        """J(n_plus) - J(n_minus) on the recorded dt sequence, formed per observation as
        (e+ - e-)(e+ + e- - 2 obs) so that the difference does not cancel in the sums."""
        out = []
        for n in (n_plus, n_minus):
            s.set_manning(n)
            s.set_state(c.U0)
            e, _ = adj.forward(replay=True)
            out.append(e[obs])
        ep, em = out
        return float(np.sum((ep - em) * (ep + em - 2.0 * eta_obs[obs])))

    yield dict(c=c, zones=zones, nz=nz, gauges=gauges, obs=obs, eta_obs=eta_obs, dt=dt, t=t, gn=gn, gz=gz,
               elems=elems, dJ_gpu=dJ_gpu, n0=n0)
    adj.close()
    s.close()


def test_every_zone_is_observable(calib):
    gz = calib["gz"]
    assert calib["obs"].size >= 4
    assert np.all(gz != 0.0) and np.all(np.isfinite(gz))


def test_zone_gradients_match_central_differences_of_the_gpu_forward(calib):
    zones, gz, n0 = calib["zones"], calib["gz"], calib["n0"]
    d = 1e-6 * N0
    worst = 0.0
    for z in range(gz.size):
        fd = calib["dJ_gpu"](np.where(zones == z, N0 + d, n0), np.where(zones == z, N0 - d, n0)) / (2.0 * d)
        rel = abs(fd - gz[z]) / abs(gz[z])
        worst = max(worst, rel)
        assert rel <= 1e-5, (z, gz[z], fd, rel)
    print(f"zones: worst relative difference {worst:.2e}")


def test_element_gradients_match_central_differences_of_the_gpu_forward(calib):
    gn, n0 = calib["gn"], calib["n0"]
    d = 1e-5 * N0
    resolved = 0
    for e in calib["elems"]:
        n_p, n_m = n0.copy(), n0.copy()
        n_p[e] += d
        n_m[e] -= d
        fd = calib["dJ_gpu"](n_p, n_m) / (2.0 * d)
        if abs(gn[e]) > 1e-8:
            resolved += 1
            assert abs(fd - gn[e]) <= 1e-5 * abs(gn[e]), (e, gn[e], fd)
        else:
            assert abs(fd - gn[e]) <= 1e-8, (e, gn[e], fd)
    assert resolved >= 10


def _oracle_eta(oracle, c, n, dt, t, obs, gauges):
    """The oracle's gauge elevations after the observed steps, replaying dt (segments between
    observations; the bed is flat, z = 0, so eta = h)."""
    import dataclasses
    case = dataclasses.replace(c, manning=n, params={**c.params, "is_override_manning": 0})
    U = c.U0.copy()
    k = 0
    out = []
    for k1 in obs:
        r = oracle.run(case, int(k1 + 1 - k), U0=U, t0=float(t[k]), dt_replay=dt[k:k1 + 1])
        assert r["rc"] in (0, 1) and r["steps"] == k1 + 1 - k
        U = r["U"]
        out.append(U[gauges, 0].copy())
        k = k1 + 1
    return np.array(out)


def test_gradients_match_central_differences_of_the_oracle_forward(calib, oracle):
    c, zones, gz, gn, n0 = calib["c"], calib["zones"], calib["gz"], calib["gn"], calib["n0"]
    obs, gauges, eta_obs = calib["obs"], calib["gauges"], calib["eta_obs"][calib["obs"]]
    assert np.all(c.z == 0.0)

    def dJ(n_plus, n_minus):
        ep = _oracle_eta(oracle, c, n_plus, calib["dt"], calib["t"], obs, gauges)
        em = _oracle_eta(oracle, c, n_minus, calib["dt"], calib["t"], obs, gauges)
        return float(np.sum((ep - em) * (ep + em - 2.0 * eta_obs)))

    z = int(np.argmax(np.abs(gz)))
    d = 1e-6 * N0
    fd = dJ(np.where(zones == z, N0 + d, n0), np.where(zones == z, N0 - d, n0)) / (2.0 * d)
    assert abs(fd - gz[z]) <= 1e-5 * abs(gz[z]), (z, gz[z], fd)
    d = 1e-5 * N0
    for e in sorted(calib["elems"], key=lambda k: -abs(gn[k]))[:2]:
        n_p, n_m = n0.copy(), n0.copy()
        n_p[e] += d
        n_m[e] -= d
        fd = dJ(n_p, n_m) / (2.0 * d)
        assert abs(fd - gn[e]) <= 1e-5 * abs(gn[e]), (e, gn[e], fd)
