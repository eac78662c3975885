"""GPU step against the CPU oracle on the same seeded inputs (called through the C ABI).

Tolerance: the benchmark spec's bound, max |h - h_oracle| <= 1e-9 m and |hu|, |hv| <= 1e-9 m^2/s
after the stated step count; the time after the steps must agree to 1e-12 relative.
"""
import numpy as np
import pytest

from cuteflow_gb300 import cases

pytestmark = pytest.mark.gpu

TOL = 1e-9


def run_gpu(case, nsteps, params=None, U0=None, chunks=1):
    from cuteflow_gb300 import Solver
    with Solver(case, params) as s:
        s.set_state(case.U0 if U0 is None else U0)
        per = nsteps // chunks
        info = None
        done = 0
        while done < nsteps:
            k = min(per, nsteps - done)
            info = s.step(k)
            done += k
        return s.get_state(), info


def compare(case, nsteps, oracle, params=None, tol=TOL, chunks=1):
    U, info = run_gpu(case, nsteps, params, chunks=chunks)
    ref = oracle.run(case, nsteps, params=params)
    d = np.abs(U - ref["U"]).max(axis=0)
    assert info.steps == nsteps
    assert abs(info.t - ref["t"]) <= 1e-12 * max(1.0, abs(ref["t"])), (info.t, ref["t"])
    assert d[0] <= tol and d[1] <= tol and d[2] <= tol, (case.name, d)
    return U, ref, info


@pytest.mark.parametrize("iflux", [1, 2])
def test_first_order_dam_break(gpu_lib, oracle, iflux):
    c = cases.circular_dam_break(40, 40, seed=3, iflux=iflux)
    compare(c, 200, oracle)


@pytest.mark.parametrize("iflux", [1, 2, 3])
def test_flooding_wet_dry(gpu_lib, oracle, iflux):
    c = cases.flooding(80, 40, seed=4, iflux=iflux)
    compare(c, 300, oracle, chunks=3)


@pytest.mark.parametrize("ilim", [0, 1, 2, 3, 4])
def test_waf_limiters(gpu_lib, oracle, ilim):
    c = cases.flooding(60, 30, seed=6, iflux=3)
    compare(c, 200, oracle, params=dict(ilimiteur=ilim))


@pytest.mark.parametrize("iflux", [1, 3])
def test_conservative_mode(gpu_lib, oracle, iflux):
    c = cases.flooding(60, 30, seed=7, iflux=iflux)
    compare(c, 200, oracle, params=dict(flux_mode=1))


@pytest.mark.parametrize("fricimplic", [0, 1, 2])
def test_friction_modes(gpu_lib, oracle, fricimplic):
    c = cases.flooding(50, 25, seed=8, iflux=1)
    compare(c, 150, oracle, params=dict(fricimplic=fricimplic))


def test_lake_at_rest(gpu_lib, oracle):
    c = cases.lake_at_rest(40, 20, iflux=3)
    U, ref, info = compare(c, 200, oracle)
    from oracle import oracle as O
    zm = O.setup(c)[2]
    eta = U[:, 0] + zm
    assert np.ptp(eta) < 1e-12
    assert np.abs(U[:, 1:]).max() < 1e-12


def test_config1_circular_dam_break_full(gpu_lib, oracle):
    """80,000 triangles, HLLC, 500 steps (the CPU-runnable benchmark case)."""
    c = cases.circular_dam_break(200, 200, seed=1, iflux=1)
    U, ref, info = compare(c, 500, oracle)
    from oracle import oracle as O
    area = O.setup(c)[1]
    m0 = float((c.U0[:, 0] * area).sum())
    m1 = float((U[:, 0] * area).sum())
    assert abs(m1 - m0) <= 1e-12 * m0
