"""Golden vectors produced by the reference itself (tests/golden/, see make_golden.py): its
boundary tables for two real CGNS calibration meshes, and the logs of three of its runs
(outflow discharge and time every 1000 steps, Tesla P100, IFLUX 2, friction, inflow and
fixed-level outflow)."""
import numpy as np
import pytest

import golden_cases as G
from cuteflow_gb300 import solver


@pytest.mark.parametrize("name", ["river_piers", "divergent_canal"])
def test_boundary_table_matches_reference(name, oracle):
    c, _, _, d = G.case(name, "" if name == "river_piers" else "min")
    ref = G.reference_table(d)
    assert np.array_equal(solver.mesh_tables(c)[0], ref)
    assert np.array_equal(oracle.setup(c)[0], ref)


def test_cfl_length_matches_log(oracle):
    c, _, log, _ = G.case("river_piers")
    assert float(oracle.setup(c)[3].min()) == pytest.approx(float(log["log_cotemin"]), rel=1e-15)


@pytest.mark.parametrize("name,tag", G.RUNS)
def test_oracle_reproduces_reference_log(name, tag, oracle):
    """The outflow discharge printed every 1000 steps is reproduced to the printed 16 digits
    (1e-13 relative allowed); the printed time is t_used + (dt1 - dt0) up to 1e-4 s, because the
    reference adds an asynchronously copied dt on the host (finite_volumes_method.cuf:232,
    cfl_condition.cuf:126): at the first step the copy had already delivered the new dt."""
    c, ic, log, _ = G.case(name, tag)
    U = oracle.initial_condition(c, ic)
    nck = 8
    r = oracle.run(c, 1000 * nck, U0=U)
    dts = r["dt_hist"]
    U, t = U, 0.0
    for k in range(nck):
        rk = oracle.run(c, 1000, U0=U, t0=t)
        U, t = rk["U"], rk["t"]
        assert rk["q_out"] == pytest.approx(float(log["log_q_out"][k]), rel=1e-13)
        assert rk["q_in"] == pytest.approx(float(log["log_q_in"][k]), rel=1e-13)
        assert abs(t + (dts[1] - dts[0]) - float(log["log_t"][k])) < 1e-4
