"""The GPU step on the reference's own logged runs (tests/golden/): the outflow and inflow
discharge after every 1000 steps must equal the reference's printed values (1e-13 relative),
and the state must equal the oracle's bit for bit."""
import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,tag", G.RUNS)
def test_gpu_reproduces_reference_log(gpu_lib, oracle, name, tag):
    from cuteflow_gb300 import Solver
    c, ic, log, _ = G.case(name, tag)
    nck = 10
    with Solver(c) as s:
        s.set_initial_condition(ic)
        U0 = s.get_state()
        assert np.array_equal(U0, oracle.initial_condition(c, ic))
        for k in range(nck):
            info = s.step(1000)
            assert info.q_out == pytest.approx(float(log["log_q_out"][k]), rel=1e-13)
            assert info.q_in == pytest.approx(float(log["log_q_in"][k]), rel=1e-13)
        U = s.get_state()
    ref = oracle.run(c, 1000 * nck, U0=U0)
    assert np.array_equal(U, ref["U"])
    assert info.t == ref["t"]
