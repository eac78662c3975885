"""Batched ensembles: members of uneven size stepped in the same launches must each equal the
same simulation run alone (and the oracle) bit for bit, with their own dt, time and status."""
import numpy as np
import pytest

from cuteflow_gb300 import _abi, cases

pytestmark = pytest.mark.gpu


def _members():
    out = []
    for i, (nx, ny) in enumerate([(30, 12), (55, 20), (18, 9), (70, 31), (40, 40)]):
        c = cases.flooding(nx, ny, seed=20 + i, lx=2.0 * nx * 10, ly=2.0 * ny * 10, iflux=3)
        c.params["debitglob"] = [(2.0 + 3 * i) * 20.0 * ny]
        out.append(c)
    return out


def test_batch_members_equal_single_runs(gpu_lib, oracle):
    from cuteflow_gb300 import Batch, Solver
    ms = _members()
    with Batch(ms) as b:
        for i, c in enumerate(ms):
            b.set_state(i, c.U0)
        infos = b.step(120)
        infos2 = b.step(33)
        got = [b.get_state(i) for i in range(len(ms))]
    for i, c in enumerate(ms):
        with Solver(c) as s:
            s.set_state(c.U0)
            s.step(153)
            single = s.get_state()
        ref = oracle.run(c, 153)
        assert np.array_equal(got[i], single), i
        assert np.array_equal(got[i], ref["U"]), i
        assert infos2[i].steps == 153 and infos2[i].t == ref["t"]
    # members have their own dt
    assert len({round(i.dt_last, 12) for i in infos2}) > 1


def test_batch_members_set_at_different_times(gpu_lib, oracle):
    from cuteflow_gb300 import Batch
    ms = _members()[:3]
    with Batch(ms) as b:
        b.set_state(0, ms[0].U0)
        b.set_state(1, ms[1].U0)
        b.step(7)                       # member 2 has no state yet: it does not step
        assert b.info(2).steps == 0
        b.set_state(2, ms[2].U0, t0=1.5)  # set at an odd buffer parity
        b.step(40)
        s0, s1, s2 = b.get_state(0), b.get_state(1), b.get_state(2)
        i2 = b.info(2)
    assert np.array_equal(s0, oracle.run(ms[0], 47)["U"])
    assert np.array_equal(s1, oracle.run(ms[1], 47)["U"])
    r2 = oracle.run(ms[2], 40, t0=1.5)
    assert np.array_equal(s2, r2["U"]) and i2.t == r2["t"] and i2.steps == 40


def test_batch_member_stop_does_not_stop_others(gpu_lib, oracle):
    """A member whose dt leaves the reference's range stops with its state; the others go on."""
    from cuteflow_gb300 import Batch
    bad = cases.flooding(40, 20, seed=8, iflux=3)
    good = cases.flooding(30, 15, seed=9, iflux=3)
    with Batch([bad, good], [dict(fricimplic=0), None]) as b:
        b.set_state(0, bad.U0)
        b.set_state(1, good.U0)
        infos = b.step(150, check=False)
        assert infos[0].status & _abi.CF_STATUS_DT_RANGE and infos[1].status == 0
        sb, sg = b.get_state(0), b.get_state(1)
    rb = oracle.run(bad, 150, params=dict(fricimplic=0), check=False)
    assert rb["rc"] == -2 and np.array_equal(sb, rb["U"])
    assert np.array_equal(sg, oracle.run(good, 150)["U"])


def test_batch_mixed_first_order_schemes_rejected(gpu_lib):
    from cuteflow_gb300 import Batch, CFError
    a = cases.circular_dam_break(10, 10, seed=1, iflux=1)
    b = cases.circular_dam_break(10, 10, seed=2, iflux=3)
    with pytest.raises(CFError):
        Batch([a, b])


def test_batch_run_until_ts(gpu_lib, oracle):
    """cf_run on a batch: every member stops at its own step (its own dt sequence), the others
    going on in the same launches."""
    from cuteflow_gb300 import Batch
    ms = [cases.channel(nx=40 + 10 * i, ny=10, seed=30 + i, q=0.5 + 0.4 * i) for i in range(3)]
    tol = float(np.float32(1e-6))
    want = []
    for c in ms:
        r = oracle.run(c, 1500)
        tc, k = 0.0, 0
        while tc - 50.0 + 2 * tol < tol:
            k += 1
            tc = tc + r["dt_hist"][k]
        want.append(k)
    with Batch(ms) as b:
        for i, c in enumerate(ms):
            b.set_state(i, c.U0)
        infos = b.run(50.0)
        got = [b.get_state(i) for i in range(len(ms))]
    assert len(set(want)) > 1
    for i, c in enumerate(ms):
        assert infos[i].steps == want[i] and infos[i].status & _abi.CF_STATUS_END
        assert np.array_equal(got[i], oracle.run(c, want[i])["U"])
