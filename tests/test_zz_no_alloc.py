"""cf_step_noalloc, the stepping entry point that allocates nothing (its edge-flux scratch is a
static device array of the library), against cf_step through the C ABI.

The two entry points run the same kernels on the same inputs, so the tolerance is the one of
every parity test here: bit for bit.  Each comparison covers two calls in a row.  This file is
collected last so that it also runs after the rest of the GPU suite has used the library.
"""
import numpy as np
import pytest

from cuteflow_gb300 import _abi, cases

pytestmark = pytest.mark.gpu


def _noalloc(lib, obj, nsteps, members=1):
    infos = (_abi.CfStepInfo * members)()
    rc = lib.cf_step_noalloc(obj._ctx, int(nsteps), infos)
    assert rc == 0, lib.cf_last_error(obj._ctx).decode()
    return infos


def _same(info_a, info_b):
    for f in ("t", "dt_last", "dt_next", "q_in", "q_out", "steps", "status"):
        assert getattr(info_a, f) == getattr(info_b, f), f


def _cases():
    flood = cases.flooding(80, 40, seed=7, lx=1600.0, ly=800.0, iflux=3)
    flood.params["debitglob"] = [8.0 * 800.0]
    return [cases.circular_dam_break(60, 60, iflux=1), flood, cases.flooding(50, 30, seed=9, iflux=2)]


@pytest.mark.parametrize("which", [0, 1, 2])
def test_noalloc_equals_cf_step(gpu_lib, which):
    from cuteflow_gb300 import Solver
    c = _cases()[which]
    with Solver(c) as a, Solver(c) as b:
        a.set_state(c.U0)
        b.set_state(c.U0)
        for n in (37, 26):           # two calls in a row (the second starts at odd parity)
            ia = a.step(n)
            ib = _noalloc(gpu_lib, b, n)[0]
            _same(ia, ib)
            assert np.array_equal(a.get_state(), b.get_state())
        if which == 1:
            assert ib.q_in > 0.0   # the discharge diagnostics read the scratch


def test_noalloc_batch_and_shared_scratch(gpu_lib):
    """Members of a batch, and two contexts taking turns on the one shared array."""
    from cuteflow_gb300 import Batch, Solver
    ms = [cases.flooding(30 + 9 * i, 12 + 4 * i, seed=30 + i, lx=600.0 + 180 * i, ly=240.0 + 80 * i, iflux=3)
          for i in range(3)]
    small = cases.circular_dam_break(24, 20, iflux=1)
    with Batch(ms) as a, Batch(ms) as b, Solver(small) as sa, Solver(small) as sb:
        for i, c in enumerate(ms):
            a.set_state(i, c.U0)
            b.set_state(i, c.U0)
        sa.set_state(small.U0)
        sb.set_state(small.U0)
        for n in (41, 18):
            ia = a.step(n)
            ib = _noalloc(gpu_lib, b, n, members=len(ms))
            for i in range(len(ms)):
                _same(ia[i], ib[i])
                assert np.array_equal(a.get_state(i), b.get_state(i)), i
            _same(sa.step(n + 3), _noalloc(gpu_lib, sb, n + 3)[0])
            assert np.array_equal(sa.get_state(), sb.get_state())


def test_noalloc_allocates_no_device_memory(gpu_lib):
    """The property the entry point exists for: once a first call has loaded the library's device
    code and its static array on the device, further calls leave the device's free memory
    (cudaMemGetInfo) exactly where it was."""
    torch = pytest.importorskip("torch")
    from cuteflow_gb300 import Solver
    c = cases.flooding(60, 30, seed=12, iflux=3)
    with Solver(c) as s:
        s.set_state(c.U0)
        _noalloc(gpu_lib, s, 3)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for n in (5, 8, 13):
            _noalloc(gpu_lib, s, n)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0
        assert s.info().steps == 29


def test_noalloc_rejects_a_context_beyond_the_scratch(gpu_lib):
    from cuteflow_gb300 import Solver
    c = cases.circular_dam_break(260, 260, iflux=1)     # 135,200 triangles: about 406,000 slots
    with Solver(c) as s:
        s.set_state(c.U0)
        info = (_abi.CfStepInfo * 1)()
        rc = gpu_lib.cf_step_noalloc(s._ctx, 5, info)
        assert rc == _abi.CF_EINVAL
        assert "static scratch" in gpu_lib.cf_last_error(s._ctx).decode()
        assert s.info().steps == 0                        # nothing ran
        s.step(2)                                         # the context itself is unharmed
        assert s.info().steps == 2

