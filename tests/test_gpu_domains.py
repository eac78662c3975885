"""A decomposed mesh stepped as separate processes, one part each, through the C ABI's part
contexts (cuteflow_gb300.domains.PartRunner): the send elements first, their states packed into
pinned host memory by the kernel and exchanged over gloo while the GPU updates the interior, the
halo unpacked, the dt the MIN over the ranks, and the phys_inflow inlet sums and the steady-state
discharges assembled from every rank's terms and summed in the undivided step's order.  The parts
run as processes on one GPU (their kernels never wait on one another: the exchange goes through
the host), and every element equals the undivided mesh's run bit for bit, as do the time, the
next dt, the discharges and the step at which the steady-state test stops the run."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

from cuteflow_gb300 import cases, domains

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _case(kind):
    if kind == "flood_waf":
        return cases.flooding(40, 20, seed=4, iflux=3), {}
    if kind == "flood_hllc":
        return cases.flooding(36, 18, seed=5, iflux=1), {}
    if kind == "channel_muscl":
        return cases.channel(nx=40, ny=8, iflux=4), {}
    if kind == "phys_inflow":
        return cases.channel(nx=48, ny=10, iflux=1, inlet=3), {}
    if kind == "phys_inflow_waf":
        return cases.channel(nx=40, ny=10, iflux=3, inlet=3), {}
    if kind == "steady":
        return cases.channel(), dict(tol_reg_perm=1.5, steady_count=30)
    raise KeyError(kind)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, kind, nsteps, port, out):
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    from cuteflow_gb300 import domains as D
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        c, prm = _case(kind)
        r = D.PartRunner(c, world, rank, dist, params=prm)
        r.set_state(np.asarray(c.U0, dtype=np.float64))
        info = r.step(nsteps)
        out.put((rank, r.get_owned_state(), info.t, info.dt_next, info.steps, info.status, info.q_in, info.q_out))
        r.close()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("kind,world,nsteps", [("flood_waf", 2, 40), ("flood_waf", 3, 30), ("flood_hllc", 2, 40),
                                               ("channel_muscl", 2, 30), ("phys_inflow", 2, 60),
                                               ("phys_inflow_waf", 3, 40), ("steady", 2, 400)])
def test_decomposed_processes_equal_the_undivided_run(gpu_lib, kind, world, nsteps):
    from cuteflow_gb300 import Solver
    c, prm = _case(kind)
    with Solver(c, prm) as s:
        s.set_state(c.U0)
        ref_info = s.step(nsteps, check=False)
        ref = s.get_state()
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, kind, nsteps, port, out), daemon=True) for r in range(world)]
    for pr in procs:
        pr.start()
    got = [out.get(timeout=300) for _ in range(world)]
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    parts = domains.partition(c, world, prm)
    U = np.empty_like(ref)
    for rank, Uown, t, dt, steps, status, qi, qo in got:
        U[parts[rank].owned] = Uown
        assert t == ref_info.t and dt == ref_info.dt_next and steps == ref_info.steps, (rank, steps, ref_info.steps)
        assert status == ref_info.status
        if kind in ("steady",):
            assert qi == ref_info.q_in and qo == ref_info.q_out
    assert np.array_equal(U, ref)
    if kind == "steady":
        assert ref_info.status == 4 and ref_info.steps < nsteps   # the steady-state test stopped both runs
