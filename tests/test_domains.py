"""Domain decomposition (cuteflow_gb300.domains): the partition, and the halo-exchange protocol
run across processes on gloo ranks with the oracle as each rank's step (no GPU), against the
undivided mesh, bit for bit."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

from cuteflow_gb300 import cases, domains, solver

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _case(kind):
    if kind == "flood_waf":
        return cases.flooding(30, 15, seed=4, iflux=3)
    if kind == "flood_hllc":
        return cases.flooding(30, 15, seed=5, iflux=1)
    if kind == "channel_muscl":
        return cases.channel(nx=40, ny=8, iflux=4)
    raise KeyError(kind)


@pytest.mark.parametrize("kind,nparts", [("flood_waf", 3), ("flood_hllc", 4), ("channel_muscl", 2)])
def test_partition_covers_the_mesh_with_exact_neighbourhoods(kind, nparts):
    c = _case(kind)
    parts = domains.partition(c, nparts)
    owned = np.concatenate([p.owned for p in parts])
    assert np.array_equal(np.sort(owned), np.arange(c.nelt))       # every element owned once
    g = solver.mesh_tables(c)
    for p in parts:
        t = solver.mesh_tables(p.case, p.params)
        loc = np.concatenate([p.owned, p.halo])
        for k in (1, 2, 3):                                          # area, bed, CFL length
            assert np.array_equal(t[k][:p.n_owned], g[k][p.owned])
        nb = t[0][:p.n_owned, :, 0]
        mapped = np.where(nb > 0, loc[np.maximum(nb, 1) - 1] + 1, nb)
        assert np.array_equal(mapped, g[0][p.owned, :, 0])          # neighbours and boundary kinds
        assert not np.intersect1d(p.owned, p.halo).size
        for r, (here, there) in p.recv.items():                     # halo sources
            assert np.array_equal(loc[here], parts[r].owned[there])


@pytest.mark.parametrize("kind,nparts", [("flood_waf", 3), ("flood_hllc", 4)])
def test_exchange_plan_sends_exactly_what_the_halos_hold(kind, nparts):
    """The part contexts' plan: an owned element is a send element exactly when another part's halo
    holds it, every part sends each neighbour the elements that neighbour receives, in its order,
    and the halo is the receive side; the whole mesh's inlet and boundary lists partition over the
    parts' own entries."""
    c = _case(kind)
    parts = domains.partition(c, nparts)
    held = set()
    for q in parts:
        for r, (_, there) in q.recv.items():
            held.update((r, int(i)) for i in there)
    g = solver.mesh_tables(c)[0]
    nb_global = len(domains.boundary_entries(g))
    seen = []
    for rank, p in enumerate(parts):
        cls, send_to, recv_from = domains.part_plan(parts, rank)
        assert np.array_equal(np.flatnonzero(cls == 2), p.n_owned + np.arange(p.halo.size))
        for i in range(p.n_owned):
            assert (cls[i] == 1) == ((rank, i) in held)
        for r, ids in send_to.items():
            assert np.array_equal(ids, parts[r].recv[rank][1])
        for r, here in recv_from.items():
            assert np.array_equal(here, p.recv[r][0])
        lb = solver.mesh_tables(p.case, p.params)[0]
        seen += [(int(p.owned[e]), k) for e, k, _ in domains.boundary_entries(lb) if e < p.n_owned]
    assert sorted(seen) == [(e, k) for e, k, _ in domains.boundary_entries(g)] and len(seen) == nb_global


def test_whole_mesh_sums_follow_the_steps_order():
    """inlet_sum is calcul_surf_entree's sum as the step forms it (blocks of 32, tree per block,
    blocks in order) and discharge_sum the discharge sums' (256 strided partial sums of one kind,
    then a tree): exact on integers, and equal to the same orders written out."""
    rng = np.random.default_rng(3)
    v = rng.standard_normal(77)
    blocks = []
    for b in range(0, 77, 32):
        s = list(v[b:b + 32]) + [0.0] * (32 - len(v[b:b + 32]))
        for i in (16, 8, 4, 2, 1):
            s = [s[l] + s[l + i] if l < i else s[l] for l in range(32)]
        blocks.append(s[0])
    total = 0.0
    for x in blocks:
        total = total + x
    assert domains.inlet_sum(v) == total
    assert domains.inlet_sum(np.arange(100.0)) == 4950.0
    q = rng.standard_normal(600)
    kinds = rng.choice([-1, -2, -3], 600)
    part = [0.0] * 256
    for j in range(600):
        if kinds[j] == -2:
            part[j % 256] += q[j]
    w = 128
    while w:
        part = [part[t] + part[t + w] if t < w else part[t] for t in range(256)]
        w //= 2
    assert domains.discharge_sum(q, kinds, -2) == part[0]
    assert domains.discharge_sum(np.ones(600), kinds, -1) == float(np.sum(kinds == -1))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, kind, nsteps, port, out):
    """One rank: its part stepped by the oracle with the global dt, halos exchanged after every
    step (all_gather of the own states), the next dt the MIN over the ranks."""
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    from oracle import oracle as O
    from cuteflow_gb300 import domains as D
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        c = _case(kind)
        p = D.partition(c, world)[rank]

        def global_dt(U):
            d = torch.tensor([O.run(p.case, 0, params=p.params, U0=U)["dt_hist"][0]], dtype=torch.float64)
            dist.all_reduce(d, op=dist.ReduceOp.MIN)
            return float(d.item())

        U = np.array(p.case.U0, dtype=np.float64)
        t = 0.0
        dt = global_dt(U)
        for _ in range(nsteps):
            r = O.run(p.case, 1, params=p.params, U0=U, t0=t, dt_replay=np.array([dt]), check=False)
            U, t = r["U"].copy(), r["t"]
            own = [None] * world
            dist.all_gather_object(own, U[: p.n_owned].copy())
            for src, (here, there) in p.recv.items():
                U[here] = own[src][there]
            dt = global_dt(U)
        out.put((rank, U[: p.n_owned], t, dt))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("kind,world,nsteps", [("flood_waf", 2, 40), ("flood_hllc", 3, 40), ("channel_muscl", 2, 30)])
def test_decomposed_run_over_gloo_ranks_is_the_undivided_run(oracle, kind, world, nsteps):
    c = _case(kind)
    ref = oracle.run(c, nsteps)
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, kind, nsteps, port, out)) for r in range(world)]
    for pr in procs:
        pr.start()
    got = [out.get(timeout=240) for _ in range(world)]
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    parts = domains.partition(c, world)
    U = np.empty_like(ref["U"])
    for rank, Uown, t, dt in got:
        U[parts[rank].owned] = Uown
        assert t == ref["t"]
        assert dt == ref["dt_hist"][nsteps]
    assert np.array_equal(U, ref["U"])
