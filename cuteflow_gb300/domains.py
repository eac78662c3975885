"""Domain decomposition of one mesh: parts with halos, halo exchange and the global dt.

The reference runs a mesh larger than one GPU as MPI ranks over pre-partitioned meshes with ghost
elements (maillage.cuf:196-396 reads the ghost blocks; finite_volumes_method.cuf:53-78, 141-171
exchanges them every step; memory_exchange_functions.cuf:129-172), and takes the minimum dt over
the ranks (MPI_ALLREDUCE MIN, :113-116, cfl_condition.cuf:117-126).  Here:

  partition(case, nparts)  splits the elements into spatially contiguous parts (Morton order of
                           the centroids, balanced counts); every part is a mesh of its own
                           elements followed by a halo of the neighbours' elements: one ring of
                           edge neighbours, two for iflux 3 and 4 (their upwind states read the
                           neighbours' neighbours), so every own element sees exactly its
                           neighbourhood in the whole mesh.  The part's parameters carry the whole
                           mesh's inlet lengths and element count (cf_params long_entree,
                           dt_reset_nelt).
  Decomposed(parts)        steps the parts as separate contexts: after every step the owners'
                           states are copied into the halos (cf_get_elements / cf_set_elements,
                           host-staged) and the minimum of the parts' next dt is applied to all
                           (cf_set_dt).  Every element evolves bit for bit as in the undivided mesh.

The same exchange protocol runs across processes (one rank per part, torch.distributed): the tests
run it with the oracle as the step on gloo ranks.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional

import numpy as np

from . import cases as _cases
from .solver import Solver, mesh_tables


def _morton(xc: np.ndarray, yc: np.ndarray, bits: int = 16) -> np.ndarray:
    """Morton (Z-order) key of the centroids on a 2^bits grid."""
    def spread(v):
        v = v.astype(np.uint64)
        out = np.zeros_like(v)
        for b in range(bits):
            out |= ((v >> np.uint64(b)) & np.uint64(1)) << np.uint64(2 * b)
        return out
    span = max(xc.max() - xc.min(), yc.max() - yc.min(), 1e-300)
    scale = (2 ** bits - 1) / span
    ix = np.floor((xc - xc.min()) * scale).astype(np.int64)
    iy = np.floor((yc - yc.min()) * scale).astype(np.int64)
    return spread(ix) | (spread(iy) << np.uint64(1))


def inlet_lengths(case, bnd: np.ndarray) -> List[float]:
    """calcul_long_entree (maillage.cuf:1423-1452) on the whole mesh: per inlet number, the sum of
    its inflow edges' lengths in element then edge order (the host preprocessing's sum)."""
    tri = np.asarray(case.tri).reshape(-1, 3) - 1
    x, y = np.asarray(case.x, dtype=np.float64), np.asarray(case.y, dtype=np.float64)
    out = [0.0] * 20
    for e, k in zip(*np.nonzero(bnd[:, :, 0] == -1)):
        a, b = int(tri[e, k]), int(tri[e, (k + 1) % 3])
        dx, dy = float(x[a]) - float(x[b]), float(y[a]) - float(y[b])
        i = int(bnd[e, k, 1]) - 1
        if 0 <= i < 20:
            out[i] = out[i] + math.sqrt(dx * dx + dy * dy)
    return out


@dataclasses.dataclass
class Part:
    case: object            # the part's mesh: own elements first, then the halo
    params: dict            # the case's parameters with the whole mesh's inlet lengths and size
    owned: np.ndarray       # global element ids of the own elements (local ids 0..n_owned-1)
    halo: np.ndarray        # global element ids of the halo (local ids n_owned..)
    recv: Dict[int, tuple]  # owner part -> (local halo ids here, local own ids there)

    @property
    def n_owned(self) -> int:
        return int(self.owned.size)


def partition(case, nparts: int, params: Optional[dict] = None, rings: Optional[int] = None) -> List[Part]:
    prm = {**getattr(case, "params", {}), **(params or {})}
    if rings is None:
        rings = 2 if int(prm.get("iflux", 1)) >= 3 else 1
    bnd = mesh_tables(case, params)[0]
    n = bnd.shape[0]
    nbr = bnd[:, :, 0]
    tri = np.asarray(case.tri).reshape(-1, 3)
    xc, yc = _cases.cell_centroids(case.x, case.y, tri)
    order = np.argsort(_morton(xc, yc), kind="stable")
    owner = np.empty(n, dtype=np.int64)
    chunks = np.array_split(order, nparts)
    for q, ch in enumerate(chunks):
        owner[ch] = q
    lengths = inlet_lengths(case, bnd)
    prm_part = {**prm, "long_entree": lengths, "dt_reset_nelt": n}
    parts = []
    for q, ch in enumerate(chunks):
        owned = np.sort(ch)
        mine = np.zeros(n, dtype=bool)
        mine[owned] = True
        halo_mask = np.zeros(n, dtype=bool)
        frontier = owned
        for _ in range(rings):
            nb = nbr[frontier].ravel()
            nb = nb[nb > 0] - 1
            new = np.unique(nb[~mine[nb] & ~halo_mask[nb]])
            halo_mask[new] = True
            frontier = new
        halo = np.flatnonzero(halo_mask)
        local = np.concatenate([owned, halo])
        nodes = np.unique(tri[local].ravel())          # 1-based node ids
        node_map = np.zeros(len(case.x) + 1, dtype=np.int64)
        node_map[nodes] = np.arange(1, nodes.size + 1)

        def keep(lst, num):
            lst = np.asarray(lst, dtype=np.int64)
            m = node_map[lst] > 0 if lst.size else np.zeros(0, bool)
            return node_map[lst[m]].astype(np.int32), np.asarray(num)[m].astype(np.int32)

        ndin, numin = keep(case.ndinput, case.numero_ndinput)
        ndout, numout = keep(case.ndoutput, case.numero_ndoutput)
        ndw, _ = keep(case.ndwall, np.zeros(len(case.ndwall), np.int32))
        sub = _cases.Case(x=np.asarray(case.x)[nodes - 1], y=np.asarray(case.y)[nodes - 1],
                          z=np.asarray(case.z)[nodes - 1], tri=node_map[tri[local]].astype(np.int32),
                          manning=np.asarray(case.manning)[local], ndinput=ndin, numero_ndinput=numin,
                          ndoutput=ndout, numero_ndoutput=numout, ndwall=ndw,
                          nombre_entrees=case.nombre_entrees, nombre_sorties=case.nombre_sorties,
                          params=dict(prm_part), U0=np.asarray(case.U0)[local],
                          name=f"{getattr(case, 'name', 'case')}_part{q}of{nparts}")
        parts.append(Part(case=sub, params=dict(prm_part), owned=owned, halo=halo, recv={}))
    # exchange plan: halo element g of part q comes from part owner[g] at its own local id
    pos = np.empty(n, dtype=np.int64)
    for p in parts:
        pos[p.owned] = np.arange(p.n_owned)
    for q, p in enumerate(parts):
        src = owner[p.halo]
        for r in np.unique(src):
            sel = np.flatnonzero(src == r)
            p.recv[int(r)] = ((p.n_owned + sel).astype(np.int32), pos[p.halo[sel]].astype(np.int32))
    return parts


class Decomposed:
    """The parts of a decomposed mesh as separate contexts on this process's GPU, with the halo
    exchange and the global dt after every step (host-staged)."""

    def __init__(self, parts: List[Part]):
        self.parts = parts
        self.solvers = [Solver(p.case, p.params) for p in parts]
        self.n = int(sum(p.n_owned for p in parts))

    def close(self):
        for s in self.solvers:
            s.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _global_dt(self):
        dt = min(s.info().dt_next for s in self.solvers)
        for s in self.solvers:
            s.set_dt(dt)
        return dt

    def exchange(self):
        for s, p in zip(self.solvers, self.parts):
            ids, vals = [], []
            for r, (here, there) in p.recv.items():
                ids.append(here)
                vals.append(self.solvers[r].get_elements(there))
            if ids:
                s.set_elements(np.concatenate(ids), np.concatenate(vals))
            else:
                s.set_elements(np.zeros(0, np.int32), np.zeros((0, 3)))
        return self._global_dt()

    def set_state(self, U: np.ndarray, t0: float = 0.0):
        for s, p in zip(self.solvers, self.parts):
            s.set_state(U[np.concatenate([p.owned, p.halo])], t0)
        self._global_dt()

    def step(self, nsteps: int):
        info = None
        for _ in range(nsteps):
            for s in self.solvers:
                info = s.step(1)
            self.exchange()
        return info

    def get_state(self) -> np.ndarray:
        U = np.empty((self.n, 3))
        for s, p in zip(self.solvers, self.parts):
            U[p.owned] = s.get_state()[: p.n_owned]
        return U


# ---- the decomposed run as a data plane: one process per part ------------------------------------

def inlet_entries(bnd: np.ndarray) -> List[tuple]:
    """The phys_inflow entry list of a mesh (compute_input_elems, maillage.cuf:1333-1363): one entry
    per (element, inflow edge) in element then local-edge order."""
    e, k = np.nonzero(bnd[:, :, 0] == -1)
    return list(zip(e.tolist(), k.tolist()))


def boundary_entries(bnd: np.ndarray) -> List[tuple]:
    """The boundary edges of a mesh in element then local-edge order, with their kinds."""
    e, k = np.nonzero(bnd[:, :, 0] < 0)
    return list(zip(e.tolist(), k.tolist(), bnd[e, k, 0].tolist()))


def inlet_sum(values: np.ndarray) -> float:
    """calcul_surf_entree's sum as the step forms it (k_surf): blocks of 32 entries in list order,
    each summed by the tree s[l] += s[l + i] (i = 16 .. 1), the block sums added in order."""
    total = 0.0
    n = len(values)
    for b in range(0, n, 32):
        s = [float(values[b + l]) if b + l < n else 0.0 for l in range(32)]
        i = 16
        while i > 0:
            for l in range(i):
                s[l] = s[l] + s[l + i]
            i >>= 1
        total = total + s[0]
    return total


def discharge_sum(q: np.ndarray, kinds: np.ndarray, kind: int) -> float:
    """The discharge sums as the step forms them (k_discharge): over the boundary edges in
    reference order, 256 strided partial sums of the edges of one kind, then a fixed tree."""
    part = [0.0] * 256
    for j in range(len(q)):
        if kinds[j] == kind:
            t = j % 256
            part[t] = part[t] + float(q[j])
    w = 128
    while w > 0:
        for t in range(w):
            part[t] = part[t] + part[t + w]
        w >>= 1
    return part[0]


def part_plan(parts: List[Part], rank: int):
    """The exchange plan of part `rank`: its element classes for cf_create_part (0 owned interior,
    1 owned and held in another part's halo, 2 halo), the own elements it sends to each other part
    (local ids, in that part's receive order) and the halo elements it receives from each (local
    ids)."""
    p = parts[rank]
    cls = np.zeros(p.n_owned + p.halo.size, dtype=np.int32)
    cls[p.n_owned:] = 2
    send_to = {}
    for r, q in enumerate(parts):
        if r != rank and rank in q.recv:
            ids = q.recv[rank][1]
            send_to[r] = ids
            cls[ids] = 1
    recv_from = {r: here for r, (here, _) in sorted(p.recv.items())}
    return cls, send_to, recv_from


class PartRunner:
    """Part `rank` of a decomposed mesh stepped by this process (one rank per part) on its GPU,
    the reference's send-cells-first scheme (finite_volumes_method.cuf:141-171,
    memory_exchange_functions.cuf:129-172) as a data plane:

      - the part's context (cf_create_part) orders its elements send, interior, halo;
      - each step (cf_part_step_begin) updates the send elements first and packs their states
        straight into a pinned host buffer (the kernel writes it over the CPU link), then updates
        the interior elements while this process exchanges the halo with its neighbour ranks over
        `comm` (torch.distributed point-to-point); cf_part_step_end unpacks the received halo;
      - the next dt is the MIN over the ranks (MPI_ALLREDUCE MIN, cfl_condition.cuf:117-126);
      - phys_inflow's inlet sums and the discharges of the steady-state test are the whole
        mesh's: every rank places its own elements' terms at their positions in the whole mesh's
        lists, a SUM all-reduce assembles the lists (each position has one contributor, so the
        sum is exact), and every rank sums them in the undivided step's order.
    Every element evolves bit for bit as in the undivided mesh."""

    def __init__(self, case, nparts: int, rank: int, comm, params: Optional[dict] = None):
        import torch
        self.comm = comm
        self.rank = rank
        self.parts = partition(case, nparts, params)
        p = self.parts[rank]
        self.part = p
        cls, self.send_to, self.recv_from = part_plan(self.parts, rank)
        self.solver = Solver(p.case, p.params, elem_class=cls)
        L, ctx = self.solver._L, self.solver._ctx
        send = np.concatenate([self.send_to[r] for r in sorted(self.send_to)]).astype(np.int32) \
            if self.send_to else np.zeros(0, np.int32)
        recv = np.concatenate([self.recv_from[r] for r in sorted(self.recv_from)]).astype(np.int32) \
            if self.recv_from else np.zeros(0, np.int32)
        ip = __import__("ctypes").POINTER(__import__("ctypes").c_int32)
        self.solver._check(L.cf_part_set_exchange(ctx, send.ctypes.data_as(ip), int(send.size),
                                                  recv.ctypes.data_as(ip), int(recv.size)))
        self.sendbuf = torch.zeros(max(3 * send.size, 1), dtype=torch.float64).pin_memory()
        self.recvbuf = torch.zeros(max(3 * recv.size, 1), dtype=torch.float64).pin_memory()
        self._send_slices, off = {}, 0
        for r in sorted(self.send_to):
            n = 3 * self.send_to[r].size
            self._send_slices[r] = (off, off + n)
            off += n
        self._recv_slices, off = {}, 0
        for r in sorted(self.recv_from):
            n = 3 * self.recv_from[r].size
            self._recv_slices[r] = (off, off + n)
            off += n
        # the whole mesh's inlet and boundary lists, and this part's entries in them
        prm = {**getattr(case, "params", {}), **(params or {})}
        gb = mesh_tables(case, params)[0]
        lb = mesh_tables(p.case, p.params)[0]
        self.phys_inflow = int(prm.get("inlet", 2)) == 3
        self.steady = float(prm.get("tol_reg_perm", 0.0)) > 0.0
        self.nin = int(case.nombre_entrees)
        gi = {ek: j for j, ek in enumerate(inlet_entries(gb))}
        self.n_inlet = len(gi)
        li = inlet_entries(lb)
        self.inlet_map = [(j, gi[(int(p.owned[e]), k)]) for j, (e, k) in enumerate(li) if e < p.n_owned]
        gq = boundary_entries(gb)
        self.q_kinds = np.array([kd for _, _, kd in gq], dtype=np.int64)
        gpos = {(e, k): j for j, (e, k, _) in enumerate(gq)}
        lq = boundary_entries(lb)
        self.n_local_q = len(lq)
        self.q_map = [(j, gpos[(int(p.owned[e]), k)]) for j, (e, k, _) in enumerate(lq) if e < p.n_owned]

    # -- collectives over the ranks --
    def _allreduce(self, t, op):
        self.comm.all_reduce(t, op=op)
        return t

    def _global_dt(self, dt_part: float) -> float:
        import torch
        t = torch.tensor([dt_part], dtype=torch.float64)
        return float(self._allreduce(t, self.comm.ReduceOp.MIN).item())

    def set_state(self, U: np.ndarray, t0: float = 0.0):
        p = self.part
        self.solver.set_state(U[np.concatenate([p.owned, p.halo])], t0)
        self.solver.set_dt(self._global_dt(self.solver.info().dt_next))

    def _inlet_sums(self):
        import torch
        L, ctx = self.solver._L, self.solver._ctx
        n_local = len(inlet_entries(mesh_tables(self.part.case, self.part.params)[0])) if not hasattr(self, "_n_li") \
            else self._n_li
        self._n_li = n_local
        terms = np.zeros(max(n_local * self.nin, 1))
        dp = __import__("ctypes").POINTER(__import__("ctypes").c_double)
        self.solver._check(L.cf_part_inlet_terms(ctx, terms.ctypes.data_as(dp)))
        G = torch.zeros((max(self.n_inlet, 1), self.nin), dtype=torch.float64)
        tv = terms[: n_local * self.nin].reshape(n_local, self.nin) if n_local else np.zeros((0, self.nin))
        for j, g in self.inlet_map:
            G[g] = torch.from_numpy(tv[j].copy())
        self._allreduce(G, self.comm.ReduceOp.SUM)
        Gn = G.numpy()
        surf = np.array([inlet_sum(Gn[: self.n_inlet, i]) for i in range(self.nin)] + [0.0] * (20 - self.nin))
        self.solver._check(L.cf_part_set_inlet_sums(ctx, surf.ctypes.data_as(dp)))

    def _discharges(self):
        import torch
        L, ctx = self.solver._L, self.solver._ctx
        dp = __import__("ctypes").POINTER(__import__("ctypes").c_double)
        terms = np.zeros(max(self.n_local_q, 1))
        self.solver._check(L.cf_part_discharge_terms(ctx, terms.ctypes.data_as(dp)))
        G = torch.zeros(max(self.q_kinds.size, 1), dtype=torch.float64)
        for j, g in self.q_map:
            G[g] = float(terms[j])
        self._allreduce(G, self.comm.ReduceOp.SUM)
        q = G.numpy()[: self.q_kinds.size]
        qi, qo = discharge_sum(q, self.q_kinds, -1), discharge_sum(q, self.q_kinds, -2)
        self.solver._check(L.cf_part_apply_discharges(ctx, qi, qo))

    def _exchange(self):
        reqs = []
        for r, (a, b) in self._recv_slices.items():
            reqs.append(self.comm.irecv(self.recvbuf[a:b], src=r))
        for r, (a, b) in self._send_slices.items():
            reqs.append(self.comm.isend(self.sendbuf[a:b], dst=r))
        for q in reqs:
            q.wait()

    def step(self, nsteps: int = 1):
        import ctypes
        from . import _abi
        L, ctx = self.solver._L, self.solver._ctx
        info = _abi.CfStepInfo()
        for _ in range(nsteps):
            if self.phys_inflow:
                self._inlet_sums()
            self.solver._check(L.cf_part_step_begin(ctx, ctypes.c_void_p(self.sendbuf.data_ptr())))
            self.solver._check(L.cf_part_wait_send(ctx))
            self._exchange()   # while the GPU updates the interior elements
            rc = L.cf_part_step_end(ctx, ctypes.c_void_p(self.recvbuf.data_ptr()), ctypes.byref(info))
            if rc not in (0, -4, -5):
                self.solver._check(rc)
            if self.steady:
                self._discharges()
            self.solver.set_dt(self._global_dt(self.solver.info().dt_next))
        return self.solver.info()

    def get_owned_state(self) -> np.ndarray:
        return self.solver.get_state()[: self.part.n_owned]

    def close(self):
        self.solver.close()
