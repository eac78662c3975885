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
