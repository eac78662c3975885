"""Discrete adjoint of the step for Manning calibration (cf_adjoint_* of the C ABI).

``Adjoint`` runs N steps from a Solver's current state, records the gauge elevations
eta[k, g] = h + z after every step and the dt sequence, and returns the gradient of

    J = sum_k sum_g w_eta[k, g] * eta[k, g] + sum_e w_state[e, :] . U^N[e, :]

with respect to the initial state and the per-element Manning n, with every step's dt held at
its recorded value.  ``gauge_run`` exposes the same run as a ``torch.autograd.Function`` of
(manning, U0) returning (eta, U^N) on the GPU.

Calibration tooling of the reference samples Manning fields and runs independent forwards; it
has no gradients.  This module has no CPU fallback: without the CUDA library the calls raise.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

import numpy as np

from .solver import CFError, Solver, load


def _ptr(a) -> C.c_void_p:
    if a is None:
        return C.c_void_p()
    if isinstance(a, int):
        return C.c_void_p(a)
    if hasattr(a, "data_ptr"):           # torch tensor
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)  # numpy array


class Adjoint:
    """Adjoint of ``nsteps`` steps of ``solver`` with gauge elements ``gauges`` (0-based,
    reference order).  ``solver`` is a Solver, or a Batch with ``gauge_member`` giving each
    gauge's member; states and gradients of a batch are concatenated in member order.
    ``checkpoint_interval`` 0 keeps ceil(sqrt(N)).  ``budget_bytes`` > 0 chooses the memory
    schedule that fits that much device memory (cf_adjoint_create_budget): the recording forward
    keeps the step records of as many of the last steps as fit, so the backward pass replays only
    the steps before them (none when the whole run fits); the gradient is the same bits."""

    def __init__(self, solver, nsteps: int, gauges, checkpoint_interval: int = 0, gauge_member=None,
                 budget_bytes: int = 0):
        self._L = load()
        self.solver = solver
        self.nsteps = int(nsteps)
        self.gauges = np.ascontiguousarray(gauges, dtype=np.int32).ravel()
        self._h = C.c_void_p()
        ip = C.POINTER(C.c_int32)
        if budget_bytes > 0:
            gm = None if gauge_member is None else np.ascontiguousarray(gauge_member, dtype=np.int32).ravel()
            rc = self._L.cf_adjoint_create_budget(solver._ctx, self.nsteps, int(checkpoint_interval),
                                                  None if gm is None else gm.ctypes.data_as(ip),
                                                  self.gauges.ctypes.data_as(ip), int(self.gauges.size),
                                                  int(budget_bytes), C.byref(self._h))
            self.gauge_member = np.zeros_like(self.gauges) if gm is None else gm
        elif gauge_member is None:
            rc = self._L.cf_adjoint_create(solver._ctx, self.nsteps, int(checkpoint_interval),
                                           self.gauges.ctypes.data_as(ip), int(self.gauges.size), C.byref(self._h))
            self.gauge_member = np.zeros_like(self.gauges)
        else:
            self.gauge_member = np.ascontiguousarray(gauge_member, dtype=np.int32).ravel()
            assert self.gauge_member.size == self.gauges.size
            rc = self._L.cf_adjoint_create_batch(solver._ctx, self.nsteps, int(checkpoint_interval),
                                                 self.gauge_member.ctypes.data_as(ip),
                                                 self.gauges.ctypes.data_as(ip), int(self.gauges.size),
                                                 C.byref(self._h))
        solver._check(rc)
        self.members = int(getattr(solver, "members", 1))
        self.nelt_total = int(sum(solver.nelt)) if isinstance(solver.nelt, (list, tuple)) else int(solver.nelt)
        k, g = C.c_int32(), C.c_int32()
        b = C.c_int64()
        self._L.cf_adjoint_sizes(self._h, None, C.byref(k), C.byref(g), C.byref(b))
        self.checkpoint_interval = int(k.value)
        self.device_bytes = int(b.value)
        st, ki, nc, nr = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        self._L.cf_adjoint_schedule(self._h, C.byref(st), C.byref(ki), C.byref(nc), C.byref(nr), None)
        # steps whose records the recording forward keeps, checkpoints of the others, record pool
        self.schedule = {"stored_steps": int(st.value), "checkpoint_interval": int(ki.value),
                         "checkpoints": int(nc.value), "records": int(nr.value), "device_bytes": int(b.value)}
        self.generation = 0

    def set_linearization(self, freeze_limiter_ratios: bool):
        """WAF only: hold the limiter ratios constant in the linearization, an approximate
        gradient for long runs over which the WAF objective is not differentiable (bounded with
        the van Albada limiter; the superbee linearization still grows)."""
        self.solver._check(self._L.cf_adjoint_set_linearization(self._h, 1 if freeze_limiter_ratios else 0))

    @property
    def ngauges(self) -> int:
        return int(self.gauges.size)

    def close(self):
        if self._h:
            self._L.cf_adjoint_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def forward(self, replay: bool = False, eta=None, state=None) -> Tuple[np.ndarray, np.ndarray]:
        """Run; returns (eta [N, G], U^N [nelt, 3]) as numpy arrays, or fills the given
        buffers (numpy arrays, torch tensors or device addresses) and returns them."""
        ret_e = np.empty((self.nsteps, self.ngauges)) if eta is None else eta
        ret_s = np.empty((self.nelt_total, 3)) if state is None else state
        self.solver._check(self._L.cf_adjoint_forward(self._h, 1 if replay else 0, _ptr(ret_e), _ptr(ret_s)))
        self.generation += 1
        return ret_e, ret_s

    def backward(self, w_eta=None, w_state=None, g_state0=None, g_manning=None):
        """Gradient of the last forward run: returns (dJ/dU0 [nelt, 3], dJ/dn [nelt])."""
        if w_eta is not None and not isinstance(w_eta, int) and not hasattr(w_eta, "data_ptr"):
            w_eta = np.ascontiguousarray(w_eta, dtype=np.float64)
            assert w_eta.size == self.nsteps * self.ngauges
        if w_state is not None and not isinstance(w_state, int) and not hasattr(w_state, "data_ptr"):
            w_state = np.ascontiguousarray(w_state, dtype=np.float64)
            assert w_state.size == 3 * self.nelt_total
        gs = np.empty((self.nelt_total, 3)) if g_state0 is None else g_state0
        gm = np.empty(self.nelt_total) if g_manning is None else g_manning
        self.solver._check(self._L.cf_adjoint_backward(self._h, _ptr(w_eta), _ptr(w_state), _ptr(gs), _ptr(gm)))
        return gs, gm

    def dt_history(self) -> Tuple[np.ndarray, np.ndarray]:
        """The recorded dt and start time of every step: [N] for one member, [N, members] for a
        batch."""
        shape = (self.nsteps,) if self.members == 1 else (self.nsteps, self.members)
        dt, t = np.empty(shape), np.empty(shape)
        self.solver._check(self._L.cf_adjoint_get_dt(self._h, _ptr(dt), _ptr(t)))
        return dt, t

    def set_dt_history(self, dt, t):
        dt = np.ascontiguousarray(dt, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.float64)
        assert dt.size == self.nsteps * self.members and t.size == self.nsteps * self.members
        self.solver._check(self._L.cf_adjoint_set_dt(self._h, _ptr(dt), _ptr(t)))


def _torch_function():
    import torch

    class GaugeRun(torch.autograd.Function):
        """(manning [nelt], U0 [nelt, 3]) -> (eta [N, G], U^N [nelt, 3]) on the GPU, float64."""

        @staticmethod
        def forward(ctx, manning, U0, adj: Adjoint, t0: float, replay: bool):
            for x in (manning, U0):
                if x.dtype != torch.float64 or not x.is_cuda or not x.is_contiguous():
                    raise CFError(-1, "manning and U0 must be contiguous float64 CUDA tensors")
            torch.cuda.current_stream().synchronize()
            s = adj.solver
            s.set_manning(int(manning.data_ptr()))
            s.set_state_device(int(U0.data_ptr()), t0)
            eta = torch.empty((adj.nsteps, adj.ngauges), dtype=torch.float64, device=U0.device)
            UN = torch.empty_like(U0)
            adj.forward(replay=replay, eta=eta, state=UN)
            ctx.adj = adj
            ctx.generation = adj.generation
            return eta, UN

        @staticmethod
        def backward(ctx, g_eta, g_UN):
            adj: Adjoint = ctx.adj
            if adj.generation != ctx.generation:
                raise CFError(-6, "the adjoint has run another forward since this one; "
                                  "call backward before the next forward")
            dev = g_eta.device if g_eta is not None else g_UN.device
            torch.cuda.current_stream().synchronize()
            ge = g_eta.contiguous() if g_eta is not None else None
            gs = g_UN.contiguous() if g_UN is not None else None
            gU0 = torch.empty((adj.solver.nelt, 3), dtype=torch.float64, device=dev)
            gn = torch.empty(adj.solver.nelt, dtype=torch.float64, device=dev)
            adj.backward(ge, gs, gU0, gn)
            return gn, gU0, None, None, None

    return GaugeRun


_GaugeRun = None


def gauge_run(adj: Adjoint, manning, U0, t0: float = 0.0, replay: bool = False):
    """torch.autograd-aware run: returns (eta [N, G], U^N [nelt, 3]); backward gives the
    gradients with respect to manning and U0 through the discrete adjoint (dt frozen)."""
    global _GaugeRun
    if _GaugeRun is None:
        _GaugeRun = _torch_function()
    return _GaugeRun.apply(manning, U0, adj, float(t0), bool(replay))


class Zones:
    """Manning zones of a context (cf_zones_*): ``zone_of_elem`` gives every element's zone
    (concatenated in member order for a batch; -1: not a parameter).  ``set`` writes zone
    values into n; ``gradient(adj)`` sums the adjoint's last dJ/dn per zone on the device in a
    fixed order; ``descend(lr, lo, hi)`` steps the values on the device and writes the new n."""

    def __init__(self, solver, zone_of_elem, nzones: int):
        self._L = load()
        self.solver = solver
        self.nzones = int(nzones)
        z = np.ascontiguousarray(zone_of_elem, dtype=np.int32).ravel()
        self._h = C.c_void_p()
        solver._check(self._L.cf_zones_create(solver._ctx, z.ctypes.data_as(C.POINTER(C.c_int32)), self.nzones,
                                              C.byref(self._h)))

    def close(self):
        if self._h:
            self._L.cf_zones_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set(self, values):
        v = values if hasattr(values, "data_ptr") else np.ascontiguousarray(values, dtype=np.float64)
        self.solver._check(self._L.cf_zones_set(self._h, _ptr(v)))

    def get(self) -> Tuple[np.ndarray, np.ndarray]:
        v, g = np.empty(self.nzones), np.empty(self.nzones)
        self.solver._check(self._L.cf_zones_get(self._h, _ptr(v), _ptr(g)))
        return v, g

    def gradient(self, adj: "Adjoint", out=None) -> np.ndarray:
        g = np.empty(self.nzones) if out is None else out
        self.solver._check(self._L.cf_zones_gradient(self._h, adj._h, _ptr(g)))
        return g

    def descend(self, lr: float, lo: float, hi: float):
        self.solver._check(self._L.cf_zones_descend(self._h, float(lr), float(lo), float(hi)))


def zone_gradient(g_manning: np.ndarray, zones: np.ndarray, nzones: Optional[int] = None) -> np.ndarray:
    """dJ/d(zone value) for a Manning field that is piecewise constant over zones: the sum of
    the per-element gradients of each zone, in element order (deterministic)."""
    nz = int(zones.max()) + 1 if nzones is None else nzones
    out = np.zeros(nz)
    np.add.at(out, zones, g_manning)
    return out
