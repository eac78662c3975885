"""Python front end of libcfgb.so (ctypes over the C ABI of include/cuteflow_gb300.h).

The reference's host side is the Fortran program main.cuf / solve_finite_volumes; this module
offers the same operations to Python tooling: build a simulation from the reference's mesh
inputs (cf_create), set or generate the initial state (cf_set_state,
cf_set_initial_condition), advance a number of steps entirely on the GPU (cf_step), and read
the state back in the reference's element order (cf_get_state).

There is no CPU fallback: if the CUDA library is missing or no GPU is present, the calls
raise.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
from typing import Optional

import numpy as np

from . import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcfgb.so")

_lib = None


class CFError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cuteflow_gb300 error {code}: {msg}")
        self.code = code


def load(build_if_missing: bool = True):
    """Load libcfgb.so (building it in-tree first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from . import build as _b
        _b.build()
    if not os.path.exists(LIB_PATH):
        raise CFError(_abi.CF_EINVAL, f"{LIB_PATH} is missing: run cuteflow_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    L.cf_default_params.argtypes = [C.POINTER(_abi.CfParams)]
    L.cf_create.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(_abi.CfParams), C.POINTER(vp)]
    L.cf_destroy.argtypes = [vp]
    L.cf_destroy.restype = None
    L.cf_set_state.argtypes = [vp, dp, C.c_double]
    L.cf_set_state_device.argtypes = [vp, vp, C.c_double]
    L.cf_set_initial_condition.argtypes = [vp, C.POINTER(_abi.CfIc), C.c_double]
    L.cf_step.argtypes = [vp, C.c_int32, C.POINTER(_abi.CfStepInfo)]
    L.cf_step_noalloc.argtypes = [vp, C.c_int32, C.POINTER(_abi.CfStepInfo)]
    L.cf_run.argtypes = [vp, C.c_double, C.c_int64, C.POINTER(_abi.CfStepInfo)]
    L.cf_set_tuning.argtypes = [vp, C.c_int32, C.c_int32]
    L.cf_probe_fp64.argtypes = [vp, dp]
    L.cf_selftest_xd.argtypes = [vp, C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]
    L.cf_advance.argtypes = [vp, dp, C.c_double, C.c_int32, dp, C.POINTER(_abi.CfStepInfo)]
    L.cf_get_elements.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.c_int32, dp]
    L.cf_set_elements.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.c_int32, dp]
    L.cf_set_dt.argtypes = [vp, C.c_int32, C.c_double]
    L.cf_get_tuning.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.cf_autotune.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp]
    L.cf_get_state.argtypes = [vp, dp]
    L.cf_get_state_device.argtypes = [vp, vp]
    L.cf_get_info.argtypes = [vp, C.POINTER(_abi.CfStepInfo)]
    L.cf_get_mesh_tables.argtypes = [vp, C.POINTER(C.c_int32), dp, dp, dp]
    L.cf_mesh_tables.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(_abi.CfParams), C.POINTER(C.c_int32), dp, dp, dp]
    L.cf_get_sizes.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.cf_get_stream.argtypes = [vp]
    L.cf_get_stream.restype = vp
    L.cf_last_error.argtypes = [vp]
    L.cf_last_error.restype = C.c_char_p
    L.cf_set_timing.argtypes = [vp, C.c_int32]
    L.cf_set_direct_io.argtypes = [vp, C.c_int32]
    L.cf_set_launch_shape.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32]
    ipp = C.POINTER(C.c_int32)
    L.cf_create_part.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(_abi.CfParams), ipp, C.POINTER(vp)]
    L.cf_part_sizes.argtypes = [vp, ipp, ipp, ipp, ipp]
    L.cf_part_set_exchange.argtypes = [vp, ipp, C.c_int32, ipp, C.c_int32]
    L.cf_part_step_begin.argtypes = [vp, vp]
    L.cf_part_wait_send.argtypes = [vp]
    L.cf_part_step_end.argtypes = [vp, vp, C.POINTER(_abi.CfStepInfo)]
    L.cf_part_inlet_terms.argtypes = [vp, dp]
    L.cf_part_set_inlet_sums.argtypes = [vp, dp]
    L.cf_part_discharge_terms.argtypes = [vp, dp]
    L.cf_part_apply_discharges.argtypes = [vp, C.c_double, C.c_double]
    L.cf_get_launch_shape.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.cf_autotune_order.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(_abi.CfParams), dp, C.c_int32,
                                    C.POINTER(C.c_int32), dp]
    L.cf_get_timing.argtypes = [vp, dp, dp, C.POINTER(C.c_int64)]
    ip = C.POINTER(C.c_int32)
    L.cf_create_batch.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(_abi.CfParams), C.c_int32, C.POINTER(vp)]
    L.cf_get_members.argtypes = [vp]
    L.cf_member_set_state.argtypes = [vp, C.c_int32, dp, C.c_double]
    L.cf_member_set_initial_condition.argtypes = [vp, C.c_int32, C.POINTER(_abi.CfIc), C.c_double]
    L.cf_member_get_state.argtypes = [vp, C.c_int32, dp]
    L.cf_member_get_info.argtypes = [vp, C.c_int32, C.POINTER(_abi.CfStepInfo)]
    L.cf_member_get_mesh_tables.argtypes = [vp, C.c_int32, ip, dp, dp, dp]
    vpp = C.POINTER(vp)
    L.cf_set_manning.argtypes = [vp, vp]
    L.cf_adjoint_create.argtypes = [vp, C.c_int32, C.c_int32, ip, C.c_int32, vpp]
    L.cf_adjoint_destroy.argtypes = [vp]
    L.cf_adjoint_destroy.restype = None
    L.cf_adjoint_forward.argtypes = [vp, C.c_int32, vp, vp]
    L.cf_adjoint_backward.argtypes = [vp, vp, vp, vp, vp]
    L.cf_adjoint_get_dt.argtypes = [vp, vp, vp]
    L.cf_adjoint_set_dt.argtypes = [vp, vp, vp]
    L.cf_adjoint_sizes.argtypes = [vp, ip, ip, ip, C.POINTER(C.c_int64)]
    L.cf_adjoint_set_linearization.argtypes = [vp, C.c_int32]
    L.cf_adjoint_create_budget.argtypes = [vp, C.c_int32, C.c_int32, ip, ip, C.c_int32, C.c_int64, vpp]
    L.cf_adjoint_schedule.argtypes = [vp, ip, ip, ip, ip, C.POINTER(C.c_int64)]
    L.cf_adjoint_create_batch.argtypes = [vp, C.c_int32, C.c_int32, ip, ip, C.c_int32, vpp]
    L.cf_member_set_manning.argtypes = [vp, C.c_int32, vp]
    L.cf_zones_create.argtypes = [vp, ip, C.c_int32, vpp]
    L.cf_zones_destroy.argtypes = [vp]
    L.cf_zones_destroy.restype = None
    L.cf_zones_set.argtypes = [vp, vp]
    L.cf_zones_get.argtypes = [vp, vp, vp]
    L.cf_zones_gradient.argtypes = [vp, vp, vp]
    L.cf_zones_descend.argtypes = [vp, C.c_double, C.c_double, C.c_double]
    for name in ("cf_adjoint_create_budget", "cf_adjoint_schedule", "cf_adjoint_create_batch", "cf_member_set_manning", "cf_zones_create", "cf_zones_set",
                 "cf_zones_get", "cf_zones_gradient", "cf_zones_descend"):
        getattr(L, name).restype = C.c_int
    for name in ("cf_set_manning", "cf_adjoint_create", "cf_adjoint_forward", "cf_adjoint_backward",
                 "cf_adjoint_get_dt", "cf_adjoint_set_dt", "cf_adjoint_sizes", "cf_adjoint_set_linearization"):
        getattr(L, name).restype = C.c_int
    for name in ("cf_create_batch", "cf_get_members", "cf_member_set_state", "cf_member_set_initial_condition",
                 "cf_member_get_state", "cf_member_get_info", "cf_member_get_mesh_tables"):
        getattr(L, name).restype = C.c_int
    for name in ("cf_default_params", "cf_create", "cf_set_state", "cf_set_state_device",
                 "cf_set_initial_condition", "cf_step", "cf_step_noalloc", "cf_run", "cf_set_tuning",
                 "cf_get_tuning", "cf_autotune", "cf_get_elements", "cf_set_elements", "cf_set_dt", "cf_get_state", "cf_get_state_device",
                 "cf_get_info", "cf_get_mesh_tables", "cf_mesh_tables", "cf_get_sizes", "cf_set_timing", "cf_get_timing",
                 "cf_set_direct_io", "cf_set_launch_shape", "cf_get_launch_shape", "cf_autotune_order",
                 "cf_create_part", "cf_part_sizes", "cf_part_set_exchange", "cf_part_step_begin", "cf_part_wait_send",
                 "cf_part_step_end", "cf_part_inlet_terms", "cf_part_set_inlet_sums", "cf_part_discharge_terms",
                 "cf_part_apply_discharges",
                 "cf_probe_fp64", "cf_selftest_xd", "cf_advance"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def mesh_tables(case, params: Optional[dict] = None):
    """Host preprocessing only (no GPU): boundary table [nelt,3,2], area, zm, cotemin."""
    L = load()
    ma = _abi.MeshArrays(case)
    p = _abi.make_params({**getattr(case, "params", {}), **(params or {})})
    n = case.nelt
    bnd = np.zeros((n, 3, 2), dtype=np.int32)
    area, zm, cm = np.zeros(n), np.zeros(n), np.zeros(n)
    rc = L.cf_mesh_tables(C.byref(ma.mesh), C.byref(p), _abi.iptr(bnd), _abi.dptr(area), _abi.dptr(zm), _abi.dptr(cm))
    if rc != 0:
        raise CFError(rc, L.cf_last_error(None).decode())
    return bnd, area, zm, cm


@dataclasses.dataclass
class StepInfo:
    t: float
    dt_last: float
    dt_next: float
    q_in: float
    q_out: float
    steps: int
    status: int


def _info(s: _abi.CfStepInfo) -> StepInfo:
    return StepInfo(s.t, s.dt_last, s.dt_next, s.q_in, s.q_out, int(s.steps), int(s.status))


class Solver:
    """One simulation on the current CUDA device."""

    def __init__(self, case, params: Optional[dict] = None, elem_class: Optional[np.ndarray] = None):
        """elem_class (a part of a decomposed mesh, cf_create_part): per element 0 owned interior,
        1 owned and read by another part, 2 halo."""
        self._L = load()
        self._ctx = C.c_void_p()
        self._mesh = _abi.MeshArrays(case)
        self.params = _abi.make_params({**getattr(case, "params", {}), **(params or {})})
        if elem_class is not None:
            self._elem_class = np.ascontiguousarray(elem_class, dtype=np.int32)
            rc = self._L.cf_create_part(C.byref(self._mesh.mesh), C.byref(self.params),
                                        self._elem_class.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(self._ctx))
        else:
            rc = self._L.cf_create(C.byref(self._mesh.mesh), C.byref(self.params), C.byref(self._ctx))
        if rc != 0:
            raise CFError(rc, self._L.cf_last_error(None).decode())
        self.nelt = int(self._mesh.mesh.nelt)
        n = C.c_int64()
        e = C.c_int64()
        self._L.cf_get_sizes(self._ctx, C.byref(n), C.byref(e))
        self.nedge = int(e.value)

    def _check(self, rc: int):
        if rc != 0:
            raise CFError(rc, self._L.cf_last_error(self._ctx).decode())

    def close(self):
        if self._ctx:
            self._L.cf_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_state(self, U: np.ndarray, t0: float = 0.0):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(self.nelt, 3)
        self._check(self._L.cf_set_state(self._ctx, _abi.dptr(U), float(t0)))

    def set_state_device(self, ptr: int, t0: float = 0.0):
        """Set the state from a device pointer of 3*nelt doubles (reference order)."""
        self._check(self._L.cf_set_state_device(self._ctx, C.c_void_p(ptr), float(t0)))

    def set_manning(self, n):
        """Per-element Manning n [nelt] (reference order): a numpy array, or an int device
        address of nelt doubles."""
        if isinstance(n, int):
            self._check(self._L.cf_set_manning(self._ctx, C.c_void_p(n)))
        else:
            n = np.ascontiguousarray(n, dtype=np.float64)
            assert n.shape == (self.nelt,)
            self._check(self._L.cf_set_manning(self._ctx, n.ctypes.data_as(C.c_void_p)))

    def set_initial_condition(self, ic: dict, t0: float = 0.0):
        c = _abi.CfIc()
        for k, v in ic.items():
            setattr(c, k, v)
        self._check(self._L.cf_set_initial_condition(self._ctx, C.byref(c), float(t0)))

    def step(self, nsteps: int, check: bool = True) -> StepInfo:
        info = _abi.CfStepInfo()
        rc = self._L.cf_step(self._ctx, int(nsteps), C.byref(info))
        if check:
            self._check(rc)
        return _info(info)

    def get_elements(self, ids) -> np.ndarray:
        """(h, hu, hv) of the listed elements (0-based, reference order) of the current state."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        out = np.empty((ids.size, 3))
        self._check(self._L.cf_get_elements(self._ctx, 0, ids.ctypes.data_as(C.POINTER(C.c_int32)), int(ids.size),
                                            _abi.dptr(out)))
        return out

    def set_elements(self, ids, values):
        """Write (h, hu, hv) of the listed elements; the next dt becomes the CFL of the new state."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(ids.size, 3)
        self._check(self._L.cf_set_elements(self._ctx, 0, ids.ctypes.data_as(C.POINTER(C.c_int32)), int(ids.size),
                                            _abi.dptr(v)))

    def set_dt(self, dt: float):
        """The dt of the next step (a decomposed mesh applies the minimum over its parts)."""
        self._check(self._L.cf_set_dt(self._ctx, 0, float(dt)))

    def set_tuning(self, int_compare: int, int_mul_warps: int):
        """cf_set_tuning: share the edge kernel's FP64 work with the integer pipes (results
        identical in every setting)."""
        self._check(self._L.cf_set_tuning(self._ctx, int(int_compare), int(int_mul_warps)))

    def tuning(self):
        a, b = C.c_int32(), C.c_int32()
        self._check(self._L.cf_get_tuning(self._ctx, C.byref(a), C.byref(b)))
        return a.value, b.value

    def autotune(self, steps_per_trial: int = 50):
        """cf_autotune: time each integer-pipe setting and launch shape on the current state
        (restored afterwards) and keep the fastest; returns (int_compare, int_mul_warps,
        ms_per_step); launch_shape() gives the shape."""
        a, b, t = C.c_int32(), C.c_int32(), C.c_double()
        self._check(self._L.cf_autotune(self._ctx, int(steps_per_trial), C.byref(a), C.byref(b), C.byref(t)))
        return a.value, b.value, t.value

    def set_launch_shape(self, edge_block: int, edges_per_thread: int, cell_block: int):
        """cf_set_launch_shape (results identical in every shape)."""
        self._check(self._L.cf_set_launch_shape(self._ctx, int(edge_block), int(edges_per_thread), int(cell_block)))

    def launch_shape(self):
        """(edge_block, edges_per_thread, cell_block) of cf_get_launch_shape."""
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self._L.cf_get_launch_shape(self._ctx, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def advance(self, U: np.ndarray, t0: float, nsteps: int, check: bool = True):
        """cf_advance: the host state U (reference order, [nelt, 3]) at time t0 advanced by nsteps
        steps in one call; returns (the new state, StepInfo)."""
        src = np.ascontiguousarray(U, dtype=np.float64)
        out = np.empty_like(src)
        info = _abi.CfStepInfo()
        dp = C.POINTER(C.c_double)
        rc = self._L.cf_advance(self._ctx, src.ctypes.data_as(dp), float(t0), int(nsteps), out.ctypes.data_as(dp),
                                C.byref(info))
        if check:
            self._check(rc)
        return out, _info(info)

    def probe_fp64(self) -> float:
        """cf_probe_fp64: the FP64 pipe's throughput on this device, FP64 instructions per second."""
        r = C.c_double()
        self._check(self._L.cf_probe_fp64(self._ctx, C.byref(r)))
        return r.value

    def selftest_xd(self, n: int, seed: int = 1) -> int:
        """cf_selftest_xd: mismatches of the integer-pipe arithmetic against the FP64 unit on n
        adversarial operand pairs (0 expected)."""
        r = C.c_int64()
        self._check(self._L.cf_selftest_xd(self._ctx, int(n), int(seed), C.byref(r)))
        return int(r.value)

    def run(self, ts: float, max_steps: int = 1 << 40, check: bool = True) -> StepInfo:
        """The reference's time loop up to time ts (cf_run): stops with CF_STATUS_END, or at a
        steady state, or after max_steps steps."""
        info = _abi.CfStepInfo()
        rc = self._L.cf_run(self._ctx, float(ts), int(max_steps), C.byref(info))
        if check:
            self._check(rc)
        return _info(info)

    def info(self) -> StepInfo:
        s = _abi.CfStepInfo()
        self._check(self._L.cf_get_info(self._ctx, C.byref(s)))
        return _info(s)

    def get_state(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.nelt, 3))
        self._check(self._L.cf_get_state(self._ctx, _abi.dptr(out)))
        return out

    def get_state_device(self, ptr: int):
        self._check(self._L.cf_get_state_device(self._ctx, C.c_void_p(ptr)))

    def mesh_tables(self):
        bnd = np.zeros((self.nelt, 3, 2), dtype=np.int32)
        area, zm, cm = np.zeros(self.nelt), np.zeros(self.nelt), np.zeros(self.nelt)
        self._check(self._L.cf_get_mesh_tables(self._ctx, _abi.iptr(bnd), _abi.dptr(area),
                                               _abi.dptr(zm), _abi.dptr(cm)))
        return bnd, area, zm, cm

    def stream(self) -> int:
        return int(self._L.cf_get_stream(self._ctx) or 0)

    def set_timing(self, on: bool):
        self._check(self._L.cf_set_timing(self._ctx, 1 if on else 0))

    def set_direct_io(self, on: bool):
        """Kernels read and write pinned or device state buffers directly (default) or through
        the staging copy (results identical)."""
        self._check(self._L.cf_set_direct_io(self._ctx, 1 if on else 0))

    def timing(self):
        f, u, n = C.c_double(), C.c_double(), C.c_int64()
        self._check(self._L.cf_get_timing(self._ctx, C.byref(f), C.byref(u), C.byref(n)))
        return f.value, u.value, int(n.value)


class Batch:
    """Many independent simulations of uneven size stepped together (cf_create_batch)."""

    def __init__(self, case_list, params_list=None):
        self._L = load()
        self._ctx = C.c_void_p()
        self._meshes = [_abi.MeshArrays(c) for c in case_list]
        n = len(case_list)
        params_list = params_list or [None] * n
        MeshArr = _abi.CfMesh * n
        ParArr = _abi.CfParams * n
        self._mesh_arr = MeshArr(*[m.mesh for m in self._meshes])
        self._par_arr = ParArr(*[_abi.make_params({**getattr(c, "params", {}), **(p or {})})
                                 for c, p in zip(case_list, params_list)])
        rc = self._L.cf_create_batch(self._mesh_arr, self._par_arr, n, C.byref(self._ctx))
        if rc != 0:
            raise CFError(rc, self._L.cf_last_error(None).decode())
        self.members = n
        self.nelt = [int(m.mesh.nelt) for m in self._meshes]

    def _check(self, rc: int):
        if rc != 0:
            raise CFError(rc, self._L.cf_last_error(self._ctx).decode())

    def close(self):
        if self._ctx:
            self._L.cf_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_state(self, member: int, U: np.ndarray, t0: float = 0.0):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(self.nelt[member], 3)
        self._check(self._L.cf_member_set_state(self._ctx, int(member), _abi.dptr(U), float(t0)))

    def set_initial_condition(self, member: int, ic: dict, t0: float = 0.0):
        c = _abi.CfIc()
        for k, v in ic.items():
            setattr(c, k, v)
        self._check(self._L.cf_member_set_initial_condition(self._ctx, int(member), C.byref(c), float(t0)))

    def step(self, nsteps: int, check: bool = True):
        infos = (_abi.CfStepInfo * self.members)()
        rc = self._L.cf_step(self._ctx, int(nsteps), infos)
        if check:
            self._check(rc)
        return [_info(i) for i in infos]

    def set_tuning(self, int_compare: int, int_mul_warps: int):
        self._check(self._L.cf_set_tuning(self._ctx, int(int_compare), int(int_mul_warps)))

    def set_launch_shape(self, edge_block: int, edges_per_thread: int, cell_block: int):
        self._check(self._L.cf_set_launch_shape(self._ctx, int(edge_block), int(edges_per_thread), int(cell_block)))

    def launch_shape(self):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self._L.cf_get_launch_shape(self._ctx, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def autotune(self, steps_per_trial: int = 50):
        """cf_autotune on the batch (every member set and running); the state is restored."""
        a, b, t = C.c_int32(), C.c_int32(), C.c_double()
        self._check(self._L.cf_autotune(self._ctx, int(steps_per_trial), C.byref(a), C.byref(b), C.byref(t)))
        return a.value, b.value, t.value

    def run(self, ts: float, max_steps: int = 1 << 40, check: bool = True):
        """Every member up to time ts (cf_run), each stopping at its own step."""
        infos = (_abi.CfStepInfo * self.members)()
        rc = self._L.cf_run(self._ctx, float(ts), int(max_steps), infos)
        if check:
            self._check(rc)
        return [_info(i) for i in infos]

    def set_manning(self, member: int, n):
        """Per-element Manning n of one member (reference order; host array or device address)."""
        if isinstance(n, int):
            self._check(self._L.cf_member_set_manning(self._ctx, int(member), C.c_void_p(n)))
            return
        n = np.ascontiguousarray(n, dtype=np.float64)
        assert n.shape == (self.nelt[member],)
        self._check(self._L.cf_member_set_manning(self._ctx, int(member), n.ctypes.data_as(C.c_void_p)))

    def get_state(self, member: int) -> np.ndarray:
        out = np.empty((self.nelt[member], 3))
        self._check(self._L.cf_member_get_state(self._ctx, int(member), _abi.dptr(out)))
        return out

    def info(self, member: int) -> StepInfo:
        s = _abi.CfStepInfo()
        self._check(self._L.cf_member_get_info(self._ctx, int(member), C.byref(s)))
        return _info(s)

    def stream(self) -> int:
        return int(self._L.cf_get_stream(self._ctx) or 0)

    def set_timing(self, on: bool):
        self._check(self._L.cf_set_timing(self._ctx, 1 if on else 0))

    def timing(self):
        f, u, n = C.c_double(), C.c_double(), C.c_int64()
        self._check(self._L.cf_get_timing(self._ctx, C.byref(f), C.byref(u), C.byref(n)))
        return f.value, u.value, int(n.value)


def autotune_order(case, params: Optional[dict] = None, U: Optional[np.ndarray] = None, steps_per_trial: int = 20):
    """cf_autotune_order: the element order (reorder 1 Hilbert, 2 Morton, 0 the case's own) with
    which a context of this case steps fastest from the state U (default case.U0), each order
    timed with the rest of its tuning; returns (reorder, ms_per_step)."""
    L = load()
    ma = _abi.MeshArrays(case)
    p = _abi.make_params({**case.params, **(params or {})})
    src = np.ascontiguousarray(case.U0 if U is None else U, dtype=np.float64)
    r, t = C.c_int32(), C.c_double()
    rc = L.cf_autotune_order(C.byref(ma.mesh), C.byref(p), src.ctypes.data_as(C.POINTER(C.c_double)),
                             int(steps_per_trial), C.byref(r), C.byref(t))
    if rc != 0:
        raise CFError(rc, L.cf_last_error(None).decode(errors="replace"))
    return r.value, t.value
