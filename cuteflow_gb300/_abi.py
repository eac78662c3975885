"""ctypes mirror of include/cuteflow_gb300.h (struct layouts and prototypes)."""
from __future__ import annotations

import ctypes as C

import numpy as np

CF_MAX_IO = 20

CF_OK = 0
CF_EINVAL = -1
CF_ECUDA = -2
CF_ENOMEM = -3
CF_EDT = -4
CF_ENONFINITE = -5
CF_ESTATE = -6
CF_ENOTSUP = -7

CF_STATUS_DT_RANGE = 1
CF_STATUS_NONFINITE = 2
CF_STATUS_STEADY = 4
CF_STATUS_END = 8

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class CfMesh(C.Structure):
    _fields_ = [
        ("nnt", C.c_int32), ("nelt", C.c_int32),
        ("x", _dp), ("y", _dp), ("z", _dp),
        ("tri", _ip),
        ("manning_elt", _dp),
        ("ndinput", _ip), ("numero_ndinput", _ip),
        ("ndoutput", _ip), ("numero_ndoutput", _ip),
        ("ndwall", _ip),
        ("ndi", C.c_int32), ("ndo", C.c_int32), ("ndw", C.c_int32),
        ("nombre_entrees", C.c_int32), ("nombre_sorties", C.c_int32), ("pad_", C.c_int32),
    ]


class CfParams(C.Structure):
    _fields_ = [
        ("gp", C.c_double), ("tolisec", C.c_double), ("cfl", C.c_double), ("tol", C.c_double),
        ("override_manning", C.c_double), ("constant_dt", C.c_double),
        ("debitglob", C.c_double * CF_MAX_IO), ("h_sortie", C.c_double * CF_MAX_IO),
        ("debitglob_start", C.c_double * CF_MAX_IO), ("ramp_time", C.c_double),
        ("iflux", C.c_int32), ("ilimiteur", C.c_int32), ("friction", C.c_int32),
        ("fricimplic", C.c_int32), ("is_override_manning", C.c_int32),
        ("is_dt_constant", C.c_int32), ("inlet", C.c_int32), ("outlet", C.c_int32),
        ("flux_mode", C.c_int32), ("reorder", C.c_int32), ("pad_", C.c_int32),
        ("tol_reg_perm", C.c_double), ("steady_count", C.c_int32), ("dt_reset_nelt", C.c_int32),
        ("long_entree", C.c_double * CF_MAX_IO),
    ]


class CfIc(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "x1eqbar", "x2eqbar", "y1eqbar", "y2eqbar", "h_amont", "u_amont", "v_amont",
        "h_aval", "u_aval", "v_aval", "xplan", "yplan", "zplan", "xpoint", "ypoint", "zpoint")] + [
        ("eqlin_barrage", C.c_int32), ("plan", C.c_int32)]


class CfStepInfo(C.Structure):
    _fields_ = [
        ("t", C.c_double), ("dt_last", C.c_double), ("dt_next", C.c_double),
        ("q_in", C.c_double), ("q_out", C.c_double), ("steps", C.c_int64),
        ("status", C.c_uint32), ("pad_", C.c_int32),
    ]


def default_params() -> CfParams:
    """The reference's namelist defaults (global_data.cuf:31-62) plus the values its own
    cases set; mirrors cf_default_params."""
    p = CfParams()
    p.gp = 9.81
    p.tolisec = 1e-5
    p.cfl = 0.9
    p.tol = float(np.float32(1e-6))
    p.override_manning = 0.0
    p.constant_dt = 0.0
    p.ramp_time = 0.0
    p.iflux = 1
    p.ilimiteur = 1
    p.friction = 0
    p.fricimplic = 1
    p.is_override_manning = 0
    p.is_dt_constant = 0
    p.inlet = 2
    p.outlet = 1
    p.flux_mode = 0
    p.reorder = 1
    p.tol_reg_perm = 0.0
    p.steady_count = 1000
    return p


def make_params(overrides: dict | None = None) -> CfParams:
    p = default_params()
    for k, v in (overrides or {}).items():
        if k in ("debitglob", "h_sortie", "debitglob_start", "long_entree"):
            arr = getattr(p, k)
            for i, val in enumerate(v):
                arr[i] = float(val)
        else:
            setattr(p, k, v)
    return p


class MeshArrays:
    """Keeps contiguous numpy copies of a Case's mesh tables alive behind a CfMesh."""

    def __init__(self, case):
        self.x = np.ascontiguousarray(case.x, dtype=np.float64)
        self.y = np.ascontiguousarray(case.y, dtype=np.float64)
        self.z = np.ascontiguousarray(case.z, dtype=np.float64)
        self.tri = np.ascontiguousarray(case.tri, dtype=np.int32).reshape(-1)
        self.manning = np.ascontiguousarray(case.manning, dtype=np.float64)
        self.ndinput = np.ascontiguousarray(case.ndinput, dtype=np.int32)
        self.numero_ndinput = np.ascontiguousarray(case.numero_ndinput, dtype=np.int32)
        self.ndoutput = np.ascontiguousarray(case.ndoutput, dtype=np.int32)
        self.numero_ndoutput = np.ascontiguousarray(case.numero_ndoutput, dtype=np.int32)
        self.ndwall = np.ascontiguousarray(case.ndwall, dtype=np.int32)
        m = CfMesh()
        m.nnt = self.x.shape[0]
        m.nelt = self.tri.shape[0] // 3
        m.x = self.x.ctypes.data_as(_dp)
        m.y = self.y.ctypes.data_as(_dp)
        m.z = self.z.ctypes.data_as(_dp)
        m.tri = self.tri.ctypes.data_as(_ip)
        m.manning_elt = self.manning.ctypes.data_as(_dp)
        m.ndinput = self.ndinput.ctypes.data_as(_ip)
        m.numero_ndinput = self.numero_ndinput.ctypes.data_as(_ip)
        m.ndoutput = self.ndoutput.ctypes.data_as(_ip)
        m.numero_ndoutput = self.numero_ndoutput.ctypes.data_as(_ip)
        m.ndwall = self.ndwall.ctypes.data_as(_ip)
        m.ndi = self.ndinput.shape[0]
        m.ndo = self.ndoutput.shape[0]
        m.ndw = self.ndwall.shape[0]
        m.nombre_entrees = int(case.nombre_entrees)
        m.nombre_sorties = int(case.nombre_sorties)
        self.mesh = m


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_ip)
