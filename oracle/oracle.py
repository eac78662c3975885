"""ctypes front end of the CPU oracle (oracle/cf_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU legs of
bench.py as the checker and the timed CPU baseline.  The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

from cuteflow_gb300 import _abi  # noqa: E402  (struct layouts are shared with the product)

LIB_PATH = os.path.join(_HERE, "_build", "libcforacle.so")
SOURCES = [os.path.join(_HERE, "cf_oracle.cpp")]


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (-ffp-contract=off keeps the reference's rounding order)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(_HERE, "cf_oracle.h")])
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB_PATH + ".tmp"] + SOURCES
    subprocess.run(cmd, check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_setup.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(C.c_int32)] + [C.POINTER(C.c_double)] * 5
        L.orc_setup.restype = C.c_int
        L.orc_initial_condition.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(_abi.CfParams),
                                            C.POINTER(_abi.CfIc), C.POINTER(C.c_double)]
        L.orc_initial_condition.restype = C.c_int
        L.orc_run.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(_abi.CfParams), C.POINTER(C.c_double),
                              C.c_double, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                              C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                              C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int32)]
        L.orc_run.restype = C.c_int
        L.orc_max_threads.restype = C.c_int
        L.orc_all_edge_fluxes.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(_abi.CfParams),
                                          C.POINTER(C.c_double), C.c_double, C.c_double,
                                          C.POINTER(C.c_double)]
        L.orc_all_edge_fluxes.restype = C.c_int
        _lib = L
    return _lib


def max_threads() -> int:
    return int(lib().orc_max_threads())


def rcbrt(x) -> np.ndarray:
    """x^(-1/3) as the restated friction term evaluates it, elementwise."""
    L = lib()
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    dp = C.POINTER(C.c_double)
    L.orc_rcbrt.argtypes = [dp, dp, C.c_int64]
    L.orc_rcbrt.restype = None
    L.orc_rcbrt(x.ctypes.data_as(dp), y.ctypes.data_as(dp), x.size)
    return y


def setup(case):
    """Boundary table [nelt,3,2], area, zm, cotemin, xc, yc in reference order."""
    ma = _abi.MeshArrays(case)
    n = case.nelt
    bnd = np.zeros((n, 3, 2), dtype=np.int32)
    outs = [np.zeros(n) for _ in range(5)]
    rc = lib().orc_setup(C.byref(ma.mesh), _abi.iptr(bnd), *[_abi.dptr(o) for o in outs])
    if rc != 0:
        raise ValueError(f"orc_setup failed ({rc})")
    return (bnd,) + tuple(outs)


def initial_condition(case, ic: dict, params: dict | None = None) -> np.ndarray:
    ma = _abi.MeshArrays(case)
    p = _abi.make_params({**case.params, **(params or {})})
    c = _abi.CfIc()
    for k, v in ic.items():
        setattr(c, k, v)
    U0 = np.zeros((case.nelt, 3))
    rc = lib().orc_initial_condition(C.byref(ma.mesh), C.byref(p), C.byref(c), _abi.dptr(U0))
    if rc != 0:
        raise ValueError(f"orc_initial_condition failed ({rc})")
    return U0


def run(case, nsteps: int, params: dict | None = None, U0: np.ndarray | None = None, t0: float = 0.0,
        dt_replay: np.ndarray | None = None, nthreads: int = 0, check: bool = True):
    """Run the oracle.  Returns dict(U, dt_hist, t, q_in, q_out, rc)."""
    ma = _abi.MeshArrays(case)
    p = _abi.make_params({**case.params, **(params or {})})
    U0 = np.ascontiguousarray(case.U0 if U0 is None else U0, dtype=np.float64)
    U = np.zeros_like(U0)
    dt_hist = np.zeros(nsteps + 1)
    t = C.c_double(0.0)
    q = np.zeros(2)
    rp = None
    if dt_replay is not None:
        dt_replay = np.ascontiguousarray(dt_replay, dtype=np.float64)
        rp = _abi.dptr(dt_replay)
    loop = C.c_double(0.0)
    steps = C.c_int32(0)
    rc = lib().orc_run(C.byref(ma.mesh), C.byref(p), _abi.dptr(U0), float(t0), int(nsteps),
                       _abi.dptr(U), _abi.dptr(dt_hist), rp, C.byref(t), _abi.dptr(q), int(nthreads),
                       C.byref(loop), C.byref(steps))
    if check and rc not in (0, 1):
        raise RuntimeError(f"orc_run failed ({rc})")
    return dict(U=U, dt_hist=dt_hist, t=t.value, q_in=q[0], q_out=q[1], rc=rc, loop_seconds=loop.value,
                steps=steps.value)


def edge_fluxes(case, U: np.ndarray, dt: float, t: float = 0.0, params: dict | None = None) -> np.ndarray:
    """flux*len of every (element, edge) of state U as [nelt, 3, 3] (per-side evaluation)."""
    ma = _abi.MeshArrays(case)
    p = _abi.make_params({**case.params, **(params or {})})
    U = np.ascontiguousarray(U, dtype=np.float64)
    out = np.zeros((case.nelt, 3, 3))
    rc = lib().orc_all_edge_fluxes(C.byref(ma.mesh), C.byref(p), _abi.dptr(U), float(dt), float(t),
                                   _abi.dptr(out))
    if rc != 0:
        raise ValueError(f"orc_all_edge_fluxes failed ({rc})")
    return out
