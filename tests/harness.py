"""Builds and loads tests/flux_harness.cpp (the GPU step's flux mathematics compiled for the
CPU).  Test infrastructure only."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "libflux_harness.so")
_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    srcs = [os.path.join(HERE, "flux_harness.cpp"), os.path.join(ROOT, "cuteflow_gb300", "csrc", "cf_mesh.cpp")]
    deps = srcs + [os.path.join(ROOT, "cuteflow_gb300", "csrc", f) for f in ("cf_flux.h", "cf_internal.h", "cf_dual.h", "cf_xd.h")]
    if not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
        import platform
        # hardware FMA on x86-64 (std::fma is otherwise a slow, equally correctly rounded, libm routine)
        extra = ["-mfma"] if platform.machine() == "x86_64" else []
        subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off"] + extra + [
                        "-Wno-deprecated-declarations", "-I", cuda_inc, "-I", os.path.join(ROOT, "include"),
                        "-o", LIB] + srcs, check=True)
    from cuteflow_gb300 import _abi
    L = C.CDLL(LIB)
    dp = C.POINTER(C.c_double)
    L.harness_edge_fluxes.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(_abi.CfParams), dp, C.c_double,
                                      C.c_double, dp, dp]
    L.harness_edge_fluxes.restype = C.c_int
    _lib = L
    return L


def edge_fluxes(case, U, dt, t=0.0, params=None):
    from cuteflow_gb300 import _abi
    ma = _abi.MeshArrays(case)
    p = _abi.make_params({**case.params, **(params or {})})
    U = np.ascontiguousarray(U, dtype=np.float64)
    out = np.zeros((case.nelt, 3, 3))
    bed = np.zeros((case.nelt, 3, 2))
    rc = lib().harness_edge_fluxes(C.byref(ma.mesh), C.byref(p), _abi.dptr(U), float(dt), float(t),
                                   _abi.dptr(out), _abi.dptr(bed))
    assert rc == 0
    return out, bed


def run(case, nsteps, params=None, U0=None):
    from cuteflow_gb300 import _abi
    L = lib()
    if not hasattr(L, "_run_typed"):
        dp = C.POINTER(C.c_double)
        L.harness_run.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(_abi.CfParams), dp, C.c_int, dp, dp, dp,
                                  C.POINTER(C.c_int)]
        L.harness_run.restype = C.c_int
        L.harness_nbhd_stats.argtypes = [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
        L.harness_nbhd_stats.restype = None
        L._run_typed = True
    ma = _abi.MeshArrays(case)
    p = _abi.make_params({**case.params, **(params or {})})
    U0 = np.ascontiguousarray(case.U0 if U0 is None else U0, dtype=np.float64)
    U = np.zeros_like(U0)
    dth = np.zeros(nsteps + 1)
    t = C.c_double(0.0)
    steps = C.c_int(0)
    rc = L.harness_run(C.byref(ma.mesh), C.byref(p), _abi.dptr(U0), int(nsteps), _abi.dptr(U), _abi.dptr(dth),
                       C.byref(t), C.byref(steps))
    took, bad = C.c_longlong(0), C.c_longlong(0)
    L.harness_nbhd_stats(C.byref(took), C.byref(bad))
    return dict(U=U, dt_hist=dth, t=t.value, rc=rc, steps=steps.value, nbhd_took=took.value, nbhd_bad=bad.value)


def set_xd(mode: int):
    """The edge arithmetic type of the harness: 0 double, 1 integer comparisons, 2 integer
    comparisons and products."""
    L = lib()
    L.harness_set_xd.argtypes = [C.c_int]
    L.harness_set_xd.restype = None
    L.harness_set_xd(int(mode))


def mul_check(n, seed=12345):
    L = lib()
    L.harness_xd_check.argtypes = [C.c_longlong, C.c_ulonglong]
    L.harness_xd_check.restype = C.c_longlong
    return int(L.harness_xd_check(int(n), int(seed)))


def rcbrt(x):
    """cf::rcbrt of the kernels, evaluated on the host, elementwise."""
    L = lib()
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    dp = C.POINTER(C.c_double)
    L.harness_rcbrt.argtypes = [dp, dp, C.c_longlong]
    L.harness_rcbrt(x.ctypes.data_as(dp), y.ctypes.data_as(dp), x.size)
    return y


def div_check(n, seed=12345):
    L = lib()
    L.harness_div_check.argtypes = [C.c_longlong, C.c_ulonglong]
    L.harness_div_check.restype = C.c_longlong
    return int(L.harness_div_check(int(n), int(seed)))


def tangent(case, params, U0, dU0, manning, dn, dt, t, gauges, freeze_r=False):
    """Tangent-linear run (forward mode along (dU0, dn)) replaying dt / t: returns
    (eta, deta, U_N, dU_N)."""
    from cuteflow_gb300 import _abi
    L = lib()
    if not hasattr(L, "_tan_typed"):
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int32)
        L.harness_tangent.argtypes = [C.POINTER(_abi.CfMesh), C.POINTER(_abi.CfParams), dp, dp, dp, dp, C.c_int, dp,
                                      dp, ip, C.c_int, dp, dp, dp, dp, C.c_int]
        L.harness_tangent.restype = C.c_int
        L._tan_typed = True
    ma = _abi.MeshArrays(case)
    p = _abi.make_params({**case.params, **(params or {})})
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    U0, dU0, manning, dn, dt, t = f(U0), f(dU0), f(manning), f(dn), f(dt), f(t)
    g = np.ascontiguousarray(gauges, dtype=np.int32)
    N, G = len(dt), len(g)
    eta, deta = np.zeros((N, G)), np.zeros((N, G))
    U, dU = np.zeros_like(U0), np.zeros_like(U0)
    rc = L.harness_tangent(C.byref(ma.mesh), C.byref(p), _abi.dptr(U0), _abi.dptr(dU0), _abi.dptr(manning),
                           _abi.dptr(dn), N, _abi.dptr(dt), _abi.dptr(t), g.ctypes.data_as(C.POINTER(C.c_int32)), G,
                           _abi.dptr(eta), _abi.dptr(deta), _abi.dptr(U), _abi.dptr(dU), int(bool(freeze_r)))
    assert rc == 0
    return eta, deta, U, dU


def dry_check(n, seed=12345):
    """(mismatches, shortcuts taken) of harness_dry_check: the dry-region shortcuts of the step
    against the general evaluation on n adversarial edges and n adversarial elements."""
    L = lib()
    L.harness_dry_check.argtypes = [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]
    L.harness_dry_check.restype = C.c_longlong
    took = C.c_longlong(0)
    bad = int(L.harness_dry_check(int(n), int(seed), C.byref(took)))
    return bad, int(took.value)


def adj_hllc_check(n, seed=12345):
    """(largest relative difference, edges handled) of harness_adj_hllc_check: the closed-form
    first-order HLLC reverse edge against the six-lane Dual differentiation of the edge."""
    L = lib()
    L.harness_adj_hllc_check.argtypes = [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]
    L.harness_adj_hllc_check.restype = C.c_double
    took = C.c_longlong(0)
    worst = float(L.harness_adj_hllc_check(int(n), int(seed), C.byref(took)))
    return worst, int(took.value)
