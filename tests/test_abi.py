"""The C ABI library on a machine without a GPU: it loads, exports every function the public
header declares, its struct layouts match the ctypes mirror, and the host preprocessing
(cf_mesh_tables) agrees bit for bit with the oracle's restatement of the reference setup."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from cuteflow_gb300 import _abi, build, cases, solver

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cuteflow_gb300.h")


@pytest.fixture(scope="module")
def lib():
    build.build()
    return solver.load()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cf_[a-z_]+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", solver.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (cf_[a-z_]+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "cuteflow_gb300.h"
#define P(T, f) printf(#T "." #f " %zu\\n", offsetof(T, f));
int main(void) {
  printf("cf_mesh %zu\\ncf_params %zu\\ncf_ic %zu\\ncf_step_info %zu\\n", sizeof(cf_mesh), sizeof(cf_params),
         sizeof(cf_ic), sizeof(cf_step_info));
  P(cf_mesh, tri) P(cf_mesh, ndwall) P(cf_mesh, ndi) P(cf_mesh, nombre_sorties)
  P(cf_params, debitglob) P(cf_params, h_sortie) P(cf_params, ramp_time) P(cf_params, iflux) P(cf_params, reorder)
  P(cf_ic, zpoint) P(cf_ic, plan) P(cf_step_info, steps) P(cf_step_info, status)
  return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    assert int(got["cf_mesh"]) == C.sizeof(_abi.CfMesh)
    assert int(got["cf_params"]) == C.sizeof(_abi.CfParams)
    assert int(got["cf_ic"]) == C.sizeof(_abi.CfIc)
    assert int(got["cf_step_info"]) == C.sizeof(_abi.CfStepInfo)
    for key, val in got.items():
        if "." in key:
            t, f = key.split(".")
            cls = {"cf_mesh": _abi.CfMesh, "cf_params": _abi.CfParams, "cf_ic": _abi.CfIc,
                   "cf_step_info": _abi.CfStepInfo}[t]
            assert getattr(cls, f).offset == int(val), key


def test_default_params(lib):
    p = _abi.CfParams()
    assert lib.cf_default_params(C.byref(p)) == 0
    ref = _abi.default_params()
    for name, _ in _abi.CfParams._fields_:
        a, b = getattr(p, name), getattr(ref, name)
        if hasattr(a, "__len__"):
            assert list(a) == list(b), name
        else:
            assert a == b, name
    assert p.tol == float(np.float32(1e-6))


@pytest.mark.parametrize("make", [lambda: cases.circular_dam_break(30, 20, seed=1),
                                  lambda: cases.flooding(50, 25, seed=2),
                                  lambda: cases.ensemble_member(3)])
def test_mesh_tables_match_oracle(lib, oracle, make):
    c = make()
    b1, a1, z1, m1 = solver.mesh_tables(c)
    b2, a2, z2, m2, _, _ = oracle.setup(c)
    assert np.array_equal(b1, b2)
    assert np.array_equal(a1, a2) and np.array_equal(z1, z2) and np.array_equal(m1, m2)


@pytest.mark.parametrize("reorder", [0, 2])
def test_mesh_tables_do_not_depend_on_the_element_order(lib, reorder):
    """The device element order (Hilbert by default, Morton, or the caller's) is undone at the
    boundary: the reference-order tables are the same."""
    c = cases.flooding(40, 20, seed=3)
    a = solver.mesh_tables(c)
    b = solver.mesh_tables(c, dict(reorder=reorder))
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_boundary_kinds(lib):
    c = cases.flooding(20, 10, seed=3)
    b, _, _, _ = solver.mesh_tables(c)
    kinds, counts = np.unique(b[:, :, 0][b[:, :, 0] < 0], return_counts=True)
    assert dict(zip(kinds.tolist(), counts.tolist())) == {-3: 40, -2: 10, -1: 10}
    assert (b[:, :, 1][b[:, :, 0] == -1] == 1).all()
    # neighbours are mutual
    n = c.nelt
    for e in range(n):
        for k in range(3):
            nb = b[e, k, 0]
            if nb > 0:
                assert (b[nb - 1, :, 0] == e + 1).sum() == 1


def _expect_error(lib, case, params=None, code=_abi.CF_EINVAL, fragment=""):
    with pytest.raises(solver.CFError) as ei:
        solver.mesh_tables(case, params)
    assert ei.value.code == code
    assert fragment in str(ei.value)


def test_input_validation(lib):
    c = cases.circular_dam_break(6, 6, seed=1)
    bad = cases.circular_dam_break(6, 6, seed=1)
    bad.tri = bad.tri.copy()
    bad.tri[3, 1] = bad.nnt + 5
    _expect_error(lib, bad, fragment="outside 1..nnt")
    deg = cases.circular_dam_break(6, 6, seed=1)
    deg.tri = deg.tri.copy()
    deg.tri[0] = [1, 2, 3]  # three collinear nodes of the bottom row
    _expect_error(lib, deg, fragment="degenerate")
    f = cases.flooding(10, 5, seed=2)
    f.numero_ndinput = np.full_like(f.numero_ndinput, 25)
    _expect_error(lib, f, fragment="inlet/outlet number")
    c.manning = None
    ma_case = cases.circular_dam_break(6, 6, seed=1)
    with pytest.raises(solver.CFError):
        m = _abi.MeshArrays(ma_case)
        m.mesh.manning_elt = C.POINTER(C.c_double)()
        p = _abi.make_params(ma_case.params)
        rc = lib.cf_mesh_tables(C.byref(m.mesh), C.byref(p), None, None, None, None)
        raise solver.CFError(rc, lib.cf_last_error(None).decode())


def test_create_reports_errors_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(solver.CFError) as ei:
        solver.Solver(cases.circular_dam_break(6, 6, seed=1))
    assert ei.value.code in (_abi.CF_ECUDA, _abi.CF_ENOMEM)


def test_unsupported_options_are_rejected(lib):
    c = cases.circular_dam_break(6, 6, seed=1)
    m = _abi.MeshArrays(c)
    ctx = C.c_void_p()
    for over, code in ((dict(iflux=5), _abi.CF_EINVAL), (dict(inlet=4), _abi.CF_EINVAL),
                       (dict(tol_reg_perm=-1.0), _abi.CF_EINVAL),
                       (dict(ilimiteur=7), _abi.CF_EINVAL), (dict(flux_mode=2), _abi.CF_EINVAL),
                       (dict(cfl=0.0), _abi.CF_EINVAL)):
        p = _abi.make_params({**c.params, **over})
        assert lib.cf_create(C.byref(m.mesh), C.byref(p), C.byref(ctx)) == code
        assert not ctx.value
        assert lib.cf_last_error(None)
