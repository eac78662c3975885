"""The reference's input files: write a ``cases.Case`` as a CuteFlow case directory and read a
case directory through the C ABI (cf_case_read), so that the same directory runs in the
reference and here.

Layout written (the reference's main program reads it, main.cuf:48-182):
  donnees.f   the donnees_namelist (global_data.cuf:65-94): numerics, boundaries, meshfile,
              the initial condition selection, ts;
  <mesh>      the ASCII triangle mesh of lec_mail_tri (maillage.cuf:196-313): a title line,
              nnt, (n, x, y, z, manning) per node; a title, nelt, (n, n1, n2, n3, manning) per
              element; inflow, outflow and wall node tables;
  <ic>        with solinit = 1, the element state of read_initial_condition
              (initial_condition.cuf:82-102): a time, then h hu hv per element.
Reals are written with 17 significant digits, so a round trip is exact.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
from typing import Optional

import numpy as np

from . import _abi
from .solver import CFError, load

_LIMITER_DEFAULT = 1


def _r(x: float) -> str:
    return repr(float(x))


def write_case(case, directory: str, ts: float, params: Optional[dict] = None, meshfile: str = "mesh.txt",
               solinit: bool = True, ic: Optional[dict] = None, namelist: str = "donnees.f",
               sol_file: str = "sol_init.txt") -> str:
    """Write ``case`` as a case directory; returns the namelist path.  ``solinit`` writes
    case.U0 to an initial-condition file; otherwise ``ic`` gives the dam line / plane keys
    (eqlin_barrage, plan, h_amont, ...)."""
    os.makedirs(directory, exist_ok=True)
    p = {**case.params, **(params or {})}
    tri = np.asarray(case.tri, dtype=np.int64).reshape(-1, 3)
    nin, nout = int(case.nombre_entrees), int(case.nombre_sorties)
    with open(os.path.join(directory, meshfile), "w") as f:
        f.write("Table des coordonnees\n")
        f.write(f"{len(case.x)}\n")
        for i, (x, y, z) in enumerate(zip(case.x, case.y, case.z)):
            f.write(f"{i + 1} {_r(x)} {_r(y)} {_r(z)} 0.0\n")
        f.write("Table de connectivite\n")
        f.write(f"{tri.shape[0]}\n")
        for i, (t, n) in enumerate(zip(tri, case.manning)):
            f.write(f"{i + 1} {t[0]} {t[1]} {t[2]} {_r(n)}\n")
        for title, count, nodes, num in (("Noeuds d'entree", nin, case.ndinput, case.numero_ndinput),
                                         ("Noeuds de sortie", nout, case.ndoutput, case.numero_ndoutput)):
            f.write(title + "\n")
            if count == 1:
                f.write(f"{len(nodes)}\n")
                for nd in nodes:
                    f.write(f"{nd}\n")
            else:
                f.write(f"{len(nodes)} {count}\n")
                for nd, k in zip(nodes, num):
                    f.write(f"{nd} {k}\n")
        f.write("Noeuds de murs\n")
        f.write(f"{len(case.ndwall)}\n")
        for nd in case.ndwall:
            f.write(f"{nd}\n")
    if solinit:
        with open(os.path.join(directory, sol_file), "w") as f:
            f.write("0\n")
            for h, hu, hv in np.asarray(case.U0, dtype=np.float64):
                f.write(f"{_r(h)} {_r(hu)} {_r(hv)}\n")
    inlet = {1: "transm", 2: "inflow", 3: "phys_inflow"}[int(p.get("inlet", 2))]
    outlet = {1: "fixedheight", 2: "transm"}[int(p.get("outlet", 1))]
    deb = list(p.get("debitglob", [0.0]))[: max(1, nin)]
    hs = list(p.get("h_sortie", [0.0]))[: max(1, nout)]
    lines = [
        "&DONNEES_NAMELIST",
        "  ! generated by cuteflow_gb300.case_files",
        f"  GP={_r(p.get('gp', 9.81))},",
        f"  is_override_manning={int(p.get('is_override_manning', 0))}, "
        f"override_manning={_r(p.get('override_manning', 0.0))},",
        "  is_cgns=0,",
        "  meshfile_path='./',",
        f"  meshfile='{meshfile}',",
        "  elt_bound=0,",
        f"  nombre_entrees={nin}, nombre_sorties={nout},",
    ]
    icd = dict(ic or {})
    for k in ("eqlin_barrage", "plan"):
        lines.append(f"  {k}={int(icd.pop(k, 0))},")
    for k, v in icd.items():
        lines.append(f"  {k}={_r(v)},")
    lines += [
        f"  solinit={1 if solinit else 0},",
        f"  fich_sol_init='{sol_file if solinit else ''}',",
        f"  inlet='{inlet}',",
        '  inlet_name="Inflow nodes",',
        "  debitglob=" + ", ".join(_r(v) for v in deb) + ",",
        f"  outlet=\"{outlet}\",",
        "  H_sortie=" + ", ".join(_r(v) for v in hs) + ",",
        f"  IFLUX={int(p.get('iflux', 1))}, ilimiteur={int(p.get('ilimiteur', _LIMITER_DEFAULT))}, iupwind=1,",
        f"  tolisec={_r(p.get('tolisec', 1e-5))},",
        f"  friction={int(p.get('friction', 0))},",
        f"  fricimplic={int(p.get('fricimplic', 1))},",
        f"  TS={_r(ts)}, CFL={_r(p.get('cfl', 0.9))},",
        f"  is_dt_constant={int(p.get('is_dt_constant', 0))}, constant_dt={_r(p.get('constant_dt', 0.0))},",
        f"  tol_reg_perm={_r(p.get('tol_reg_perm', 0.0))},",
        "  freqaffich=1000,",
        "  solrestart=0,",
        "  solvisu=0, visu_snapshots=0,",
        "  sortie_finale_bluekenue=0/",
    ]
    path = os.path.join(directory, namelist)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


@dataclasses.dataclass
class CaseFiles:
    """A case directory read through cf_case_read; usable wherever a cases.Case is (Solver,
    oracle): params is the parameter dict, cparams the cf_params record."""

    params: dict
    cparams: "_abi.CfParams"
    ic: "_abi.CfIc"
    ts: float
    solinit: int
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    tri: np.ndarray
    manning: np.ndarray
    ndinput: np.ndarray
    numero_ndinput: np.ndarray
    ndoutput: np.ndarray
    numero_ndoutput: np.ndarray
    ndwall: np.ndarray
    nombre_entrees: int
    nombre_sorties: int
    U0: Optional[np.ndarray]
    t_file: float

    @property
    def nelt(self) -> int:
        return int(self.tri.shape[0])


def _param_dict(p: "_abi.CfParams") -> dict:
    out = {}
    for name, _ in _abi.CfParams._fields_:
        if name.startswith("pad"):
            continue
        v = getattr(p, name)
        out[name] = list(v) if hasattr(v, "__len__") else v
    return out


def _bind(L):
    if getattr(L, "_case_typed", False):
        return
    vp = C.c_void_p
    L.cf_case_read.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(vp)]
    L.cf_case_read.restype = C.c_int
    L.cf_case_free.argtypes = [vp]
    L.cf_case_free.restype = None
    L.cf_case_last_error.argtypes = []
    L.cf_case_last_error.restype = C.c_char_p
    L.cf_case_get.argtypes = [vp, C.POINTER(C.POINTER(_abi.CfMesh)), C.POINTER(C.POINTER(_abi.CfParams)),
                              C.POINTER(_abi.CfIc), C.POINTER(C.c_double), C.POINTER(C.c_int32)]
    L.cf_case_get.restype = C.c_int
    L.cf_case_initial_state.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.cf_case_initial_state.restype = C.c_int
    L.cf_write_state_file.argtypes = [C.c_char_p, C.POINTER(C.c_double), C.c_int32, C.c_double]
    L.cf_write_state_file.restype = C.c_int
    L._case_typed = True


def read_case(directory: str, namelist: Optional[str] = None) -> CaseFiles:
    """Read a case directory (host code only: no GPU needed)."""
    L = load()
    _bind(L)
    h = C.c_void_p()
    rc = L.cf_case_read(directory.encode(), namelist.encode() if namelist else None, C.byref(h))
    if rc != 0:
        raise CFError(rc, L.cf_case_last_error().decode())
    try:
        mp = C.POINTER(_abi.CfMesh)()
        pp = C.POINTER(_abi.CfParams)()
        ic = _abi.CfIc()
        ts = C.c_double()
        si = C.c_int32()
        L.cf_case_get(h, C.byref(mp), C.byref(pp), C.byref(ic), C.byref(ts), C.byref(si))
        m = mp.contents
        params = _abi.CfParams()
        C.memmove(C.byref(params), pp, C.sizeof(params))

        def arr(ptr, n, dt):
            return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt).copy() if n > 0 else np.zeros(0, dt)

        nnt, nelt = m.nnt, m.nelt
        U0, t_file = None, 0.0
        if si.value == 1:
            U0 = np.empty((nelt, 3))
            tf = C.c_double()
            rc = L.cf_case_initial_state(h, U0.ctypes.data_as(C.POINTER(C.c_double)), C.byref(tf))
            if rc != 0:
                raise CFError(rc, L.cf_case_last_error().decode())
            t_file = tf.value
        return CaseFiles(params=_param_dict(params), cparams=params, ic=ic, ts=ts.value, solinit=si.value, x=arr(m.x, nnt, np.float64),
                         y=arr(m.y, nnt, np.float64), z=arr(m.z, nnt, np.float64),
                         tri=arr(m.tri, 3 * nelt, np.int32).reshape(nelt, 3),
                         manning=arr(m.manning_elt, nelt, np.float64), ndinput=arr(m.ndinput, m.ndi, np.int32),
                         numero_ndinput=arr(m.numero_ndinput, m.ndi, np.int32),
                         ndoutput=arr(m.ndoutput, m.ndo, np.int32),
                         numero_ndoutput=arr(m.numero_ndoutput, m.ndo, np.int32),
                         ndwall=arr(m.ndwall, m.ndw, np.int32), nombre_entrees=m.nombre_entrees,
                         nombre_sorties=m.nombre_sorties, U0=U0, t_file=t_file)
    finally:
        L.cf_case_free(h)


def write_state_file(path: str, U: np.ndarray, t: float) -> None:
    """save_sol_for_restart's layout (6 decimals per value)."""
    L = load()
    _bind(L)
    U = np.ascontiguousarray(U, dtype=np.float64)
    rc = L.cf_write_state_file(path.encode(), U.ctypes.data_as(C.POINTER(C.c_double)), int(U.shape[0]), float(t))
    if rc != 0:
        raise CFError(rc, L.cf_case_last_error().decode())
