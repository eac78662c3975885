"""The reference's input files through the C ABI (cf_case_read, cf_write_state_file): host
code only, no GPU.  A case written by case_files.write_case reads back exactly; the namelist
reader follows Fortran namelist syntax as the reference's case files use it; errors are
reported, not fatal."""
import numpy as np
import pytest

from cuteflow_gb300 import _abi, case_files, cases, solver


def _same_mesh(a, b):
    for k in ("x", "y", "z", "manning", "ndinput", "numero_ndinput", "ndoutput", "numero_ndoutput", "ndwall"):
        assert np.array_equal(np.asarray(getattr(a, k)), np.asarray(getattr(b, k))), k
    assert np.array_equal(np.asarray(a.tri).reshape(-1, 3), np.asarray(b.tri).reshape(-1, 3))
    assert a.nombre_entrees == b.nombre_entrees and a.nombre_sorties == b.nombre_sorties


@pytest.mark.parametrize("make", [lambda: cases.flooding(30, 15, seed=3, iflux=3),
                                  lambda: cases.channel(inlet=3),
                                  lambda: cases.circular_dam_break(12, 12, seed=2, iflux=4)],
                         ids=["flooding", "channel_phys_inflow", "dam_muscl"])
def test_round_trip(tmp_path, make):
    c = make()
    case_files.write_case(c, str(tmp_path), ts=123.5)
    r = case_files.read_case(str(tmp_path))
    _same_mesh(c, r)
    assert np.array_equal(r.U0, c.U0) and r.solinit == 1 and r.ts == 123.5
    p = _abi.make_params(c.params)
    for k in ("gp", "tolisec", "cfl", "iflux", "ilimiteur", "friction", "fricimplic", "inlet", "outlet",
              "is_override_manning"):
        assert r.params[k] == getattr(p, k), k
    assert r.params["debitglob"][0] == p.debitglob[0] and r.params["h_sortie"][0] == p.h_sortie[0]
    # the host preprocessing of the read case equals that of the original
    t1 = solver.mesh_tables(c)
    t2 = solver.mesh_tables(r, r.params)
    for a, b in zip(t1, t2):
        assert np.array_equal(a, b)


def test_read_case_runs_like_the_original(tmp_path, oracle):
    c = cases.channel(inlet=3)
    case_files.write_case(c, str(tmp_path), ts=50.0)
    r = case_files.read_case(str(tmp_path))
    a = oracle.run(c, 40)
    b = oracle.run(r, 40, params=r.params)
    assert np.array_equal(a["U"], b["U"]) and a["t"] == b["t"]


MESH = """Table des coordonnees
4
1 0.0 0.0 0.5 0.03
2, 10.0, 0.0, 0.5, 0.03
3 10.0 10.0 0.5 0.03 this is ignored
4
0.0 10.0 0.5 0.03
Table de connectivite
2
1 1 2 3 0.025
2 1 3 4 2.5d-2
Noeuds d'entree
2 2
1 1
4 2
Noeuds de sortie
2
2
3
Noeuds de murs
0
"""

NAMELIST = """&DONNEES_NAMELIST
  ! comments, upper and lower case, no commas between some entries
  GP=9.81,
  is_override_manning=0 override_manning=0.,
  is_cgns=0, meshfile_path='./', meshfile="m.txt",
  nombre_entrees=2, nombre_sorties=1,    ! two inlets: numbered inflow records
  eqlin_barrage=1, x1eqbar=5.0, x2eqbar=5.0, y1eqbar=0.0, y2eqbar=10.0,
  H_AMONT=1., U_AMONT=0, V_AMONT=0,
  H_AVAL=0.2, U_AVAL =0, V_AVAL =0,
  plan=0
  solinit=0, fich_sol_init='',
  inlet='phys_inflow', inlet_name="Inflow nodes",
  debitglob=3.0, debitglob(2)=4.5d0,
  outlet="fixedheight", outlet_name='it''s the outlet',
  H_sortie=2*0.75,
  IFLUX=3, ilimiteur=2, iupwind=1,
  tolisec=1.0E-05, friction=1, fricimplic=2,
  TS=360.0, CFL=0.6,
  is_dt_constant=0, constant_dt=1e-5,
  tol_reg_perm=1.0E-15,
  freqaffich=1000, sol_z_offset=0.
  solrestart=0, solvisu=3, visu_snapshots=180,
  sortie_finale_bluekenue=0/
"""


def test_namelist_and_mesh_syntax(tmp_path):
    (tmp_path / "donnees.f").write_text(NAMELIST)
    (tmp_path / "m.txt").write_text(MESH)
    r = case_files.read_case(str(tmp_path))
    p = r.params
    assert p["iflux"] == 3 and p["ilimiteur"] == 2 and p["friction"] == 1 and p["fricimplic"] == 2
    assert p["inlet"] == 3 and p["outlet"] == 1
    assert p["tolisec"] == 1e-5 and p["cfl"] == 0.6 and p["tol_reg_perm"] == 1e-15 and p["gp"] == 9.81
    assert p["debitglob"][:2] == [3.0, 4.5] and p["h_sortie"][:2] == [0.75, 0.75]
    assert r.ts == 360.0 and r.solinit == 0 and r.U0 is None
    assert r.ic.eqlin_barrage == 1 and r.ic.h_amont == 1.0 and r.ic.h_aval == 0.2 and r.ic.x1eqbar == 5.0
    # mesh: list-directed records (commas, a record continued on the next line, trailing text)
    assert np.array_equal(r.x, [0.0, 10.0, 10.0, 0.0]) and np.array_equal(r.y, [0.0, 0.0, 10.0, 10.0])
    assert np.array_equal(r.tri, [[1, 2, 3], [1, 3, 4]]) and np.array_equal(r.manning, [0.025, 0.025])
    assert np.array_equal(r.ndinput, [1, 4]) and np.array_equal(r.numero_ndinput, [1, 2])
    assert r.nombre_entrees == 2 and np.array_equal(r.ndoutput, [2, 3]) and r.ndwall.size == 0


@pytest.mark.parametrize("change,code,words", [
    (("GP=9.81,", "GP=9.81, bogus_key=3,"), _abi.CF_EINVAL, "unknown key"),
    (("is_cgns=0", "is_cgns=1"), _abi.CF_EINVAL, "not an HDF5 file"),   # an ASCII mesh named as CGNS
    (('meshfile="m.txt"', 'meshfile="missing.txt"'), _abi.CF_EINVAL, "cannot open"),
    (("IFLUX=3", "IFLUX=three"), _abi.CF_EINVAL, "iflux"),
    (("inlet='phys_inflow'", "inlet='sideways'"), _abi.CF_EINVAL, "inlet"),
    (("sortie_finale_bluekenue=0/", "sortie_finale_bluekenue=0"), _abi.CF_EINVAL, "not closed"),
    (("GP=9.81,", "GP=9.81, diffusion=1,"), _abi.CF_ENOTSUP, "diffusion"),
])
def test_namelist_errors(tmp_path, change, code, words):
    (tmp_path / "donnees.f").write_text(NAMELIST.replace(*change))
    (tmp_path / "m.txt").write_text(MESH)
    with pytest.raises(solver.CFError) as ei:
        case_files.read_case(str(tmp_path))
    assert ei.value.code == code and words in str(ei.value)


def test_mesh_errors(tmp_path):
    (tmp_path / "donnees.f").write_text(NAMELIST)
    (tmp_path / "m.txt").write_text(MESH.replace("2 1 3 4 2.5d-2", "2 1 3 9 2.5d-2"))
    with pytest.raises(solver.CFError) as ei:
        case_files.read_case(str(tmp_path))
    assert "out of range" in str(ei.value)
    (tmp_path / "m.txt").write_text(MESH[:120])
    with pytest.raises(solver.CFError):
        case_files.read_case(str(tmp_path))
    # a count beyond the mesh tables' int32 range is an error, not an allocation of it
    (tmp_path / "m.txt").write_text(MESH.replace("Table des coordonnees\n4\n", "Table des coordonnees\n1000000000000\n", 1))
    with pytest.raises(solver.CFError) as ei:
        case_files.read_case(str(tmp_path))
    assert "node count" in str(ei.value)


def test_restart_file_layout(tmp_path):
    """save_sol_for_restart writes '(4f16.6)' records: 6 decimals, 16 columns per value; the
    file reads back as an initial condition (solinit = 1)."""
    c = cases.channel()
    U = c.U0.copy()
    U[:, 1] = np.linspace(-2.0, 3.0, c.nelt)
    case_files.write_case(c, str(tmp_path), ts=1.0, sol_file="restart.txt", solinit=True)
    path = str(tmp_path / "restart.txt")
    case_files.write_state_file(path, U, 12.25)
    lines = open(path).read().splitlines()
    assert float(lines[0]) == 12.25 and len(lines) == c.nelt + 1
    assert all(len(line) == 48 for line in lines[1:])
    r = case_files.read_case(str(tmp_path))
    assert r.t_file == 12.25
    assert np.abs(r.U0 - U).max() <= 5e-7


def _reference_root():
    """The reference checkout named by CUTEFLOW_REFERENCE (the tree the golden fixtures were made
    from), or None when the variable is unset."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden
    return make_golden.reference_root()


def _reference_case_dir(sub):
    """A case directory of the reference checkout named by CUTEFLOW_REFERENCE; None when the
    variable is unset or the directory is absent."""
    import os
    root = _reference_root()
    if not root:
        return None
    d = os.path.join(root, "Calibration_manning", "docs_calibration", sub)
    return d if os.path.isfile(os.path.join(d, "donnees.f")) else None


@pytest.mark.parametrize("name,sub", [("river_piers", "River_piers/Froude"),
                                      ("divergent_canal", "Divergent_Canal/Froude")])
def test_cgns_case_directories_of_the_reference(tmp_path, name, sub):
    """is_cgns = 1: the reference's own case directories (donnees.f + CGNS/HDF5 mesh) read through
    cf_case_read give the mesh, boundary node lists and parameters of the golden fixtures (which a
    separate Python HDF5 reader decoded from the same files), and the boundary table CuteFlow wrote;
    with is_override_manning = 0 the per-element Manning n comes from the mesh's user data."""
    d = _reference_case_dir(sub)
    if d is None:
        pytest.skip("CUTEFLOW_REFERENCE does not name a reference checkout")
    import os
    import golden_cases as G
    g = G.load(name)
    r = case_files.read_case(d)
    assert r.nelt == g["tri"].shape[0]
    for k in ("x", "y", "z", "ndinput", "ndoutput"):
        assert np.array_equal(np.asarray(getattr(r, k)), g[k]), k
    assert np.array_equal(np.asarray(r.tri).reshape(-1, 3), g["tri"])
    assert set(np.asarray(r.numero_ndinput).tolist()) == {1} and len(r.ndwall) == 0
    for k in ("iflux", "ilimiteur", "fricimplic", "tolisec", "cfl", "gp"):
        assert r.params[k] == g[k].item(), k
    assert r.params["is_override_manning"] == 1
    assert np.array_equal(solver.mesh_tables(r, r.params)[0], G.reference_table(g))
    # the same case with the mesh's own Manning field
    text = open(os.path.join(d, "donnees.f")).read()
    text = text.replace("is_override_manning=1", "is_override_manning=0")
    text = text.replace("meshfile_path='./'", f"meshfile_path='{d}/'")
    (tmp_path / "donnees.f").write_text(text)
    r0 = case_files.read_case(str(tmp_path))
    assert r0.params["is_override_manning"] == 0
    assert np.array_equal(np.asarray(r0.manning), g["manning"])


def test_cgns_mesh_without_boundary_lists(tmp_path):
    """A CGNS mesh of the reference's calibration example (32-bit connectivity, no ZoneBC, no Manning
    data): read with an override Manning n, every node of it as the independent Python HDF5 reader
    of the golden-fixture script decodes it, and no inflow or outflow node."""
    import os
    d = _reference_case_dir("River_piers/Froude")
    if d is None:
        pytest.skip("CUTEFLOW_REFERENCE does not name a reference checkout")
    from hdf5_min import H5
    mesh = os.path.join(_reference_root(), "Calibration_manning", "Exemple2", "base_files", "mesh_6072.cgns")
    (tmp_path / "donnees.f").write_text(
        f"&donnees_namelist\n is_cgns=1, meshfile_path='{os.path.dirname(mesh)}/', meshfile='mesh_6072.cgns',\n"
        " is_override_manning=1, override_manning=0.03,\n/\n")
    r = case_files.read_case(str(tmp_path))
    h = H5(mesh)
    Z = ["Base", "Zone"]
    for k, name in (("x", "CoordinateX"), ("y", "CoordinateY"), ("z", "CoordinateZ")):
        assert np.array_equal(np.asarray(getattr(r, k)), h.cgns_data(Z + ["GridCoordinates", name])), k
    conn = h.cgns_data(Z + ["Elements", "ElementConnectivity"]).reshape(-1, 3)
    assert r.nelt == 6072 and np.array_equal(np.asarray(r.tri).reshape(-1, 3), conn)
    assert len(r.ndinput) == 0 and len(r.ndoutput) == 0 and np.all(np.asarray(r.manning) == 0.03)


def test_cgns_errors_are_reported(tmp_path):
    """A CGNS mesh that is not HDF5, or is cut short, is an error code with a message."""
    (tmp_path / "mesh.cgns").write_bytes(b"not an hdf5 file at all" * 10)
    (tmp_path / "donnees.f").write_text("&donnees_namelist\n is_cgns=1, meshfile='mesh.cgns',\n/\n")
    with pytest.raises(Exception) as e:
        case_files.read_case(str(tmp_path))
    assert "HDF5" in str(e.value)
    d = _reference_case_dir("River_piers/Froude")
    if d is not None:
        import os
        raw = open(os.path.join(d, "manning_River_wth_piers.cgns"), "rb").read()
        for cut in (100, 2000, len(raw) // 2):
            (tmp_path / "mesh.cgns").write_bytes(raw[:cut])
            with pytest.raises(Exception):
                case_files.read_case(str(tmp_path))
        # one changed byte in an object header fails its checksum
        bad = bytearray(raw)
        at = bad.find(b"OHDR", 64)
        bad[at + 9] ^= 0x01
        (tmp_path / "mesh.cgns").write_bytes(bytes(bad))
        with pytest.raises(Exception) as e:
            case_files.read_case(str(tmp_path))
        assert "checksum" in str(e.value)
