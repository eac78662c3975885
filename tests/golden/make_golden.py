"""Build the golden fixtures of tests/golden/ from the reference checkout (run here, once; the
outputs are committed, so the tests never read the reference at run time).

Sources, all produced by the reference itself on a Tesla P100 and shipped in its repository:
  Calibration_manning/docs_calibration/River_piers/Froude/
      manning_River_wth_piers.cgns             mesh (CGNS/HDF5): 767 nodes, 1408 triangles
      boundary_table_manning_River_wth_piers.cgns   the neighbour/boundary table CuteFlow wrote
      donnees.f                                the namelist of the run
      outfile.out                              the run's log: t and outflow discharge every 1000 steps
  Calibration_manning/docs_calibration/Divergent_Canal/Froude/
      manning_Canal_divergent.cgns, boundary_table_manning_Canal_divergent.cgns,
      outfile_manning_min.out, outfile_manning_max.out   two runs on the same mesh

The Divergent_Canal logs differ from the donnees.f next to them only in the printed values
(debitglob 0.5, H_sortie 0.02); the Manning override of each run is not printed.  The values used
here (0.01 and 0.05) are the ones that reproduce the logged discharge to every printed digit.

    python tests/golden/make_golden.py /path/to/reference   (or CUTEFLOW_REFERENCE=/path/to/reference)
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from hdf5_min import H5  # noqa: E402


def read_mesh(path):
    h = H5(path)
    Z = ["Base", "Zone"]
    return dict(
        x=h.cgns_data(Z + ["GridCoordinates", "CoordinateX"]).astype(np.float64),
        y=h.cgns_data(Z + ["GridCoordinates", "CoordinateY"]).astype(np.float64),
        z=h.cgns_data(Z + ["GridCoordinates", "CoordinateZ"]).astype(np.float64),
        tri=h.cgns_data(Z + ["Elements", "ElementConnectivity"]).reshape(-1, 3).astype(np.int32),
        ndinput=h.cgns_data(Z + ["ZoneBC", "Inflow nodes", "PointList"]).ravel().astype(np.int32),
        ndoutput=h.cgns_data(Z + ["ZoneBC", "Outflow nodes", "PointList"]).ravel().astype(np.int32),
        manning=h.cgns_data(Z + ["Manning", "{DataArray}"]).ravel().astype(np.float64),
    )


def read_log(path):
    text = open(path).read()
    steps = [int(v) for v in re.findall(r"Iteration number\s+(\d+) , t =", text)]
    t = [float(v) for v in re.findall(r"Iteration number\s+\d+ , t =\s+(\S+)", text)]
    q_in = [float(v) for v in re.findall(r"debit_entree_sum =\s+(\S+)", text)]
    q_out = [float(v) for v in re.findall(r"debit_sortie\s+=\s+(\S+)", text)]
    cotemin = float(re.search(r"cotemin\s+=\s+(\S+)", text).group(1))
    n = min(len(steps), len(t), len(q_out), len(q_in))
    return dict(log_steps=np.array(steps[:n]), log_t=np.array(t[:n]), log_q_in=np.array(q_in[:n]),
                log_q_out=np.array(q_out[:n]), log_cotemin=cotemin)


def read_table(path):
    a = np.loadtxt(path, dtype=np.int64)
    return np.stack([a[:, 0:3], a[:, 3:6]], axis=2).astype(np.int32)  # boundary(k, j, 1:2), before walls


# where the reference checkout is read from when no path is given: the CUTEFLOW_REFERENCE
# environment variable (tests that read its case directories directly use the same variable and
# are skipped when it is unset)
def reference_root():
    return os.environ.get("CUTEFLOW_REFERENCE") or None


def main(ref):
    cal = os.path.join(ref, "Calibration_manning", "docs_calibration")
    rp = os.path.join(cal, "River_piers", "Froude")
    dc = os.path.join(cal, "Divergent_Canal", "Froude")
    m = read_mesh(os.path.join(rp, "manning_River_wth_piers.cgns"))
    np.savez_compressed(
        os.path.join(HERE, "river_piers.npz"), **m, **read_log(os.path.join(rp, "outfile.out")),
        boundary_table=read_table(os.path.join(rp, "boundary_table_manning_River_wth_piers.cgns")),
        # donnees.f of the run
        override_manning=0.01, debitglob=62.0, h_sortie=0.0001, cfl=0.6, tolisec=1e-5, gp=9.81, iflux=2,
        ilimiteur=3, fricimplic=1, zpoint=0.05, xpoint=14.6282, ypoint=17.8976)
    m = read_mesh(os.path.join(dc, "manning_Canal_divergent.cgns"))
    logs = {}
    for tag, fname, nman in (("min", "outfile_manning_min.out", 0.01), ("max", "outfile_manning_max.out", 0.05)):
        lg = read_log(os.path.join(dc, fname))
        logs.update({f"{k}_{tag}": v for k, v in lg.items()})
        logs[f"override_manning_{tag}"] = nman
    np.savez_compressed(
        os.path.join(HERE, "divergent_canal.npz"), **m, **logs,
        boundary_table=read_table(os.path.join(dc, "boundary_table_manning_Canal_divergent.cgns")),
        debitglob=0.5, h_sortie=0.02, cfl=0.9, tolisec=1e-5, gp=9.81, iflux=2, ilimiteur=3, fricimplic=1,
        zpoint=0.016, xpoint=10.0, ypoint=0.75)
    print("wrote river_piers.npz, divergent_canal.npz")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else reference_root()
    if not root:
        sys.exit("usage: make_golden.py /path/to/reference  (or set CUTEFLOW_REFERENCE)")
    main(root)
