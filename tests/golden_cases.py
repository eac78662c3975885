"""Cases built from the golden fixtures (tests/golden/*.npz, made by make_golden.py from the
reference's own calibration meshes, boundary tables and run logs)."""
import os

import numpy as np

from cuteflow_gb300 import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def case(name, tag=""):
    """(Case, initial condition dict, log dict) of a logged reference run."""
    d = load(name)
    sfx = f"_{tag}" if tag else ""
    params = dict(gp=float(d["gp"]), is_override_manning=1, override_manning=float(d["override_manning" + sfx]),
                  inlet=2, outlet=1, debitglob=[float(d["debitglob"])], h_sortie=[float(d["h_sortie"])],
                  iflux=int(d["iflux"]), ilimiteur=int(d["ilimiteur"]), tolisec=float(d["tolisec"]), friction=1,
                  fricimplic=int(d["fricimplic"]), cfl=float(d["cfl"]))
    c = cases.Case(x=d["x"], y=d["y"], z=d["z"], tri=d["tri"], manning=d["manning"], ndinput=d["ndinput"],
                   numero_ndinput=np.ones_like(d["ndinput"]), ndoutput=d["ndoutput"],
                   numero_ndoutput=np.ones_like(d["ndoutput"]), ndwall=np.zeros(0, np.int32), nombre_entrees=1,
                   nombre_sorties=1, params=params, U0=np.zeros((d["tri"].shape[0], 3)), name=name + sfx)
    ic = dict(eqlin_barrage=0, plan=1, xplan=0.0, yplan=0.0, zplan=1.0, xpoint=float(d["xpoint"]),
              ypoint=float(d["ypoint"]), zpoint=float(d["zpoint"]))
    log = {k[:-len(sfx)] if sfx and k.endswith(sfx) else k: d[k] for k in d if k.startswith("log_") and k.endswith(sfx)}
    return c, ic, log, d


def reference_table(d):
    """The boundary table the reference wrote (before set_undefined_boudaries_as_walls turns
    the remaining self-references into walls, main.cuf:76)."""
    b = d["boundary_table"].copy()
    ids = np.arange(1, b.shape[0] + 1)[:, None]
    b[:, :, 0] = np.where(b[:, :, 0] == ids, -3, b[:, :, 0])
    return b


RUNS = [("river_piers", ""), ("divergent_canal", "min"), ("divergent_canal", "max")]
