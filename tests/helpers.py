"""Shared helpers: golden fixtures and running the engine on a case."""
import glob
import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_paths(pattern="c*.npz"):
    return sorted(glob.glob(os.path.join(GOLDEN_DIR, pattern)))


def load_golden(path):
    z = np.load(path)
    par = json.loads(str(z["par"]))
    return par, {k: z[k] for k in z.files if k != "par"}


def desc_from_par(par, precision=0, scheme=1, coords=0):
    from wavefield_imaging_gb300 import make_desc

    nd = len(par["n"])
    return make_desc(nd, par["n"], par["d"], par["o"], par["nt"], par["dt"], coords=coords, scheme=scheme,
                     nb=par.get("nb", -1), fdorder=par.get("fdorder", 0), optfd=par.get("optfd", 0),
                     dabc=par.get("dabc", 0), hybrid=par.get("hybrid", 0), fsrf=par.get("fsrf", 0),
                     expl=par.get("expl", 0), refl=par.get("refl", 0), jdata=par.get("jdata", 1),
                     jsnap=par.get("jsnap", 0), bnds=par.get("bnds", 0), precision=precision)


def run_engine(par, vel, wav, sou, rec, den=None, precision=0, scheme=1, coords=0, rfl=None):
    from wavefield_imaging_gb300 import Plan

    with Plan(desc_from_par(par, precision, scheme, coords)) as p:
        p.set_model(vel, den=den, rfl=rfl)
        p.set_geometry(sou, rec)
        if par.get("jsnap", 0) > 0:
            dat, snaps = p.forward(wav, snapshots=True)
        else:
            dat, snaps = p.forward(wav), None
        return dat, snaps, p.last_launch_count()


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)
