"""Golden fixtures for the point-cloud tools, written by the reference's own
programs: CODE/Mbycloudwin3d.c and CODE/Mbycloudmerge3d.c (+ hash.c), built
unchanged by oracle/ref/Makefile against the project's RSF stand-in.  Seeded
ground clouds on a patch of a sphere (Mars radius, outward normals), orbit
stretches above it, random data columns; each case windows the cloud for
every orbit stretch and merges the windows' data back.  Needs the reference
checkout:

    python tests/golden/make_golden_cloud.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from wavefield_imaging_gb300 import rsf  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(ROOT, "oracle", "_ref")
R_MARS = 3390.0  # km

CASES = [
    dict(name="pc_complex_norm", ng=700, nf=5, apt=3.0, complex=True, norm=True, seed=51,
         stretches=[(-0.010, 0.0), (-0.002, 0.006)]),
    dict(name="pc_real_fold", ng=500, nf=4, apt=5.0, complex=False, norm=False, seed=52,
         stretches=[(-0.012, -0.004), (-0.006, 0.002), (0.0, 0.008)]),
]


def make_cloud(case):
    rng = np.random.default_rng(case["seed"])
    ng = case["ng"]
    th = rng.uniform(-0.02, 0.02, ng)
    ph = rng.uniform(-0.02, 0.02, ng)
    rad = R_MARS + rng.normal(0, 0.05, ng)
    xyz = np.stack([rad * np.cos(th) * np.cos(ph), rad * np.cos(th) * np.sin(ph), rad * np.sin(th)], 1)
    nrm = xyz / np.linalg.norm(xyz, axis=1, keepdims=True)
    nrm = nrm + rng.normal(0, 0.02, nrm.shape)  # rough surface: tilted normals
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    cloud = np.zeros((ng, 9), np.float32)
    cloud[:, :3] = xyz
    cloud[:, 3:6] = nrm
    cloud[:, 6:] = rng.normal(size=(ng, 3))
    orbits = []
    for s0, s1 in case["stretches"]:
        t = np.linspace(s0, s1, 9)
        o = np.zeros((t.size, 9), np.float32)
        o[:, 0] = (R_MARS + 300) * np.cos(t)
        o[:, 1] = (R_MARS + 300) * np.sin(0.3 * t)
        o[:, 2] = (R_MARS + 300) * np.sin(t)
        orbits.append(o)
    shape = (case["nf"], ng)
    if case["complex"]:
        data = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64)
    else:
        data = rng.normal(size=shape).astype(np.float32)
    return cloud, orbits, data


def run(args, stdin_path, stdout_path):
    with open(stdin_path) if stdin_path else open(os.devnull) as fi, open(stdout_path, "w") as fo:
        r = subprocess.run(args, stdin=fi, stdout=fo, stderr=subprocess.PIPE)
    if r.returncode != 0:
        raise RuntimeError("%s failed: %s" % (args[0], r.stderr.decode()[-500:]))


def main():
    oracle.build(with_reference=True)
    for case in CASES:
        cloud, orbits, data = make_cloud(case)
        out = dict(par=np.array(json.dumps({k: v for k, v in case.items() if k != "stretches"})), cloud=cloud,
                   data=data)
        with tempfile.TemporaryDirectory() as tmp:
            rsf.write(os.path.join(tmp, "cloud.rsf"), cloud, [(9, 0, 1), (cloud.shape[0], 0, 1)])
            if not case["complex"]:
                # Mbycloudwin3d reads complex data; real windows are cut from the real part
                dc = data.astype(np.complex64)
            else:
                dc = data
            rsf.write(os.path.join(tmp, "dat.rsf"), dc, [(cloud.shape[0], 0, 1), (data.shape[0], 0, 1)])
            cw, dw = [], []
            for k, orb in enumerate(orbits):
                rsf.write(os.path.join(tmp, "oo%d.rsf" % k), orb, [(9, 0, 1), (orb.shape[0], 0, 1)])
                run([os.path.join(REF, "sfbycloudwin3d"), "oo=" + os.path.join(tmp, "oo%d.rsf" % k),
                     "dat=" + os.path.join(tmp, "dat.rsf"), "dout=" + os.path.join(tmp, "dw%d.rsf" % k),
                     "apt=%g" % case["apt"], "verb=n"], os.path.join(tmp, "cloud.rsf"), os.path.join(tmp, "cw%d.rsf" % k))
                c, _ = rsf.read(os.path.join(tmp, "cw%d.rsf" % k))
                d, _ = rsf.read(os.path.join(tmp, "dw%d.rsf" % k))
                if not case["complex"]:  # real window data files for the merge
                    d = d.real.astype(np.float32)
                    rsf.write(os.path.join(tmp, "dw%d.rsf" % k), d, [(d.shape[1], 0, 1), (d.shape[0], 0, 1)])
                out["orbit%d" % k] = orb
                out["win%d" % k] = c
                out["wdat%d" % k] = d
                cw.append(os.path.join(tmp, "cw%d.rsf" % k))
                dw.append(os.path.join(tmp, "dw%d.rsf" % k))
            run([os.path.join(REF, "sfbycloudmerge3d"), *cw, *dw, "all=" + os.path.join(tmp, "cloud.rsf"),
                 "norm=%s" % ("y" if case["norm"] else "n")], None, os.path.join(tmp, "merged.rsf"))
            m, _ = rsf.read(os.path.join(tmp, "merged.rsf"))
            out["merged"] = m
        np.savez_compressed(os.path.join(HERE, case["name"] + ".npz"), **out)
        print("%-22s windows %s merged %s %s" % (case["name"], [out["win%d" % k].shape[0] for k in range(len(orbits))],
                                                 m.shape, m.dtype))


if __name__ == "__main__":
    main()
