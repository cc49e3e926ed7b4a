"""Generate golden fixtures by running the reference's own CPU programs.

Runs oracle/_ref/sfAWEFDcart2Dcpu and sfAWEFDcart3Dcpu - built unchanged from
Nacnud04/wavefield_imaging CODE/ sources by oracle/ref/Makefile - on small
seeded inputs, and stores inputs + outputs as tests/golden/<case>.npz.
The fixtures pin the oracle restatement (tests/test_oracle_golden.py) and,
through it, the CUDA path.  Needs the reference checkout, so it only runs in
the development container:

    python tests/golden/make_golden.py
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


def ricker(nt, dt, f0, t0):
    t = np.arange(nt) * dt - t0
    a = (np.pi * f0 * t) ** 2
    w = (1 - 2 * a) * np.exp(-a)
    return (w / np.abs(w).max()).astype(np.float32)


def layered(rng, shape_zx, dz, vmin=110.0, vmax=300.0):
    """Seeded layered model: vacuum (300) over ice (168, with thin dust
    layers) over basalt (110), random interfaces.  shape_zx = (nz, nx[, ny])."""
    nz = shape_zx[0]
    lat = shape_zx[1:]
    z = np.arange(nz)[:, None] * dz
    surf = nz * dz * 0.2 + rng.normal(0, 2 * dz, size=int(np.prod(lat)))
    base = nz * dz * 0.75 + rng.normal(0, 2 * dz, size=int(np.prod(lat)))
    v = np.where(z < surf[None, :], 300.0, np.where(z < base[None, :], 168.0, 110.0))
    for _ in range(2):
        zd = rng.uniform(0.3, 0.65) * nz * dz
        th = rng.uniform(1.5, 3.0) * dz
        v = np.where((np.abs(z - zd) < th) & (v == 168.0), 168.0 * rng.choice([0.95, 1.05]), v)
    v = v.reshape((nz,) + tuple(lat)).astype(np.float32)
    # reorder to [.. n2][n1] (axis 1 = z fastest)
    return np.ascontiguousarray(np.moveaxis(v, 0, -1)) if v.ndim == 2 else np.ascontiguousarray(
        np.transpose(v, (2, 1, 0))
    )


CASES_2D = [
    dict(name="c2d_o8_sponge", n=(48, 64), nb=12, nt=360, fdorder=8, dabc=1, expl=1, jsnap=90, seed=1),
    dict(name="c2d_o4_free_den", n=(40, 52), nb=8, nt=300, fdorder=4, dabc=1, fsrf=1, expl=0, den=1, ns=2,
         jsnap=100, seed=2),
    dict(name="c2d_o2_plain", n=(36, 44), nb=-1, nt=250, fdorder=2, dabc=0, expl=1, jsnap=0, seed=3),
    dict(name="c2d_o6_optfd_bnds", n=(40, 40), nb=10, nt=240, fdorder=6, optfd=1, dabc=1, expl=1, jsnap=80,
         bnds=1, seed=4),
    dict(name="c2d_o8_hybrid", n=(44, 50), nb=14, nt=300, fdorder=8, dabc=1, hybrid=1, expl=1, jsnap=0, seed=5),
    dict(name="c2d_o8_edge_geometry", n=(32, 36), nb=8, nt=200, fdorder=8, dabc=1, expl=1, jsnap=0, seed=6,
         edge=1),
    # snapshot window reaching into the padding, with strides and a non-node origin
    dict(name="c2d_o8_window", n=(48, 64), nb=12, nt=200, fdorder=8, dabc=1, expl=1, jsnap=50, seed=7,
         win=dict(nqz=20, oqz=-20.0, dqz=10.0, nqx=15, oqx=32.5, dqx=15.0)),
]
CASES_3D = [
    dict(name="c3d_o8_sponge", n=(22, 24, 20), nb=8, nt=140, fdorder=8, dabc=1, expl=1, jsnap=70, seed=11),
    dict(name="c3d_o4_free_den", n=(18, 20, 22), nb=6, nt=120, fdorder=4, dabc=1, fsrf=1, expl=0, den=1, ns=2,
         jsnap=0, seed=12),
    dict(name="c3d_o8_hybrid", n=(20, 18, 18), nb=10, nt=110, fdorder=8, dabc=1, hybrid=1, expl=1, jsnap=0,
         seed=13),
    dict(name="c3d_o2_plain", n=(16, 18, 20), nb=-1, nt=100, fdorder=2, dabc=0, expl=1, jsnap=0, seed=14),
    # padded axis 1 a multiple of 4: the shape the TMA-staged 3D kernel takes
    dict(name="c3d_o8_tma_shape", n=(24, 20, 18), nb=8, nt=120, fdorder=8, dabc=1, expl=1, jsnap=60, seed=15),
    dict(name="c3d_o8_tma_free", n=(28, 22, 20), nb=10, nt=100, fdorder=8, dabc=1, fsrf=1, expl=0, ns=2, jsnap=0,
         seed=16),
    # snapshot window on all three axes, partly in the padding
    dict(name="c3d_o8_window", n=(24, 20, 18), nb=8, nt=80, fdorder=8, dabc=1, expl=1, jsnap=40, seed=17,
         win=dict(nqz=10, oqz=-15.0, dqz=10.0, nqx=6, oqx=12.0, dqx=5.0, nqy=4, oqy=-10.0, dqy=15.0)),
    # bnds=y: whole padded planes; oqy at the padded origin keeps the reference's y planes on the grid
    dict(name="c3d_o8_bnds", n=(24, 20, 18), nb=8, nt=80, fdorder=8, dabc=1, expl=1, jsnap=40, bnds=1, seed=18,
         win=dict(oqy=-40.0)),
]


def make_inputs(case):
    rng = np.random.default_rng(case["seed"])
    n = case["n"]
    ndim = len(n)
    d = 5.0
    dt = 0.005
    nz = n[0]
    lat = n[1:]
    vel = layered(rng, (nz,) + tuple(lat[::-1]) if ndim == 3 else (nz, lat[0]), d)
    if ndim == 3:
        vel = vel.reshape(n[2], n[1], n[0])
    else:
        vel = vel.reshape(n[1], n[0])
    den = None
    if case.get("den"):
        den = (1.0 + 0.5 * rng.random(vel.shape)).astype(np.float32)
    ns = case.get("ns", 1)
    nt = case["nt"]
    o = [0.0] * ndim
    ext = [(k - 1) * d for k in n]  # model extent per axis (z, x, y)
    if ndim == 2:
        sou = np.stack([rng.uniform(0.3, 0.7, ns) * ext[1], np.full(ns, 0.35 * ext[0]) + rng.uniform(0, d, ns)], 1)
        nr = 12
        rec = np.stack([np.linspace(0.05, 0.95, nr) * ext[1], np.full(nr, 0.3 * ext[0] + 1.3)], 1)
        if case.get("edge"):
            # receivers outside the padded grid (fall back to node (0,0)), on
            # grid nodes and at the padded edge; a source on a grid node
            rec[0] = [-1000.0, 5.0]
            rec[1] = [3 * d, 4 * d]
            rec[2] = [ext[1], ext[0]]
            sou[0] = [10 * d, 8 * d]
    else:
        sou = np.stack(
            [
                rng.uniform(0.3, 0.7, ns) * ext[1],
                rng.uniform(0.3, 0.7, ns) * ext[2],
                np.full(ns, 0.35 * ext[0]) + rng.uniform(0, d, ns),
            ],
            1,
        )
        gx, gy = np.meshgrid(np.linspace(0.1, 0.9, 4) * ext[1], np.linspace(0.1, 0.9, 3) * ext[2], indexing="ij")
        rec = np.stack([gx.ravel(), gy.ravel(), np.full(gx.size, 0.3 * ext[0] + 1.1)], 1)
    sou = sou.astype(np.float32)
    rec = rec.astype(np.float32)
    w = ricker(nt, dt, 5.0, 0.3)
    if case.get("expl", 0):
        wav = w
    else:
        wav = np.stack([w * (1.0 + 0.5 * s) for s in range(ns)], 1).astype(np.float32)
    par = dict(n=list(n), d=[d] * ndim, o=o, nb=case["nb"], nt=nt, dt=dt, fdorder=case["fdorder"],
               optfd=case.get("optfd", 0), dabc=case.get("dabc", 0), fsrf=case.get("fsrf", 0),
               hybrid=case.get("hybrid", 0), expl=case.get("expl", 0), jsnap=case.get("jsnap", 0),
               bnds=case.get("bnds", 0))
    if case.get("win"):
        par["win"] = case["win"]
    return par, vel, den, wav, sou, rec


def run_reference(par, vel, den, wav, sou, rec, tmp):
    ndim = len(par["n"])
    prog = os.path.join(ROOT, "oracle", "_ref", "sfAWEFDcart%dDcpu" % ndim)
    ax = [(par["n"][i], par["o"][i], par["d"][i]) for i in range(ndim)]
    rsf.write(os.path.join(tmp, "vel.rsf"), vel, ax)
    if den is not None:
        rsf.write(os.path.join(tmp, "den.rsf"), den, ax)
    nt = par["nt"]
    if par["expl"]:
        rsf.write(os.path.join(tmp, "wav.rsf"), wav.reshape(nt, 1), [(1, 0, 1), (nt, 0, par["dt"])])
    else:
        rsf.write(os.path.join(tmp, "wav.rsf"), wav, [(wav.shape[1], 0, 1), (nt, 0, par["dt"])])
    rsf.write(os.path.join(tmp, "sou.rsf"), sou, [(ndim, 0, 1), (sou.shape[0], 0, 1)])
    rsf.write(os.path.join(tmp, "rec.rsf"), rec, [(ndim, 0, 1), (rec.shape[0], 0, 1)])
    yn = lambda b: "y" if b else "n"  # noqa: E731
    args = [prog, "vel=vel.rsf", "sou=sou.rsf", "rec=rec.rsf", "fdorder=%d" % par["fdorder"],
            "dabc=" + yn(par["dabc"]), "free=" + yn(par["fsrf"]), "expl=" + yn(par["expl"]),
            "hybridbc=" + yn(par["hybrid"]), "optfd=" + yn(par["optfd"]), "ompnth=2", "verb=n"]
    if par["nb"] >= 0:
        args.append("nb=%d" % par["nb"])
    if den is not None:
        args.append("den=den.rsf")
    else:
        args.append("cden=y")
    if par["jsnap"] > 0:
        args += ["snap=y", "jsnap=%d" % par["jsnap"], "wfl=wfl.rsf", "bnds=" + yn(par["bnds"])]
        args += ["%s=%s" % (k, v) for k, v in par.get("win", {}).items()]
    with open(os.path.join(tmp, "wav.rsf")) as fin, open(os.path.join(tmp, "dat.rsf"), "w") as fout:
        subprocess.check_call(args, stdin=fin, stdout=fout, stderr=subprocess.DEVNULL, cwd=tmp)
    dat = np.fromfile(os.path.join(tmp, "dat.rsf@"), dtype="<f4").reshape(nt, rec.shape[0])
    snaps = None
    if par["jsnap"] > 0:
        snaps = np.fromfile(os.path.join(tmp, "wfl.rsf@"), dtype="<f4")
    return dat, snaps


def main():
    oracle.build(with_reference=True)
    only = set(sys.argv[1:])  # case names to (re)make; all when none are given
    for case in CASES_2D + CASES_3D:
        if only and case["name"] not in only:
            continue
        par, vel, den, wav, sou, rec = make_inputs(case)
        with tempfile.TemporaryDirectory() as tmp:
            dat, snaps = run_reference(par, vel, den, wav, sou, rec, tmp)
        out = dict(par=np.array(json.dumps(par)), vel=vel, wav=wav, sou=sou, rec=rec, dat=dat)
        if den is not None:
            out["den"] = den
        if snaps is not None:
            out["snaps"] = snaps
        np.savez_compressed(os.path.join(HERE, case["name"] + ".npz"), **out)
        print("%-24s dat %s max|dat| %.3e snaps %s" % (case["name"], dat.shape, np.abs(dat).max(),
                                                        None if snaps is None else snaps.shape))


if __name__ == "__main__":
    main()
