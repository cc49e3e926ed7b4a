"""Golden fixtures for the scheme of the reference's GPU programs.

The reference's CUDA kernel files (CODE/cart_kernels.cu, CODE/spher_kernels.cu)
are compiled as host code by oracle/ref/Makefile and driven through the
per-step sequence of each program's main() (oracle/ref/gpu_emul.cpp).  This
script runs that emulation on small seeded cases and stores inputs and
outputs as tests/golden/A_<case>.npz.  Needs the reference checkout:

    python tests/golden/make_golden_gpu.py [case names]
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
R_MARS = 3387.0  # km


def ricker(nt, dt, f0, t0):
    t = np.arange(nt) * dt - t0
    a = (np.pi * f0 * t) ** 2
    w = (1 - 2 * a) * np.exp(-a)
    return (w / np.abs(w).max()).astype(np.float32)


def layered_cart(rng, n, d):
    """[.. ][n2][n1] velocity: vacuum 300 / ice 168 / basalt 110 (m/us)."""
    n1 = n[0]
    lat = tuple(n[1:])
    z = np.arange(n1) * d
    surf = n1 * d * 0.25 + rng.normal(0, d, size=lat)
    base = n1 * d * 0.7 + rng.normal(0, d, size=lat)
    zz = z.reshape((1,) * len(lat) + (n1,))
    v = np.where(zz < surf[..., None], 300.0, np.where(zz < base[..., None], 168.0, 110.0))
    v = v.astype(np.float32)
    return np.ascontiguousarray(np.transpose(v, tuple(range(len(lat)))[::-1] + (len(lat),)))


CASES = [
    dict(name="A_cart2d_const", kind="cart2d", n=(40, 40), d=(5.0, 5.0), o=(0.0, 0.0), nb=10, nt=300, dt=0.005,
         expl=0, jsnap=100, ns=1, seed=31),
    dict(name="A_cart2d_expl_bnds", kind="cart2d", n=(36, 36), d=(5.0, 5.0), o=(0.0, 0.0), nb=8, nt=240, dt=0.005,
         expl=1, jsnap=80, bnds=1, ns=2, seed=32),
    dict(name="A_cart2d_refl", kind="cart2d", n=(32, 32), d=(5.0, 5.0), o=(0.0, 0.0), nb=6, nt=200, dt=0.005,
         expl=1, refl=1, jsnap=0, ns=1, seed=33),
    dict(name="A_cart3d_const", kind="cart3d", n=(20, 20, 18), d=(5.0, 5.0, 5.0), o=(0.0, 0.0, 0.0), nb=6, nt=110,
         dt=0.005, expl=0, jsnap=55, ns=1, seed=34),
    dict(name="A_cart3d_expl", kind="cart3d", n=(18, 18, 16), d=(5.0, 5.0, 5.0), o=(0.0, 0.0, 0.0), nb=5, nt=90,
         dt=0.005, expl=1, jsnap=0, ns=2, seed=35),
    dict(name="A_polar2d_const", kind="polar2d", n=(48, 40), d=(0.005, 1.5e-6), o=(R_MARS, np.pi / 2 - 20 * 1.5e-6),
         nb=8, nt=300, dt=0.005, expl=0, jsnap=100, ns=1, seed=36),
    dict(name="A_polar2d_free_expl", kind="polar2d", n=(44, 36), d=(0.005, 1.5e-6),
         o=(R_MARS, np.pi / 2 - 18 * 1.5e-6), nb=6, nt=240, dt=0.005, expl=1, fsrf=1, jsnap=80, bnds=1, ns=1,
         seed=37),
    dict(name="A_spher3d_const", kind="spher3d", n=(28, 20, 18), d=(0.005, 1.5e-6, 1.5e-6),
         o=(R_MARS, np.pi / 2 - 10 * 1.5e-6, -9 * 1.5e-6), nb=5, nt=100, dt=0.005, expl=0, jsnap=50, ns=2, seed=38),
    dict(name="A_spher3d_free_expl_bnds", kind="spher3d", n=(24, 18, 16), d=(0.005, 1.5e-6, 1.5e-6),
         o=(R_MARS, np.pi / 2 - 9 * 1.5e-6, -8 * 1.5e-6), nb=5, nt=80, dt=0.005, expl=1, fsrf=1, jsnap=40, bnds=1,
         ns=1, seed=39),
]


def make_inputs(case):
    rng = np.random.default_rng(case["seed"])
    kind, n, d, o = case["kind"], case["n"], case["d"], case["o"]
    nd = len(n)
    ns = case.get("ns", 1)
    if kind.startswith("cart"):
        vel = layered_cart(rng, n, d[0])
        ext = [(n[a] - 1) * d[a] for a in range(nd)]
        if nd == 2:
            sou = np.stack([o[1] + rng.uniform(0.3, 0.7, ns) * ext[1], o[0] + np.full(ns, 0.4 * ext[0])], 1)
            rec = np.stack([o[1] + np.linspace(0.05, 0.95, 10) * ext[1], o[0] + np.full(10, 0.3 * ext[0] + 1.3)], 1)
        else:
            sou = np.stack([o[1] + rng.uniform(0.3, 0.7, ns) * ext[1], o[2] + rng.uniform(0.3, 0.7, ns) * ext[2],
                            o[0] + np.full(ns, 0.4 * ext[0])], 1)
            gx, gy = np.meshgrid(np.linspace(0.1, 0.9, 3) * ext[1], np.linspace(0.1, 0.9, 3) * ext[2], indexing="ij")
            rec = np.stack([o[1] + gx.ravel(), o[2] + gy.ravel(), o[0] + np.full(gx.size, 0.3 * ext[0] + 1.1)], 1)
    else:
        # radius axis 1 (m/us velocities converted to km/us), vacuum above ~r_top - 50 m
        nr_ = n[0]
        r = o[0] + np.arange(nr_) * d[0]
        rtop = o[0] + 0.7 * (nr_ - 1) * d[0]
        shape = tuple(n[1:][::-1]) + (nr_,)
        v = np.where(r[None, :] > rtop, 0.300, np.where(r[None, :] > o[0] + 0.3 * (nr_ - 1) * d[0], 0.168, 0.110))
        v = np.broadcast_to(v.reshape((1,) * (len(shape) - 1) + (nr_,)), shape).astype(np.float32)
        vel = np.ascontiguousarray(v * (1.0 + 0.02 * rng.random(shape).astype(np.float32)))
        if nd == 2:
            sou = np.stack([np.full(ns, rtop - 2.3 * d[0]), o[1] + rng.uniform(0.3, 0.7, ns) * (n[1] - 1) * d[1]], 1)
            rec = np.stack([np.full(10, rtop - 1.5 * d[0]), o[1] + np.linspace(0.05, 0.95, 10) * (n[1] - 1) * d[1]], 1)
        else:
            sou = np.stack([np.full(ns, rtop - 2.3 * d[0]), o[2] + rng.uniform(0.3, 0.7, ns) * (n[2] - 1) * d[2],
                            o[1] + rng.uniform(0.3, 0.7, ns) * (n[1] - 1) * d[1]], 1)
            gp, gt = np.meshgrid(np.linspace(0.1, 0.9, 3) * (n[2] - 1) * d[2],
                                 np.linspace(0.1, 0.9, 3) * (n[1] - 1) * d[1], indexing="ij")
            rec = np.stack([np.full(gp.size, rtop - 1.5 * d[0]), o[2] + gp.ravel(), o[1] + gt.ravel()], 1)
    sou = sou.astype(np.float32)
    rec = rec.astype(np.float32)
    wav = ricker(case["nt"], case["dt"], 5.0, 0.3)
    rfl = None
    if case.get("refl"):
        rfl = (0.2 * rng.random(vel.shape)).astype(np.float32)
    par = dict(kind=kind, n=list(n), d=[float(x) for x in d], o=[float(x) for x in o], nb=case["nb"],
               nt=case["nt"], dt=case["dt"], jdata=1, jsnap=case.get("jsnap", 0), bnds=case.get("bnds", 0),
               fsrf=case.get("fsrf", 0), expl=case.get("expl", 0), refl=case.get("refl", 0))
    return par, vel, wav, sou, rec, rfl


# sfDYNAWEFDcart2Dgpu: sources and receivers read from tables of ns*nst and
# nr*nrt points (entry k*(it+1) at step it), unscaled injection
DYN_CASES = [
    dict(name="A_dyncart2d_move", n=(40, 44), d=(5.0, 5.0), o=(0.0, 0.0), nb=8, nt=220, dt=0.005, ns=3, nr=5,
         jsnap=70, bnds=0, fsrf=0, seed=41),
    dict(name="A_dyncart2d_free_bnds", n=(36, 40), d=(5.0, 5.0), o=(0.0, 0.0), nb=6, nt=180, dt=0.005, ns=2, nr=4,
         jsnap=60, bnds=1, fsrf=1, seed=42),
]


def make_dyn_inputs(case):
    """Tables with nst = nrt = nt rows: every entry k*(it+1), k < n, it < nt,
    exists ((n-1)*nt < n*nt).  Entry e sits on a track crossing the model."""
    rng = np.random.default_rng(case["seed"])
    n, d, o, nt = case["n"], case["d"], case["o"], case["nt"]
    vel = layered_cart(rng, n, d[0])
    ext = [(n[a] - 1) * d[a] for a in range(2)]
    ns, nr = case["ns"], case["nr"]

    def track(count, depth, phase):
        e = np.arange(count)
        u = 0.15 + 0.7 * np.mod(e * 0.618034 + phase, 1.0)
        return np.stack([o[1] + u * ext[1], o[0] + depth * ext[0] + 0.3 * d[0] * np.sin(e * 0.05)], 1)

    sou = track(ns * nt, 0.42, 0.1).astype(np.float32)
    rec = track(nr * nt, 0.3, 0.55).astype(np.float32)
    wav = ricker(nt, case["dt"], 5.0, 0.3)
    par = dict(kind="dyncart2d", n=list(n), d=[float(x) for x in d], o=[float(x) for x in o], nb=case["nb"], nt=nt,
               dt=case["dt"], jdata=1, jsnap=case["jsnap"], bnds=case["bnds"], fsrf=case["fsrf"], expl=0, refl=0,
               ns=ns, nst=nt, nr=nr, nrt=nt)
    return par, vel, wav, sou, rec


# sfAWEFDspher3Dgpu adj=y: the traces of a forward run of the same case go
# back in at the receivers; kt picks the image step nt-kt
ADJ_CASES = [
    dict(name="Aadj_spher3d_snap", base="A_spher3d_const", kt=30, jsnap=25, bnds=0, fsrf=0),
    dict(name="Aadj_spher3d_free_bnds", base="A_spher3d_free_expl_bnds", kt=20, jsnap=20, bnds=1, fsrf=1),
    dict(name="Aadj_spher3d_first_step", base="A_spher3d_const", kt=100, jsnap=0, bnds=0, fsrf=0),
]


def main(only=None):
    oracle.build(with_reference=True)
    by_name = {c["name"]: c for c in CASES}
    for case in ADJ_CASES:
        if only and case["name"] not in only:
            continue
        base = dict(by_name[case["base"]], expl=0, jsnap=0, bnds=0)
        par, vel, wav, sou, rec, _ = make_inputs(base)
        data, _ = oracle.gpu_scheme("spher3d", par, vel, wav, sou, rec, use_reference_emulation=True)
        par = dict(par, jsnap=case["jsnap"], bnds=case["bnds"], fsrf=case["fsrf"], kt=case["kt"])
        image, snaps = oracle.spher3d_adj(par, vel, data, rec, case["kt"], use_reference_emulation=True)
        out = dict(par=np.array(json.dumps(par)), vel=vel, data=data, sou=sou, rec=rec, image=image)
        if snaps is not None:
            out["snaps"] = snaps
        np.savez_compressed(os.path.join(HERE, case["name"] + ".npz"), **out)
        print("%-28s image %s max|image| %.3e frames %s" % (case["name"], image.shape, np.abs(image).max(),
                                                            None if snaps is None else snaps.shape))
    for case in DYN_CASES:
        if only and case["name"] not in only:
            continue
        par, vel, wav, sou, rec = make_dyn_inputs(case)
        dat, snaps = oracle.gpu_cart2d_moving(par, vel, wav, sou, par["nst"], rec, par["nrt"], 1,
                                              use_reference_emulation=True)
        out = dict(par=np.array(json.dumps(par)), vel=vel, wav=wav, sou=sou, rec=rec, dat=dat, snaps=snaps)
        np.savez_compressed(os.path.join(HERE, case["name"] + ".npz"), **out)
        print("%-28s dat %s max|dat| %.3e snaps %s" % (case["name"], dat.shape, np.abs(dat).max(), snaps.shape))
    for case in CASES:
        if only and case["name"] not in only:
            continue
        par, vel, wav, sou, rec, rfl = make_inputs(case)
        dat, snaps = oracle.gpu_scheme(par["kind"], par, vel, wav, sou, rec, rfl=rfl, use_reference_emulation=True)
        out = dict(par=np.array(json.dumps(par)), vel=vel, wav=wav, sou=sou, rec=rec, dat=dat)
        if rfl is not None:
            out["rfl"] = rfl
        if snaps is not None:
            out["snaps"] = snaps
        np.savez_compressed(os.path.join(HERE, case["name"] + ".npz"), **out)
        print("%-28s dat %s max|dat| %.3e snaps %s" % (case["name"], dat.shape, np.abs(dat).max(),
                                                        None if snaps is None else snaps.shape))


if __name__ == "__main__":
    main(sys.argv[1:] or None)
