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
    """One engine run of a fixture's case.  A fixture with a snapshot window
    (par["win"], written by the cpu programs) is run with padded frames, cut
    to the window as the programs cut them (oracle.snapshot_window)."""
    from wavefield_imaging_gb300 import Plan

    jsnap = par.get("jsnap", 0)
    windowed = bool(par.get("win")) and jsnap > 0 and not (len(par["n"]) == 2 and par.get("bnds"))
    with Plan(desc_from_par(dict(par, bnds=1) if windowed else par, precision, scheme, coords)) as p:
        p.set_model(vel, den=den, rfl=rfl)
        p.set_geometry(sou, rec)
        if jsnap > 0:
            dat, snaps = p.forward(wav, snapshots=True)
        else:
            dat, snaps = p.forward(wav), None
        launches = p.last_launch_count()
    if windowed:
        from oracle import oracle

        nbd, n1p, n2p, n3p = oracle.padded(par)
        win = oracle.snapshot_window(par, nbd, (n1p, n2p, n3p))
        frames = np.asarray(snaps).reshape(-1, n1p * n2p * n3p)
        snaps = np.stack([oracle.cut_window(f, win, (n1p, n2p, n3p)) for f in frames])
    return dat, snaps, launches


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def ricker(nt, dt, f0=5.0):
    t = np.arange(nt) * dt - 1.5 / f0
    a = (np.pi * f0 * t) ** 2
    return ((1 - 2 * a) * np.exp(-a)).astype(np.float32)


def grad_case(nd, fsrf=0, dabc=1, nt=200, seed=0, n=None, nb=8, nrec=9):
    """A small seeded gradient problem of the CPU-program scheme (8th order):
    returns (par, vel, wav, sou, rec, vtrue) with vtrue a perturbed model for
    the observed data."""
    rng = np.random.default_rng(seed)
    if n is None:
        n = [48, 56] if nd == 2 else [24, 26, 22]
    shape = tuple(n[::-1])
    d = 5.0
    vel = (150 + 30 * rng.random(shape)).astype(np.float32)
    vtrue = (vel * (1 + 0.05 * rng.standard_normal(shape))).astype(np.float32)
    par = dict(n=list(n), d=[d] * nd, o=[0.0] * nd, nb=nb, nt=nt, dt=0.005, fdorder=8, dabc=dabc, fsrf=fsrf, expl=1)
    wav = ricker(nt, 0.005)
    if nd == 2:
        sou = np.array([[0.5 * (n[1] - 1) * d, 0.3 * (n[0] - 1) * d]], np.float32)
        rec = np.stack([np.linspace(10, (n[1] - 2) * d, nrec), np.full(nrec, 0.6 * (n[0] - 1) * d)], 1)
    else:
        sou = np.array([[0.5 * (n[1] - 1) * d, 0.45 * (n[2] - 1) * d, 0.3 * (n[0] - 1) * d]], np.float32)
        gx, gy = np.meshgrid(np.linspace(10, (n[1] - 2) * d, 4), np.linspace(10, (n[2] - 2) * d, 3), indexing="ij")
        rec = np.stack([gx.ravel(), gy.ravel(), np.full(gx.size, 0.6 * (n[0] - 1) * d)], 1)
    return par, vel, wav, sou, rec.astype(np.float32), vtrue


def tapered_direction(shape, rng, margin=3):
    """Random model direction, zero within `margin` cells of every face (so the
    padding and the one-way ABC coefficients do not move)."""
    dm = rng.standard_normal(shape)
    for ax in range(len(shape)):
        idx = [slice(None)] * len(shape)
        for k in range(margin):
            idx[ax] = k
            dm[tuple(idx)] = 0
            idx[ax] = -1 - k
            dm[tuple(idx)] = 0
    return dm


def spher_grad_case(fsrf=0, nt=150, seed=3, n=(45, 20, 20), nb=8):
    """A small seeded gradient problem of the spherical GPU-program scheme:
    the 700 x 512 x 512 shell's spacing (5 m in r, 0.04/512 rad in theta and phi) on a (r, theta,
    phi) = n grid near r = 3388 km, ice over basalt with 2 % noise, one
    source and 7 receivers above it, close to the free surface.  Returns
    (par, vel, wav, sou, rec, vtrue); models are [nphi][ntheta][nr]."""
    rng = np.random.default_rng(seed)
    d = (0.005, 0.04 / 512, 0.04 / 512)
    o = (3388.0, np.pi / 2 - 10 * d[1], -10 * d[2])
    r = o[0] + np.arange(n[0]) * d[0]
    vel = np.full((n[2], n[1], n[0]), 0.168, np.float32)
    vel[:, :, r > o[0] + 0.15] = 0.110
    vel *= (1 + 0.02 * rng.standard_normal(vel.shape)).astype(np.float32)
    vtrue = vel.copy()
    vtrue[:, :, 20:30] *= np.float32(1.05)
    par = dict(n=list(n), d=list(d), o=list(o), nb=nb, nt=nt, dt=0.005, fsrf=fsrf, expl=0)
    th0, ph0 = o[1] + 9.5 * d[1], o[2] + 9.5 * d[2]
    sou = np.array([[o[0] + 0.17, ph0, th0]], np.float32)
    rec = np.array([[o[0] + 0.12 + 0.012 * k, ph0 + (k - 3) * d[2], th0 + (k % 3 - 1) * d[1]] for k in range(7)],
                   np.float32)
    return par, vel, ricker(nt, 0.005), sou, rec, vtrue


def spher_desc(par, precision=0):
    import wavefield_imaging_gb300 as awe

    return awe.make_desc(3, par["n"], par["d"], par["o"], par["nt"], par["dt"], coords=awe.SPHER,
                         scheme=awe.SCHEME_GPU, nb=par["nb"], fsrf=par.get("fsrf", 0), expl=par.get("expl", 0),
                         precision=precision)
