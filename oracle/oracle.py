"""ctypes front end of the C oracle (awe_oracle.c) - test infrastructure only.

``build()`` compiles liboracle.so (exact float restatement),
liboracle64.so (same scheme, FP64 wavefields) and liboracle_adj.so (FP64
adjoint / misfit gradient, awe_adjoint.c) with gcc and, when the
reference sources are present, the reference's own CPU programs into
oracle/_ref/ (via oracle/ref/Makefile).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# The reference checkout (its CODE/ directory holds the programs): the
# AWE_REFERENCE environment variable, else a directory named "reference"
# beside this repository.  Absent (as on a machine without the checkout),
# build() skips the reference programs.
REF_SRC = os.path.join(os.environ.get("AWE_REFERENCE") or
                       os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"), "CODE")

CFLAGS = ["-std=gnu99", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall"]


def build(with_reference: bool = True) -> None:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "awe_oracle.c"), os.path.join(HERE, "awe_oracle_gpu.c"), os.path.join(HERE, "awe_cloud.c")]
    for name, extra in (("liboracle.so", []), ("liboracle64.so", ["-DAWE_REAL_DOUBLE"])):
        out = os.path.join(BUILD, name)
        if not os.path.exists(out) or os.path.getmtime(out) < max(
            [os.path.getmtime(x) for x in srcs] + [os.path.getmtime(os.path.join(HERE, "awe_oracle.h"))]
        ):
            subprocess.check_call(["gcc", *CFLAGS, *extra, *srcs, "-o", out, "-lm"])
    # FP64 adjoint of the CPU-program scheme (includes awe_oracle.c)
    # and of the spherical GPU-program scheme (awe_adjoint_sph.c, includes awe_oracle_gpu.c)
    adj = [os.path.join(HERE, "awe_adjoint.c"), os.path.join(HERE, "awe_adjoint_sph.c")]
    out = os.path.join(BUILD, "liboracle_adj.so")
    deps = adj + [os.path.join(HERE, x) for x in ("awe_oracle.c", "awe_oracle_gpu.c", "awe_oracle.h")]
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(x) for x in deps):
        subprocess.check_call(["gcc", *CFLAGS, *adj, "-o", out, "-lm"])
    if with_reference and os.path.isdir(REF_SRC):
        subprocess.check_call(
            ["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + REF_SRC, "OUT=" + REF_OUT],
            stdout=subprocess.DEVNULL,
        )
    # the reference's sfAWEFDcart3Dcpu from its staged sources (also where the
    # checkout is absent), the CPU reference timed by bench.py --impl reference
    if os.path.isfile(os.path.join(REF_OUT, "cpuprog", "MAWEFDcart3Dcpu.c")):
        r = subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "-f", "Makefile.cpu", "OUT=" + REF_OUT],
                           stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
        if r.returncode != 0:  # the port stays the CPU reference
            print("oracle: the reference CPU program did not build: %s" % r.stderr[-500:])


class Par(C.Structure):
    _fields_ = [
        ("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int),
        ("d1", C.c_float), ("d2", C.c_float), ("d3", C.c_float),
        ("o1", C.c_float), ("o2", C.c_float), ("o3", C.c_float),
        ("nb", C.c_int), ("nt", C.c_int), ("dt", C.c_float),
        ("fdorder", C.c_int), ("optfd", C.c_int), ("dabc", C.c_int), ("fsrf", C.c_int),
        ("hybrid", C.c_int), ("expl", C.c_int), ("jsnap", C.c_int), ("bnds", C.c_int),
        ("nthreads", C.c_int),
    ]


class GPar(C.Structure):
    _fields_ = [
        ("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int),
        ("d1", C.c_float), ("d2", C.c_float), ("d3", C.c_float),
        ("o1", C.c_float), ("o2", C.c_float), ("o3", C.c_float),
        ("nb", C.c_int), ("nt", C.c_int), ("dt", C.c_float),
        ("jdata", C.c_int), ("jsnap", C.c_int), ("bnds", C.c_int), ("fsrf", C.c_int), ("expl", C.c_int),
        ("refl", C.c_int),
    ]


GPU_KINDS = {"cart2d": 0, "cart3d": 1, "polar2d": 2, "spher3d": 3}

_libs: dict = {}


def lib(fp64: bool = False):
    name = "liboracle64.so" if fp64 else "liboracle.so"
    if name not in _libs:
        path = os.path.join(BUILD, name)
        if not os.path.exists(path):
            build(with_reference=False)
        L = C.CDLL(path)
        fp = C.POINTER(C.c_float)
        for fn in ("orc_cart2d_cpu", "orc_cart3d_cpu"):
            f = getattr(L, fn)
            f.argtypes = [C.POINTER(Par), fp, fp, fp, C.c_int, fp, C.c_int, fp, fp, fp]
            f.restype = C.c_int
        L.orc_cart_padded.argtypes = [C.POINTER(Par)] + [C.POINTER(C.c_int)] * 4
        L.orc_gpu_forward.argtypes = [C.c_int, C.POINTER(GPar), fp, fp, fp, C.c_int, fp, C.c_int, fp, fp, fp]
        L.orc_gpu_forward.restype = C.c_int
        L.orc_gpu_spher3d_fp64.argtypes = [C.POINTER(GPar), fp, fp, C.c_int, fp, C.c_int, fp,
                                           C.POINTER(C.c_double)]
        L.orc_gpu_spher3d_fp64.restype = C.c_int
        L.orc_cart3d_cpu_steps.argtypes = [C.c_int] * 6
        L.orc_cart3d_cpu_steps.restype = C.c_double
        _libs[name] = L
    return _libs[name]


def _fp(a):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_float))


def make_par(p: dict) -> Par:
    q = Par()
    q.n1, q.n2, q.n3 = p["n"][0], p["n"][1], (p["n"][2] if len(p["n"]) > 2 else 1)
    d = list(p["d"]) + [1.0] * (3 - len(p["d"]))
    o = list(p["o"]) + [0.0] * (3 - len(p["o"]))
    q.d1, q.d2, q.d3 = d
    q.o1, q.o2, q.o3 = o
    q.nb = p.get("nb", -1)
    q.nt = p["nt"]
    q.dt = p["dt"]
    q.fdorder = p.get("fdorder", 4)
    q.optfd = int(p.get("optfd", 0))
    q.dabc = int(p.get("dabc", 0))
    q.fsrf = int(p.get("fsrf", 0))
    q.hybrid = int(p.get("hybrid", 0))
    q.expl = int(p.get("expl", 0))
    q.jsnap = p.get("jsnap", 0)
    q.bnds = int(p.get("bnds", 0))
    q.nthreads = p.get("nthreads", 0)
    return q


def padded(p: dict):
    q = make_par(p)
    vals = [C.c_int() for _ in range(4)]
    lib().orc_cart_padded(C.byref(q), *[C.byref(v) for v in vals])
    return tuple(v.value for v in vals)


def snapshot_window(p: dict, nbd: int, npad):
    """The cpu programs' snapshot window as (count, first padded index,
    stride) per axis z, x, y.  Parameters nq*, oq*, dq* default to the model
    axes (MAWEFDcart2Dcpu.c:186-196, MAWEFDcart3Dcpu.c:180-195); first =
    floor((oq - opad) / d) with opad = o - nb*d, stride = floor(dq / d), all in
    float32 (fdutil.c:574-604 cut2d, :687-717 cut3d_slice, :292-293 and
    :348-350 for opad).  3D bnds=y: the padded counts and whole z-x planes, y
    planes still from oqy, dqy (MAWEFDcart3Dcpu.c:226-233, :341-353)."""
    ndim = len(p["n"])
    win = p.get("win", {})
    out = []
    f32 = np.float32
    for a, ax in enumerate("zxy"):
        if a >= ndim:
            out.append((1, 0, 0))
            continue
        n, o, d = p["n"][a], f32(p["o"][a]), f32(p["d"][a])
        nq = int(win.get("nq" + ax, n))
        oq, dq = f32(win.get("oq" + ax, o)), f32(win.get("dq" + ax, d))
        opad = f32(o - f32(nbd) * d)
        first, stride = int(np.floor(f32(f32(oq - opad) / d))), int(np.floor(f32(dq / d)))
        if p.get("bnds") and ndim == 3:
            nq = npad[a]
            if a < 2:
                first, stride = 0, 1
        if nq < 1 or first < 0 or stride < 0 or first + (nq - 1) * stride >= npad[a]:
            raise ValueError("snapshot window on %s leaves the padded grid" % ax)
        out.append((nq, first, stride))
    return out


def cut_window(frame, win, npad):
    """One padded frame [n3pad][n2pad][n1pad] cut to the window of
    snapshot_window, in the order the cpu programs write it (y planes, then
    x columns, z fastest)."""
    f = np.asarray(frame).reshape(npad[2], npad[1], npad[0])
    idx = [first + stride * np.arange(n) for n, first, stride in win]
    return f[np.ix_(idx[2], idx[1], idx[0])].ravel()


def cart_cpu(p: dict, vel, wav, sou, rec, den=None, fp64: bool = False):
    """Run the scheme of MAWEFDcart{2D,3D}cpu.c.  Arrays are C-order numpy
    float32 with axis 1 last (vel [n2][n1] or [n3][n2][n1]).  Returns
    (dat [nt][nr], snaps [nsnap][...] or None); with p["win"] (nq*, oq*, dq*)
    the frames are cut to that snapshot window as the programs write them."""
    q = make_par(p)
    ndim = 3 if q.n3 > 1 else 2
    nbd, n1p, n2p, n3p = padded(p)
    windowed = bool(p.get("win")) and q.jsnap > 0 and not (ndim == 2 and q.bnds)
    if windowed:
        q.bnds = 1  # padded frames, cut below
    vel = np.ascontiguousarray(vel, np.float32)
    den = None if den is None else np.ascontiguousarray(den, np.float32)
    wav = np.ascontiguousarray(wav, np.float32)
    sou = np.ascontiguousarray(sou, np.float32).reshape(-1, ndim)
    rec = np.ascontiguousarray(rec, np.float32).reshape(-1, ndim)
    ns, nr = sou.shape[0], rec.shape[0]
    dat = np.zeros((q.nt, nr), np.float32)
    snaps = None
    if q.jsnap > 0:
        nsnap = (q.nt - 1) // q.jsnap + 1
        frame = (n1p * n2p * n3p) if q.bnds else (q.n1 * q.n2 * q.n3)
        snaps = np.zeros((nsnap, frame), np.float32)
    fn = lib(fp64).orc_cart3d_cpu if ndim == 3 else lib(fp64).orc_cart2d_cpu
    rc = fn(C.byref(q), _fp(vel), _fp(den), _fp(wav), ns, _fp(sou), nr, _fp(rec), _fp(dat), _fp(snaps))
    if rc != 0:
        raise RuntimeError("oracle returned %d" % rc)
    if windowed:
        npad = (n1p, n2p, n3p)
        win = snapshot_window(p, nbd, npad)
        snaps = np.stack([cut_window(fr, win, npad) for fr in snaps])
    return dat, snaps


def cart3d_steps_seconds(n1pad, n2pad, n3pad, fdorder, nsteps, nthreads):
    return lib().orc_cart3d_cpu_steps(n1pad, n2pad, n3pad, fdorder, nsteps, nthreads)


def make_gpar(p: dict) -> GPar:
    q = GPar()
    n = list(p["n"]) + [1] * (3 - len(p["n"]))
    d = list(p["d"]) + [1.0] * (3 - len(p["d"]))
    o = list(p["o"]) + [0.0] * (3 - len(p["o"]))
    q.n1, q.n2, q.n3 = n
    q.d1, q.d2, q.d3 = d
    q.o1, q.o2, q.o3 = o
    q.nb, q.nt, q.dt = p.get("nb", 4), p["nt"], p["dt"]
    q.jdata, q.jsnap, q.bnds = p.get("jdata", 1), p.get("jsnap", 0), int(p.get("bnds", 0))
    q.fsrf, q.expl, q.refl = int(p.get("fsrf", 0)), int(p.get("expl", 0)), int(p.get("refl", 0))
    return q


def gpu_shapes(kind: str, p: dict, nr: int):
    """(data rows, snapshot frames, floats per frame) of a GPU-program run."""
    n = list(p["n"]) + [1] * (3 - len(p["n"]))
    nb = max(p.get("nb", 4), 4)
    nt, jdata, jsnap = p["nt"], max(p.get("jdata", 1), 1), p.get("jsnap", 0)
    rows = nt if kind == "spher3d" else nt // jdata
    frames = (nt - 1) // jsnap + 1 if jsnap > 0 else 0
    nd = 3 if kind in ("cart3d", "spher3d") else 2
    if p.get("bnds", 0):
        elems = int(np.prod([n[a] + 2 * nb for a in range(nd)]))
    else:
        elems = int(np.prod(n[:nd]))
    return rows, frames, elems


def gpu_scheme(kind: str, p: dict, vel, wav, sou, rec, rfl=None, use_reference_emulation: bool = False):
    """Run the GPU-program scheme.  use_reference_emulation=True runs the
    reference's own kernel files through the host emulation
    (oracle/_ref/libgpuref.so, built only where the reference is present);
    otherwise the oracle restatement.  Returns (dat, snaps)."""
    nd = 3 if kind in ("cart3d", "spher3d") else 2
    q = make_gpar(p)
    vel = np.ascontiguousarray(vel, np.float32)
    rfl = None if rfl is None else np.ascontiguousarray(rfl, np.float32)
    wav = np.ascontiguousarray(wav, np.float32).ravel()
    sou = np.ascontiguousarray(sou, np.float32).reshape(-1, nd)
    rec = np.ascontiguousarray(rec, np.float32).reshape(-1, nd)
    rows, frames, elems = gpu_shapes(kind, p, rec.shape[0])
    dat = np.zeros((rows, rec.shape[0]), np.float32)
    snaps = np.zeros((frames, elems), np.float32) if frames else None
    args = (C.byref(q),)
    if use_reference_emulation:
        L = C.CDLL(os.path.join(REF_OUT, "libgpuref.so"))
        fp = C.POINTER(C.c_float)
        fn = getattr(L, "gpuref_" + kind)
        if kind == "cart2d":
            fn.argtypes = [C.POINTER(GPar), fp, fp, fp, C.c_int, fp, C.c_int, fp, fp, fp]
            rc = fn(C.byref(q), _fp(vel), _fp(rfl), _fp(wav), sou.shape[0], _fp(sou), rec.shape[0], _fp(rec),
                    _fp(dat), _fp(snaps))
        else:
            fn.argtypes = [C.POINTER(GPar), fp, fp, C.c_int, fp, C.c_int, fp, fp, fp]
            rc = fn(C.byref(q), _fp(vel), _fp(wav), sou.shape[0], _fp(sou), rec.shape[0], _fp(rec), _fp(dat),
                    _fp(snaps))
    else:
        rc = lib().orc_gpu_forward(GPU_KINDS[kind], *args, _fp(vel), _fp(rfl), _fp(wav), sou.shape[0], _fp(sou),
                                   rec.shape[0], _fp(rec), _fp(dat), _fp(snaps))
    if rc != 0:
        raise RuntimeError("GPU-scheme run returned %d" % rc)
    return dat, snaps


def gpu_cart2d_moving(p: dict, vel, wav, sou, nst: int, rec, nrt: int, move: int,
                      use_reference_emulation: bool = False):
    """sfAWEFDcart2Dgpu's scheme with moving sources and receivers: sou holds
    ns*nst (x, z) points and rec nr*nrt; move 0 = row min(it, rows-1) per
    step, 1 = sfDYNAWEFDcart2Dgpu (entry k*(it+1), free surface only with
    fsrf).  use_reference_emulation=True runs MDYNAWEFDcart2Dgpu's own
    kernels through the host emulation (move 1 only).  Returns (dat, snaps)."""
    q = make_gpar(p)
    vel = np.ascontiguousarray(vel, np.float32)
    wav = np.ascontiguousarray(wav, np.float32).ravel()
    sou = np.ascontiguousarray(sou, np.float32).reshape(-1, 2)
    rec = np.ascontiguousarray(rec, np.float32).reshape(-1, 2)
    ns, nr = sou.shape[0] // nst, rec.shape[0] // nrt
    assert ns * nst == sou.shape[0] and nr * nrt == rec.shape[0]
    rows, frames, elems = gpu_shapes("cart2d", p, nr)
    dat = np.zeros((rows, nr), np.float32)
    snaps = np.zeros((frames, elems), np.float32) if frames else None
    if use_reference_emulation:
        if move != 1:
            raise ValueError("the reference emulation covers sfDYNAWEFDcart2Dgpu (move=1) only")
        L = C.CDLL(os.path.join(REF_OUT, "libgpuref.so"))
        fp = C.POINTER(C.c_float)
        fn = L.gpuref_dyncart2d
        fn.argtypes = [C.POINTER(GPar), fp, fp, C.c_int, C.c_int, fp, C.c_int, C.c_int, fp, fp, fp]
        rc = fn(C.byref(q), _fp(vel), _fp(wav), ns, nst, _fp(sou), nr, nrt, _fp(rec), _fp(dat), _fp(snaps))
    else:
        rc = lib().orc_gpu_cart2d_moving(C.byref(q), _fp(vel), _fp(wav), ns, nst, _fp(sou), nr, nrt, _fp(rec), move,
                                         _fp(dat), _fp(snaps))
    if rc != 0:
        raise RuntimeError("moving-geometry run returned %d" % rc)
    return dat, snaps


def cloud_window(ground, orbit, apt: float, data=None):
    """Mbycloudwin3d (fast=y): ground [ng][9], orbit [no][9], aperture in
    degrees, data [nf][ng] complex64 or float32 (optional).  Returns (index,
    window points [nw][9], window data [nf][nw] or None)."""
    g = np.ascontiguousarray(ground, np.float32).reshape(-1, 9)
    o = np.ascontiguousarray(orbit, np.float32).reshape(-1, 9)
    ng = g.shape[0]
    nf, ncomp, dflat = 0, 2, None
    if data is not None:
        ncomp = 2 if np.iscomplexobj(data) else 1
        d = np.ascontiguousarray(data, np.complex64 if ncomp == 2 else np.float32)
        nf = d.shape[0]
        dflat = d.view(np.float32).reshape(-1)
    index = np.zeros(max(ng, 1), np.int64)
    win = np.zeros((max(ng, 1), 9), np.float32)
    wd = np.zeros(max(nf * ng * ncomp, 1), np.float32)
    nw = C.c_longlong()
    L = lib()
    lp = C.POINTER(C.c_longlong)
    rc = L.orc_cloud_window(_fp(g), C.c_longlong(ng), _fp(o), C.c_longlong(o.shape[0]), C.c_float(apt),
                            C.c_longlong(nf), ncomp, _fp(dflat), C.byref(nw), index.ctypes.data_as(lp), _fp(win),
                            _fp(wd))
    if rc != 0:
        raise RuntimeError("orc_cloud_window returned %d" % rc)
    n = nw.value
    wdat = None
    if data is not None:
        wdat = wd[: nf * n * ncomp].view(np.complex64 if ncomp == 2 else np.float32).reshape(nf, n)
    return index[:n].copy(), win[:n].copy(), wdat


def cloud_merge(all_pts, windows, norm: bool = True, hashscale: float = 2.0):
    """Mbycloudmerge3d: all_pts [na][9]; windows: list of (points [nw][9],
    data [nf][nw]) with one dtype (complex64 or float32).  Returns [nf][na]."""
    a = np.ascontiguousarray(all_pts, np.float32).reshape(-1, 9)
    na = a.shape[0]
    ncomp = 2 if np.iscomplexobj(windows[0][1]) else 1
    dt = np.complex64 if ncomp == 2 else np.float32
    nf = windows[0][1].shape[0]
    nwp = np.array([w[0].reshape(-1, 9).shape[0] for w in windows], np.int64)
    pts = np.ascontiguousarray(np.concatenate([np.asarray(w[0], np.float32).reshape(-1, 9) for w in windows]))
    dat = np.ascontiguousarray(np.concatenate([np.asarray(w[1], dt).reshape(-1) for w in windows])).view(np.float32)
    out = np.zeros(nf * na * ncomp, np.float32)
    lp = C.POINTER(C.c_longlong)
    rc = lib().orc_cloud_merge(_fp(a), C.c_longlong(na), len(windows), nwp.ctypes.data_as(lp), _fp(pts), _fp(dat),
                               C.c_longlong(nf), ncomp, int(norm), C.c_float(hashscale), _fp(out))
    if rc != 0:
        raise RuntimeError("orc_cloud_merge returned %d" % rc)
    return out.view(dt).reshape(nf, na)


_adj = None


def _adj_lib():
    global _adj
    if _adj is None:
        path = os.path.join(BUILD, "liboracle_adj.so")
        if not os.path.exists(path):
            build(with_reference=False)
        L = C.CDLL(path)
        fp = C.POINTER(C.c_float)
        dp = C.POINTER(C.c_double)
        L.orc_grad.argtypes = [C.POINTER(Par), C.c_int, C.c_int, fp, fp, C.c_int, fp, C.c_int, fp, fp, dp, dp, dp]
        L.orc_grad.restype = C.c_int
        L.orc_grad_m.argtypes = [C.POINTER(Par), C.c_int, C.c_int, dp, fp, C.c_int, fp, C.c_int, fp, fp, dp, dp, dp]
        L.orc_grad_m.restype = C.c_int
        L.orc_grad_ckpt.argtypes = [C.POINTER(Par), C.c_int, C.c_int, fp, fp, C.c_int, fp, C.c_int, fp, fp, C.c_int,
                                    C.c_int, dp, dp, dp]
        L.orc_grad_ckpt.restype = C.c_int
        L.orc_image.argtypes = [C.POINTER(Par), C.c_int, C.c_int, fp, fp, C.c_int, fp, C.c_int, fp, fp, C.c_int, dp]
        L.orc_image.restype = C.c_int
        L.orc_gpu_spher3d_grad.argtypes = [C.POINTER(GPar), fp, dp, fp, C.c_int, fp, C.c_int, fp, fp, C.c_int,
                                           C.c_int, dp, dp, dp]
        L.orc_gpu_spher3d_grad.restype = C.c_int
        L.orc_gpu_spher3d_image.argtypes = [C.POINTER(GPar), fp, fp, C.c_int, fp, C.c_int, fp, fp, C.c_int, dp]
        L.orc_gpu_spher3d_image.restype = C.c_int
        _adj = L
    return _adj


def misfit_gradient(p: dict, vel, wav, sou, rec, dobs, jdata: int = 1, m=None, ckpt_every: int = 0,
                    ckpt_bits: int = 0):
    """FP64 misfit J = 0.5 sum (d - dobs)^2 of the CPU-program scheme and its
    gradient with respect to m = 1/v^2 (boundary coefficients held fixed).
    The model is `vel` (float32 velocity, v^2 dt^2 formed in float as the
    engine does) or, when `m` is given, slowness squared in float64 (for
    finite differences free of float rounding; `vel` then only sets the shape).
    ckpt_bits > 0 emulates checkpointed recompute from levels rounded to that
    many significant bits every ckpt_every steps (8 = BF16); ckpt_bits = -1
    emulates the block floating point checkpoints (AWE_CKPT_BFP16).
    Returns (grad [model shape] float64, J, dsyn [nsmp][nr] float64)."""
    q = make_par(p)
    ndim = len(p["n"])
    vel = np.ascontiguousarray(vel, np.float32)
    wav = np.ascontiguousarray(wav, np.float32)
    sou = np.ascontiguousarray(sou, np.float32).reshape(-1, ndim)
    rec = np.ascontiguousarray(rec, np.float32).reshape(-1, ndim)
    ns, nr = sou.shape[0], rec.shape[0]
    nsmp = (q.nt - 1) // jdata + 1
    dobs = np.ascontiguousarray(dobs, np.float32).reshape(nsmp, nr)
    grad = np.zeros(vel.shape, np.float64)
    dsyn = np.zeros((nsmp, nr), np.float64)
    J = C.c_double()
    dp = C.POINTER(C.c_double)
    if ckpt_bits:
        rc = _adj_lib().orc_grad_ckpt(C.byref(q), ndim, jdata, _fp(vel), _fp(wav), ns, _fp(sou), nr, _fp(rec),
                                      _fp(dobs), ckpt_every, ckpt_bits, grad.ctypes.data_as(dp), C.byref(J),
                                      dsyn.ctypes.data_as(dp))
    elif m is None:
        rc = _adj_lib().orc_grad(C.byref(q), ndim, jdata, _fp(vel), _fp(wav), ns, _fp(sou), nr, _fp(rec), _fp(dobs),
                                 grad.ctypes.data_as(dp), C.byref(J), dsyn.ctypes.data_as(dp))
    else:
        m = np.ascontiguousarray(m, np.float64).reshape(vel.shape)
        rc = _adj_lib().orc_grad_m(C.byref(q), ndim, jdata, m.ctypes.data_as(dp), _fp(wav), ns, _fp(sou), nr,
                                   _fp(rec), _fp(dobs), grad.ctypes.data_as(dp), C.byref(J), dsyn.ctypes.data_as(dp))
    if rc != 0:
        raise ValueError("orc_grad rejected the parameters")
    return grad, J.value, dsyn


def rtm_image(p: dict, vel, wav, sou, rec, data, condition: int, jdata: int = 1):
    """FP64 reverse-time migration image of the CPU-program scheme on the
    exact adjoint driven by `data` [nsmp][nr]: condition 0 = zero-lag
    cross-correlation of the adjoint and forward wavefields (model window),
    1 = the Born adjoint (the gradient formula with the data as residual).
    Returns the image (model shape, float64)."""
    q = make_par(p)
    ndim = len(p["n"])
    vel = np.ascontiguousarray(vel, np.float32)
    wav = np.ascontiguousarray(wav, np.float32)
    sou = np.ascontiguousarray(sou, np.float32).reshape(-1, ndim)
    rec = np.ascontiguousarray(rec, np.float32).reshape(-1, ndim)
    nsmp = (q.nt - 1) // jdata + 1
    data = np.ascontiguousarray(data, np.float32).reshape(nsmp, rec.shape[0])
    img = np.zeros(vel.shape, np.float64)
    rc = _adj_lib().orc_image(C.byref(q), ndim, jdata, _fp(vel), _fp(wav), sou.shape[0], _fp(sou), rec.shape[0],
                              _fp(rec), _fp(data), condition, img.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise ValueError("orc_image rejected the parameters")
    return img


def _gpar_spher(p: dict) -> GPar:
    q = GPar()
    q.n1, q.n2, q.n3 = p["n"]
    q.d1, q.d2, q.d3 = p["d"]
    q.o1, q.o2, q.o3 = p["o"]
    q.nb, q.nt, q.dt = p["nb"], p["nt"], p["dt"]
    q.jdata, q.jsnap, q.bnds = 1, 0, 0
    q.fsrf, q.expl, q.refl = int(p.get("fsrf", 0)), int(p.get("expl", 0)), 0
    return q


def spher3d_gradient(p: dict, vel, wav, sou, rec, dobs, m=None, ckpt_every: int = 0, ckpt_bits: int = 0):
    """FP64 misfit J = 0.5 sum (d - dobs)^2 of the spherical GPU-program
    scheme and its gradient with respect to m = 1/v^2 (the discrete adjoint
    of that scheme, awe_adjoint_sph.c).  The model is `vel` (float32) or,
    when `m` is given, slowness squared in float64.  ckpt_bits != 0 emulates
    checkpointed recompute every ckpt_every steps from levels rounded as the
    engine's checkpoint format (8 BF16, 11 FP16, -1 block floating point).
    Returns (grad [nph][nth][nr] float64, J, dsyn [nt][nrec] float64)."""
    q = _gpar_spher(p)
    vel = np.ascontiguousarray(vel, np.float32)
    wav = np.ascontiguousarray(wav, np.float32)
    sou = np.ascontiguousarray(sou, np.float32).reshape(-1, 3)
    rec = np.ascontiguousarray(rec, np.float32).reshape(-1, 3)
    nr = rec.shape[0]
    dobs = np.ascontiguousarray(dobs, np.float32).reshape(q.nt, nr)
    grad = np.zeros(vel.shape, np.float64)
    dsyn = np.zeros((q.nt, nr), np.float64)
    J = C.c_double()
    dp = C.POINTER(C.c_double)
    mp = None
    if m is not None:
        m = np.ascontiguousarray(m, np.float64).reshape(vel.shape)
        mp = m.ctypes.data_as(dp)
    rc = _adj_lib().orc_gpu_spher3d_grad(C.byref(q), _fp(vel), mp, _fp(wav), sou.shape[0], _fp(sou), nr, _fp(rec),
                                         _fp(dobs), ckpt_every, ckpt_bits, grad.ctypes.data_as(dp), C.byref(J),
                                         dsyn.ctypes.data_as(dp))
    if rc != 0:
        raise ValueError("orc_gpu_spher3d_grad rejected the parameters")
    return grad, J.value, dsyn


def spher3d_image(p: dict, vel, wav, sou, rec, data, condition: int):
    """FP64 images of the spherical GPU-program scheme on its exact adjoint
    driven by `data` [nt][nrec]: condition 0 = zero-lag cross-correlation
    (model window), 1 = Born adjoint.  Returns [nph][nth][nr] float64."""
    q = _gpar_spher(p)
    vel = np.ascontiguousarray(vel, np.float32)
    wav = np.ascontiguousarray(wav, np.float32)
    sou = np.ascontiguousarray(sou, np.float32).reshape(-1, 3)
    rec = np.ascontiguousarray(rec, np.float32).reshape(-1, 3)
    data = np.ascontiguousarray(data, np.float32).reshape(q.nt, rec.shape[0])
    img = np.zeros(vel.shape, np.float64)
    rc = _adj_lib().orc_gpu_spher3d_image(C.byref(q), _fp(vel), _fp(wav), sou.shape[0], _fp(sou), rec.shape[0],
                                          _fp(rec), _fp(data), condition, img.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise ValueError("orc_gpu_spher3d_image rejected the parameters")
    return img


def spher3d_adj_frames(nt: int, kt: int, jsnap: int) -> int:
    """Frames sfAWEFDspher3Dgpu adj=y snap=y writes: steps it <= nt-kt with
    it % jsnap == 0, and step nt-kt."""
    last = nt - kt
    return last // jsnap + 1 + (1 if last % jsnap else 0)


def spher3d_adj(p: dict, vel, data, rec, kt: int, use_reference_emulation: bool = False):
    """sfAWEFDspher3Dgpu adj=y: data [nt][nr] back-injected (reversed in time,
    unscaled) at the receivers rec [nr][3]; stops after step nt-kt.  p as for
    gpu_scheme (jsnap > 0 with snap frames, bnds).  Returns (image
    [nph][nth][nra], frames [nframes][...] or None).  use_reference_emulation
    runs the reference's own kernels (oracle/_ref/libgpuref.so)."""
    q = make_gpar(p)
    vel = np.ascontiguousarray(vel, np.float32)
    rec = np.ascontiguousarray(rec, np.float32).reshape(-1, 3)
    nr = rec.shape[0]
    data = np.ascontiguousarray(data, np.float32).reshape(q.nt, nr)
    image = np.zeros(vel.shape, np.float32)
    snaps = None
    if q.jsnap > 0:
        _, _, elems = gpu_shapes("spher3d", p, nr)
        snaps = np.zeros((spher3d_adj_frames(q.nt, kt, q.jsnap), elems), np.float32)
    if use_reference_emulation:
        L = C.CDLL(os.path.join(REF_OUT, "libgpuref.so"))
        fp = C.POINTER(C.c_float)
        fn = L.gpuref_spher3d_adj
        fn.argtypes = [C.POINTER(GPar), fp, fp, C.c_int, fp, C.c_int, fp, fp]
        fn.restype = C.c_int
    else:
        fn = lib().orc_gpu_spher3d_adj
        fn.argtypes = [C.POINTER(GPar), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float),
                       C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        fn.restype = C.c_int
    n = fn(C.byref(q), _fp(vel), _fp(data), nr, _fp(rec), kt, _fp(image), _fp(snaps))
    if n < 0:
        raise ValueError("kt must be in [1, nt]")
    if snaps is not None and n != snaps.shape[0]:
        raise RuntimeError("adjoint run wrote %d frames, expected %d" % (n, snaps.shape[0]))
    return image, snaps


def spher3d_fp64(p: dict, vel, wav, sou, rec):
    """Traces [nt][nr] (float64) of the spherical GPU-program scheme with FP64
    wavefields; p as for gpu_scheme."""
    q = GPar()
    q.n1, q.n2, q.n3 = p["n"]
    q.d1, q.d2, q.d3 = p["d"]
    q.o1, q.o2, q.o3 = p["o"]
    q.nb, q.nt, q.dt = p["nb"], p["nt"], p["dt"]
    q.jdata, q.jsnap, q.bnds = 1, 0, 0
    q.fsrf, q.expl, q.refl = int(p.get("fsrf", 0)), int(p.get("expl", 0)), 0
    vel = np.ascontiguousarray(vel, np.float32)
    wav = np.ascontiguousarray(wav, np.float32)
    sou = np.ascontiguousarray(sou, np.float32).reshape(-1, 3)
    rec = np.ascontiguousarray(rec, np.float32).reshape(-1, 3)
    dat = np.zeros((q.nt, rec.shape[0]), np.float64)
    rc = lib().orc_gpu_spher3d_fp64(C.byref(q), _fp(vel), _fp(wav), sou.shape[0], _fp(sou), rec.shape[0], _fp(rec),
                                    dat.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise ValueError("orc_gpu_spher3d_fp64 failed")
    return dat

