"""Pins the oracle (oracle/awe_oracle.c) to the reference itself: the golden
fixtures were produced by the reference's own CPU programs
(MAWEFDcart{2D,3D}cpu.c built from source, tests/golden/make_golden.py); the
oracle must reproduce them bit for bit."""
import glob
import json
import os

import numpy as np
import pytest

from oracle import oracle

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "c*.npz")))


def load(path):
    z = np.load(path)
    par = json.loads(str(z["par"]))
    return par, {k: z[k] for k in z.files if k != "par"}


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_bit_exact(path):
    par, a = load(path)
    dat, snaps = oracle.cart_cpu(par, a["vel"], a["wav"], a["sou"], a["rec"], den=a.get("den"))
    assert dat.shape == a["dat"].shape
    assert np.array_equal(dat, a["dat"])
    if "snaps" in a:
        assert np.array_equal(snaps.ravel(), a["snaps"])


def test_golden_set_covers_options():
    names = [os.path.basename(p) for p in GOLDEN]
    assert len(names) >= 10
    pars = [load(p)[0] for p in GOLDEN]
    assert {len(p["n"]) for p in pars} == {2, 3}
    assert {p["fdorder"] for p in pars} >= {2, 4, 6, 8}
    assert any(p["hybrid"] for p in pars) and any(p["fsrf"] for p in pars) and any(p["bnds"] for p in pars)


def test_fp64_oracle_close_to_fp32():
    par, a = load(GOLDEN[0])
    d32, _ = oracle.cart_cpu(par, a["vel"], a["wav"], a["sou"], a["rec"], den=a.get("den"))
    d64, _ = oracle.cart_cpu(par, a["vel"], a["wav"], a["sou"], a["rec"], den=a.get("den"), fp64=True)
    rel = np.linalg.norm(d32 - d64) / np.linalg.norm(d64)
    assert 0 < rel < 1e-4


GOLDEN_A = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "A_*.npz")))


@pytest.mark.parametrize("path", GOLDEN_A, ids=[os.path.basename(p)[:-4] for p in GOLDEN_A])
def test_gpu_scheme_oracle_matches_reference_kernels_bit_exact(path):
    """Fixtures from the reference's own CUDA kernel files run through the host
    emulation of the GPU programs (tests/golden/make_golden_gpu.py)."""
    par, a = load(path)
    if par["kind"] == "dyncart2d":  # sfDYNAWEFDcart2Dgpu: moving-geometry tables
        dat, snaps = oracle.gpu_cart2d_moving(par, a["vel"], a["wav"], a["sou"], par["nst"], a["rec"], par["nrt"], 1)
    else:
        dat, snaps = oracle.gpu_scheme(par["kind"], par, a["vel"], a["wav"], a["sou"], a["rec"], rfl=a.get("rfl"))
    assert np.array_equal(dat, a["dat"])
    if "snaps" in a:
        assert np.array_equal(snaps, a["snaps"])


GOLDEN_ADJ = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "Aadj_*.npz")))


@pytest.mark.parametrize("path", GOLDEN_ADJ, ids=[os.path.basename(p)[:-4] for p in GOLDEN_ADJ])
def test_spherical_adjoint_oracle_matches_reference_kernels_bit_exact(path):
    """sfAWEFDspher3Dgpu adj=y: the traces back-injected at the receivers, the
    image after step nt-kt and the frames, against the reference's kernels
    run through the host emulation of the program's adj branch."""
    par, a = load(path)
    image, snaps = oracle.spher3d_adj(par, a["vel"], a["data"], a["rec"], par["kt"])
    assert np.abs(a["image"]).max() > 0
    assert np.array_equal(image, a["image"])
    if "snaps" in a:
        assert np.array_equal(snaps, a["snaps"])
    else:
        assert snaps is None


def test_gpu_scheme_golden_set_covers_programs():
    kinds = {load(p)[0]["kind"] for p in GOLDEN_A}
    assert kinds == {"cart2d", "cart3d", "polar2d", "spher3d", "dyncart2d"}


def test_moving_geometry_oracle_modes():
    """The per-step mode with every row equal is the fixed geometry, and the
    sfDYNAWEFDcart2Dgpu mode with one point (entry 0 at every step) too,
    except for its free surface, which needs free=y."""
    par, a = load(os.path.join(os.path.dirname(__file__), "golden", "A_cart2d_const.npz"))
    ref, rsn = oracle.gpu_scheme("cart2d", par, a["vel"], a["wav"], a["sou"], a["rec"])
    sou_t = np.tile(a["sou"], (7, 1))
    rec_t = np.tile(a["rec"], (7, 1))
    dat, snaps = oracle.gpu_cart2d_moving(par, a["vel"], a["wav"], sou_t, 7, rec_t, 7, 0)
    assert np.array_equal(dat, ref) and np.array_equal(snaps, rsn)
    one = dict(par, fsrf=1)
    d1, _ = oracle.gpu_cart2d_moving(one, a["vel"], a["wav"], a["sou"][:1], 1, a["rec"][:1], 1, 1)
    r1, _ = oracle.gpu_scheme("cart2d", par, a["vel"], a["wav"], a["sou"][:1], a["rec"][:1])
    assert np.array_equal(d1, r1)
    d0, _ = oracle.gpu_cart2d_moving(par, a["vel"], a["wav"], a["sou"][:1], 1, a["rec"][:1], 1, 1)
    assert not np.array_equal(d0, r1)


def test_snapshot_window_rule():
    """The cpu programs' window rule restated in the oracle: first padded index
    floor((oq - opad)/d), stride floor(dq/d), float32 arithmetic; defaults the
    model window; 3D bnds=y takes the padded counts and whole z-x planes; a
    window leaving the padded grid is an error."""
    p = dict(n=[48, 64], d=[5.0, 5.0], o=[0.0, 0.0], nb=12, jsnap=10)
    npad = (72, 88, 1)
    assert oracle.snapshot_window(p, 12, npad) == [(48, 12, 1), (64, 12, 1), (1, 0, 0)]
    p["win"] = dict(nqz=20, oqz=-20.0, dqz=10.0, nqx=15, oqx=32.5, dqx=15.0)
    assert oracle.snapshot_window(p, 12, npad) == [(20, 8, 2), (15, 18, 3), (1, 0, 0)]
    p["win"] = dict(oqz=-61.0)
    with pytest.raises(ValueError):
        oracle.snapshot_window(p, 12, npad)
    p3 = dict(n=[24, 20, 18], d=[5.0] * 3, o=[0.0] * 3, nb=8, jsnap=10, bnds=1, win=dict(oqy=-40.0))
    assert oracle.snapshot_window(p3, 8, (40, 36, 34)) == [(40, 0, 1), (36, 0, 1), (34, 0, 1)]
    p3["win"] = {}  # the reference's default oqy = oy starts at plane nb: outside the grid
    with pytest.raises(ValueError):
        oracle.snapshot_window(p3, 8, (40, 36, 34))
    frame = np.arange(72 * 88, dtype=np.float32)
    cut = oracle.cut_window(frame, [(2, 8, 2), (3, 18, 3), (1, 0, 0)], npad)
    assert cut.tolist() == [18 * 72 + 8, 18 * 72 + 10, 21 * 72 + 8, 21 * 72 + 10, 24 * 72 + 8, 24 * 72 + 10]
