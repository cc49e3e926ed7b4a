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
    dat, snaps = oracle.gpu_scheme(par["kind"], par, a["vel"], a["wav"], a["sou"], a["rec"], rfl=a.get("rfl"))
    assert np.array_equal(dat, a["dat"])
    if "snaps" in a:
        assert np.array_equal(snaps, a["snaps"])


def test_gpu_scheme_golden_set_covers_programs():
    kinds = {load(p)[0]["kind"] for p in GOLDEN_A}
    assert kinds == {"cart2d", "cart3d", "polar2d", "spher3d"}
