"""CUDA path vs the scheme of the reference's GPU programs
(sfAWEFD{cart,spher}{2D,3D}gpu).  The golden fixtures come from the
reference's own CUDA kernel files run through the host emulation of each
program's time loop (tests/golden/make_golden_gpu.py).  EXACT precision must
match bit for bit, FAST within rel-L2 <= 1e-5."""
import numpy as np
import pytest

from helpers import golden_paths, load_golden, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5
GOLDEN_A = golden_paths("A_*.npz")
KIND = {"cart2d": (0, 2), "cart3d": (0, 3), "polar2d": (1, 2), "spher3d": (1, 3)}


def run_gpu_scheme(par, a, precision):
    import wavefield_imaging_gb300 as awe

    coords, nd = KIND[par["kind"]]
    desc = awe.make_desc(nd, par["n"], par["d"], par["o"], par["nt"], par["dt"], coords=coords,
                         scheme=awe.SCHEME_GPU, nb=par["nb"], jdata=par.get("jdata", 1), jsnap=par.get("jsnap", 0),
                         bnds=par.get("bnds", 0), fsrf=par.get("fsrf", 0), expl=par.get("expl", 0),
                         refl=par.get("refl", 0), precision=precision)
    with awe.Plan(desc) as p:
        p.set_model(a["vel"], rfl=a.get("rfl"))
        p.set_geometry(a["sou"], a["rec"])
        if par.get("jsnap", 0) > 0:
            return p.forward(a["wav"], snapshots=True)
        return p.forward(a["wav"]), None


@pytest.mark.parametrize("path", GOLDEN_A, ids=[p.split("/")[-1][:-4] for p in GOLDEN_A])
def test_exact_mode_bit_exact_vs_reference_kernels(path):
    par, a = load_golden(path)
    dat, snaps = run_gpu_scheme(par, a, precision=1)
    np.testing.assert_array_equal(dat, a["dat"])
    if "snaps" in a:
        np.testing.assert_array_equal(snaps, a["snaps"])


@pytest.mark.parametrize("path", GOLDEN_A, ids=[p.split("/")[-1][:-4] for p in GOLDEN_A])
def test_fast_mode_within_tolerance(path):
    par, a = load_golden(path)
    dat, snaps = run_gpu_scheme(par, a, precision=0)
    assert rel_l2(dat, a["dat"]) <= TOL
    if "snaps" in a:
        assert rel_l2(snaps, a["snaps"]) <= TOL


def test_larger_spherical_case_vs_oracle():
    """A bigger spherical shell than the fixtures (free surface, two sources),
    EXACT against the oracle restatement."""
    from oracle import oracle
    import wavefield_imaging_gb300 as awe

    rng = np.random.default_rng(41)
    n = (60, 40, 36)
    d = (0.005, 1.5e-6, 1.5e-6)
    o = (3387.0, np.pi / 2 - 20 * 1.5e-6, -18 * 1.5e-6)
    vel = (0.168 + 0.01 * rng.random((n[2], n[1], n[0]))).astype(np.float32)
    vel[:, :, 45:] = 0.3
    nt = 160
    t = np.arange(nt) * 0.005 - 0.3
    wav = ((1 - 2 * (np.pi * 5 * t) ** 2) * np.exp(-(np.pi * 5 * t) ** 2)).astype(np.float32)
    sou = np.array([[o[0] + 40 * d[0], o[2] + 15 * d[2], o[1] + 20 * d[1]],
                    [o[0] + 38 * d[0], o[2] + 20 * d[2], o[1] + 17 * d[1]]], np.float32)
    rec = np.array([[o[0] + 42 * d[0], o[2] + k * d[2], o[1] + 19 * d[1]] for k in range(4, 32, 3)], np.float32)
    par = dict(kind="spher3d", n=list(n), d=list(d), o=list(o), nb=6, nt=nt, dt=0.005, jsnap=0, fsrf=1)
    ref, _ = oracle.gpu_scheme("spher3d", par, vel, wav, sou, rec)
    desc = awe.make_desc(3, n, d, o, nt, 0.005, coords=awe.SPHER, scheme=awe.SCHEME_GPU, nb=6, fsrf=1,
                         precision=awe.EXACT)
    with awe.Plan(desc) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        dat = p.forward(wav)
    np.testing.assert_array_equal(dat, ref)


def test_spherical_shots_advance_together_as_separate_runs():
    """awe_set_shots: three shots on one spherical grid in one step launch give
    exactly the traces of three single-shot runs."""
    import wavefield_imaging_gb300 as awe

    rng = np.random.default_rng(43)
    n = (40, 30, 28)
    d = (0.005, 1.5e-6, 1.5e-6)
    o = (3387.0, np.pi / 2 - 15 * 1.5e-6, -14 * 1.5e-6)
    vel = (0.168 + 0.01 * rng.random((n[2], n[1], n[0]))).astype(np.float32)
    nt = 120
    t = np.arange(nt) * 0.005 - 0.3
    wav = ((1 - 2 * (np.pi * 5 * t) ** 2) * np.exp(-(np.pi * 5 * t) ** 2)).astype(np.float32)
    shots = []
    for k in range(3):
        sou = np.array([[o[0] + 25 * d[0], o[2] + (10 + 4 * k) * d[2], o[1] + 15 * d[1]]], np.float32)
        rec = np.array([[o[0] + 28 * d[0], o[2] + j * d[2], o[1] + (12 + k) * d[1]] for j in range(4, 24, 4)],
                       np.float32)
        shots.append((sou, rec))
    desc = awe.make_desc(3, n, d, o, nt, 0.005, coords=awe.SPHER, scheme=awe.SCHEME_GPU, nb=6, precision=awe.FAST)
    with awe.Plan(desc) as p:
        p.set_model(vel)
        p.set_shots(shots)
        together = p.forward(wav)
    off = 0
    for sou, rec in shots:
        with awe.Plan(desc) as p:
            p.set_model(vel)
            p.set_geometry(sou, rec)
            single = p.forward(wav)
        np.testing.assert_array_equal(together[:, off:off + rec.shape[0]], single)
        off += rec.shape[0]
