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
KIND = {"cart2d": (0, 2), "cart3d": (0, 3), "polar2d": (1, 2), "spher3d": (1, 3), "dyncart2d": (0, 2)}


def run_gpu_scheme(par, a, precision):
    import wavefield_imaging_gb300 as awe

    coords, nd = KIND[par["kind"]]
    desc = awe.make_desc(nd, par["n"], par["d"], par["o"], par["nt"], par["dt"], coords=coords,
                         scheme=awe.SCHEME_GPU, nb=par["nb"], jdata=par.get("jdata", 1), jsnap=par.get("jsnap", 0),
                         bnds=par.get("bnds", 0), fsrf=par.get("fsrf", 0), expl=par.get("expl", 0),
                         refl=par.get("refl", 0), precision=precision)
    with awe.Plan(desc) as p:
        p.set_model(a["vel"], rfl=a.get("rfl"))
        if par["kind"] == "dyncart2d":  # sfDYNAWEFDcart2Dgpu's moving tables
            p.set_moving_geometry(a["sou"], par["nst"], a["rec"], par["nrt"], awe.MOVE_DYN)
        else:
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


def _moving_case(seed, nt, rows):
    rng = np.random.default_rng(seed)
    n = (44, 52)
    vel = np.full((n[1], n[0]), 168.0, np.float32)
    vel[:, 30:] = 110.0
    vel *= (1 + 0.02 * rng.random(vel.shape)).astype(np.float32)
    t = np.arange(nt) * 0.005 - 0.3
    wav = ((1 - 2 * (np.pi * 5 * t) ** 2) * np.exp(-(np.pi * 5 * t) ** 2)).astype(np.float32)
    e = np.arange(rows)
    sou = np.stack([60 + 0.8 * e[:, None] + 30 * np.arange(2)[None, :],
                    np.full((rows, 2), 90.0)], -1).reshape(-1, 2).astype(np.float32)
    rec = np.stack([10 + 0.7 * e[:, None] + 35 * np.arange(4)[None, :],
                    np.full((rows, 4), 60.5)], -1).reshape(-1, 2).astype(np.float32)
    par = dict(kind="cart2d", n=list(n), d=[5.0, 5.0], o=[0.0, 0.0], nb=8, nt=nt, dt=0.005, jsnap=60, bnds=0)
    return par, vel, wav, sou, rec


@pytest.mark.parametrize("precision", [1, 0], ids=["exact", "fast"])
def test_moving_geometry_per_step_vs_oracle(precision):
    """AWE_MOVE_PER_STEP on the GPU-program scheme: two sources and four
    receivers step along the model (row min(it, rows-1) of the tables, the
    last row held for the final 60 steps) against the oracle restatement."""
    from oracle import oracle
    import wavefield_imaging_gb300 as awe

    nt, rows = 200, 140
    par, vel, wav, sou, rec = _moving_case(5, nt, rows)
    ref, rsn = oracle.gpu_cart2d_moving(par, vel, wav, sou, rows, rec, rows, 0)
    desc = awe.make_desc(2, par["n"], par["d"], par["o"], nt, par["dt"], scheme=awe.SCHEME_GPU, nb=par["nb"],
                         jsnap=par["jsnap"], precision=precision)
    with awe.Plan(desc) as p:
        p.set_model(vel)
        p.set_moving_geometry(sou, rows, rec, rows, awe.MOVE_PER_STEP)
        dat, snaps = p.forward(wav, snapshots=True)
    if precision == 1:
        np.testing.assert_array_equal(dat, ref)
        np.testing.assert_array_equal(snaps, rsn)
    else:
        assert rel_l2(dat, ref) <= TOL and rel_l2(snaps, rsn) <= TOL


def test_moving_geometry_argument_checks():
    import wavefield_imaging_gb300 as awe

    nt = 50
    par, vel, wav, sou, rec = _moving_case(6, nt, nt)
    desc = awe.make_desc(2, par["n"], par["d"], par["o"], nt, par["dt"], scheme=awe.SCHEME_GPU, nb=8)
    with awe.Plan(desc) as p:
        p.set_model(vel)
        # sfDYNAWEFDcart2Dgpu's index k*(it+1) needs (n-1)*nt < n*rows
        with pytest.raises(awe.AweError, match="AWE_MOVE_DYN reads entry"):
            p.set_moving_geometry(sou[:2 * 20], 20, rec[:4 * 20], 20, awe.MOVE_DYN)
        p.set_moving_geometry(sou, nt, rec, nt, awe.MOVE_DYN)
        p.forward(wav)
    desc_b = awe.make_desc(2, par["n"], par["d"], par["o"], nt, par["dt"], scheme=awe.SCHEME_CPU, nb=8)
    with awe.Plan(desc_b) as p:
        p.set_model(vel)
        with pytest.raises(awe.AweError, match="cartesian 2D, AWE_SCHEME_GPU"):
            p.set_moving_geometry(sou, nt, rec, nt, awe.MOVE_DYN)
        p.set_moving_geometry(sou, nt, rec, nt, awe.MOVE_PER_STEP)
        with pytest.raises(awe.AweError, match="fixed sources and receivers"):
            p.gradient(wav, np.zeros((nt, 4), np.float32))
    desc_e = awe.make_desc(2, par["n"], par["d"], par["o"], nt, par["dt"], scheme=awe.SCHEME_GPU, nb=8, expl=1)
    with awe.Plan(desc_e) as p:
        p.set_model(vel)
        with pytest.raises(awe.AweError, match="expl = 0"):
            p.set_moving_geometry(sou, nt, rec, nt, awe.MOVE_PER_STEP)
