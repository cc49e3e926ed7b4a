"""The TMA-staged 3D 8th-order step kernel (k_stepB3_o8) against the oracle
and against the one-thread-per-cell kernel: EXACT precision bit for bit,
FAST within rel-L2 1e-5, across y-chunk boundaries, partial tiles, free
surface and no-ABC runs."""
import numpy as np
import pytest

from helpers import golden_paths, load_golden, rel_l2, run_engine

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _oracle(par, vel, wav, sou, rec, den=None):
    from oracle import oracle

    return oracle.cart_cpu(par, vel, wav, sou, rec, den=den)


def _case(n=(40, 36, 30), nb=8, nt=90, fsrf=0, dabc=1, seed=21):
    rng = np.random.default_rng(seed)
    nz, nx, ny = n
    vel = (168.0 + 20.0 * rng.random((ny, nx, nz))).astype(np.float32)
    vel[:, :, : nz // 5] = 300.0
    t = np.arange(nt) * 0.005 - 0.3
    a = (np.pi * 5.0 * t) ** 2
    wav = ((1 - 2 * a) * np.exp(-a)).astype(np.float32)
    d = 5.0
    sou = np.array([[0.5 * (nx - 1) * d, 0.4 * (ny - 1) * d, 0.45 * (nz - 1) * d]], np.float32)
    gx, gy = np.meshgrid(np.linspace(0.1, 0.9, 5) * (nx - 1) * d, np.linspace(0.1, 0.9, 4) * (ny - 1) * d,
                         indexing="ij")
    rec = np.stack([gx.ravel(), gy.ravel(), np.full(gx.size, 0.3 * (nz - 1) * d)], 1).astype(np.float32)
    par = dict(n=list(n), d=[d] * 3, o=[0.0] * 3, nb=nb, nt=nt, dt=0.005, fdorder=8, dabc=dabc, fsrf=fsrf, expl=1,
               jsnap=30)
    return par, vel, wav, sou, rec


def _plan_kernel(par):
    import wavefield_imaging_gb300 as awe
    from helpers import desc_from_par

    with awe.Plan(desc_from_par(par)) as p:
        return p.step_kernel


@pytest.mark.parametrize("chunk", ["0", "8", "5"])
def test_exact_tma_bit_exact_vs_oracle(monkeypatch, chunk):
    monkeypatch.setenv("AWE_TMA_CHUNK", chunk)
    par, vel, wav, sou, rec = _case()
    assert _plan_kernel(par) == "tma3d"
    dat, snaps, _ = run_engine(par, vel, wav, sou, rec, precision=1)
    ref, rsnaps = _oracle(par, vel, wav, sou, rec)
    np.testing.assert_array_equal(dat, ref)
    np.testing.assert_array_equal(snaps.ravel(), rsnaps.ravel())


@pytest.mark.parametrize("fsrf,dabc", [(1, 1), (0, 0)])
def test_exact_tma_free_surface_and_no_abc(fsrf, dabc):
    par, vel, wav, sou, rec = _case(n=(44, 34, 26), nb=6, fsrf=fsrf, dabc=dabc, seed=22)
    dat, _, _ = run_engine(par, vel, wav, sou, rec, precision=1)
    ref, _ = _oracle(par, vel, wav, sou, rec)
    np.testing.assert_array_equal(dat, ref)


@pytest.mark.parametrize("precision", [1, 0])
def test_tma_tiles_inside_the_undamped_interior(precision):
    """Tiles whose sponge factors are all 1 skip the sponge multiplies; a grid
    with such tiles next to damped ones (axis 1 padded to 136: the tile
    [64, 128) is undamped) must still match the oracle."""
    par, vel, wav, sou, rec = _case(n=(120, 40, 28), nb=8, nt=110, seed=24)
    dat, snaps, _ = run_engine(par, vel, wav, sou, rec, precision=precision)
    ref, rsnaps = _oracle(par, vel, wav, sou, rec)
    if precision == 1:
        np.testing.assert_array_equal(dat, ref)
        np.testing.assert_array_equal(snaps.ravel(), rsnaps.ravel())
    else:
        assert rel_l2(dat, ref) <= TOL


def test_fast_tma_within_tolerance_and_matches_simple_kernel(monkeypatch):
    par, vel, wav, sou, rec = _case(n=(56, 48, 40), nb=10, nt=150, seed=23)
    dat, _, _ = run_engine(par, vel, wav, sou, rec, precision=0)
    ref, _ = _oracle(par, vel, wav, sou, rec)
    assert rel_l2(dat, ref) <= TOL
    monkeypatch.setenv("AWE_STEP_KERNEL", "simple")
    assert _plan_kernel(par) == "simple"
    simple, _, _ = run_engine(par, vel, wav, sou, rec, precision=0)
    assert rel_l2(dat, simple) <= TOL


def test_golden_tma_shapes_take_the_tma_kernel():
    for path in golden_paths("c3d_o8_tma_*.npz"):
        par, _ = load_golden(path)
        assert _plan_kernel(par) == "tma3d"
