"""The TMA-staged spherical step (k_stepA_sph_tma, AWE_FAST) against the
register-march kernel it replaces (k_stepA_sph_march2, forced with
AWE_STEP_KERNEL=simple) and against the oracle restatement of
sfAWEFDspher3Dgpu: traces and whole snapshot frames, across partial r and
theta tiles, phi-chunk boundaries, the free-surface mask and several shots
in one launch.  Both kernels evaluate the same packed FP32x2 expressions, so
they agree to rel-L2 1e-6 (bit for bit where the compiler schedules both
alike); the oracle bar is the FAST tolerance of the other parity tests,
rel-L2 1e-5."""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu
TOL_KERNELS = 1e-6
TOL_ORACLE = 1e-5

D = (0.005, 1.5e-6, 1.5e-6)


def _case(n, seed, nt=120, nsrc=1):
    rng = np.random.default_rng(seed)
    o = (3387.0, np.pi / 2 - (n[1] // 2) * D[1], -(n[2] // 2) * D[2])
    vel = (0.168 + 0.01 * rng.random((n[2], n[1], n[0]))).astype(np.float32)
    vel[:, :, int(0.75 * n[0]):] = 0.3
    t = np.arange(nt) * 0.005 - 0.3
    wav = ((1 - 2 * (np.pi * 5 * t) ** 2) * np.exp(-(np.pi * 5 * t) ** 2)).astype(np.float32)
    sou = np.array([[o[0] + (0.6 * n[0] - k) * D[0], o[2] + (0.4 * n[2] + 2 * k) * D[2],
                     o[1] + (0.5 * n[1] - k) * D[1]] for k in range(nsrc)], np.float32)
    rec = np.array([[o[0] + 0.7 * n[0] * D[0], o[2] + k * D[2], o[1] + 0.45 * n[1] * D[1]]
                    for k in range(3, n[2] - 3, 3)], np.float32)
    return o, vel, wav, sou, rec


def _run(monkeypatch, kernel, n, o, vel, wav, sou, rec, nb=6, fsrf=0, jsnap=0, chunk=None, shots=None):
    import wavefield_imaging_gb300 as awe

    if kernel == "simple":
        monkeypatch.setenv("AWE_STEP_KERNEL", "simple")
    else:
        monkeypatch.delenv("AWE_STEP_KERNEL", raising=False)
    if chunk is not None:
        monkeypatch.setenv("AWE_TMA_CHUNK", str(chunk))
    else:
        monkeypatch.delenv("AWE_TMA_CHUNK", raising=False)
    desc = awe.make_desc(3, n, D, o, wav.shape[0], 0.005, coords=awe.SPHER, scheme=awe.SCHEME_GPU, nb=nb,
                         fsrf=fsrf, jsnap=jsnap, precision=awe.FAST)
    with awe.Plan(desc) as p:
        assert p.step_kernel == ("simple" if kernel == "simple" else "tma_sph")
        p.set_model(vel)
        if shots is not None:
            p.set_shots(shots)
            return p.forward(wav), None
        p.set_geometry(sou, rec)
        if jsnap > 0:
            return p.forward(wav, snapshots=True)
        return p.forward(wav), None


# padded grids: (72, 52, 48) two r tiles (the second 8 wide), a partial
# theta tile, 5-plane phi chunks; (128, 32, 37) whole tiles, one chunk;
# (60, 30, 26) one partial r tile, 3-plane chunks
CASES = [((60, 40, 36), 1, 5), ((116, 20, 25), 0, None), ((48, 18, 14), 1, 3)]


@pytest.mark.parametrize("n,fsrf,chunk", CASES, ids=["partial_tiles_free", "whole_tiles", "small_chunks_free"])
def test_tma_matches_register_march_traces_and_frames(monkeypatch, n, fsrf, chunk):
    o, vel, wav, sou, rec = _case(n, seed=51 + n[0])
    dat_s, snap_s = _run(monkeypatch, "simple", n, o, vel, wav, sou, rec, fsrf=fsrf, jsnap=40)
    dat_t, snap_t = _run(monkeypatch, "tma", n, o, vel, wav, sou, rec, fsrf=fsrf, jsnap=40, chunk=chunk)
    assert np.abs(dat_s).max() > 0 and np.abs(snap_s).max() > 0
    assert rel_l2(dat_t, dat_s) <= TOL_KERNELS
    assert rel_l2(snap_t, snap_s) <= TOL_KERNELS
    # every frame cell, not only the norm: no tile is left unwritten or misplaced
    scale = np.abs(snap_s).max()
    assert np.abs(snap_t - snap_s).max() <= 1e-5 * scale


@pytest.mark.parametrize("n,fsrf,chunk", CASES[:2], ids=["partial_tiles_free", "whole_tiles"])
def test_tma_vs_oracle(monkeypatch, n, fsrf, chunk):
    from oracle import oracle

    o, vel, wav, sou, rec = _case(n, seed=61 + n[0], nsrc=2)
    dat, _ = _run(monkeypatch, "tma", n, o, vel, wav, sou, rec, fsrf=fsrf, chunk=chunk)
    par = dict(kind="spher3d", n=list(n), d=list(D), o=list(o), nb=6, nt=wav.shape[0], dt=0.005, jsnap=0, fsrf=fsrf)
    ref, _ = oracle.gpu_scheme("spher3d", par, vel, wav, sou, rec)
    assert np.abs(ref).max() > 0
    assert rel_l2(dat, ref) <= TOL_ORACLE


def test_tma_several_shots_in_one_launch(monkeypatch):
    """Three shots stacked along phi in one launch per step: their traces
    equal those of the register-march kernel's multi-shot run, and the shots
    do not see each other (each equals its own single-shot TMA run)."""
    n = (40, 30, 28)
    o, vel, wav, _, _ = _case(n, seed=71)
    shots = []
    for k in range(3):
        sou = np.array([[o[0] + 25 * D[0], o[2] + (10 + 4 * k) * D[2], o[1] + 15 * D[1]]], np.float32)
        rec = np.array([[o[0] + 28 * D[0], o[2] + j * D[2], o[1] + (12 + k) * D[1]] for j in range(4, 24, 4)],
                       np.float32)
        shots.append((sou, rec))
    tma, _ = _run(monkeypatch, "tma", n, o, vel, wav, None, None, chunk=7, shots=shots)
    simple, _ = _run(monkeypatch, "simple", n, o, vel, wav, None, None, shots=shots)
    assert rel_l2(tma, simple) <= TOL_KERNELS
    off = 0
    for sou, rec in shots:
        single, _ = _run(monkeypatch, "tma", n, o, vel, wav, sou, rec, chunk=7)
        np.testing.assert_array_equal(tma[:, off:off + rec.shape[0]], single)
        off += rec.shape[0]
