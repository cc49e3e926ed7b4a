"""Batched 2D forward (awe_batch_*): shots on uneven windows of one model,
one launch per time step for all shots, replayed as a CUDA graph.  Each
shot's traces must equal a single-shot run on its window (and the oracle of
the reference scheme) within the FAST tolerance."""
import numpy as np
import pytest

from helpers import rel_l2, ricker

TOL = 1e-5


def _survey(nshots=5, nz=60, nxm=220, seed=3):
    rng = np.random.default_rng(seed)
    vel = (150.0 + 30.0 * rng.random((nxm, nz))).astype(np.float32)
    vel[:, :10] = 300.0
    d = 5.0
    shots = []
    for s in range(nshots):
        nx = int(rng.integers(40, 90))
        x0 = int(rng.integers(0, nxm - nx))
        xs = (x0 + nx / 2) * d
        sou = np.array([[xs, 12 * d]], np.float32)
        rec = np.stack([np.linspace(xs - 15 * d, xs + 15 * d, 11), np.full(11, 8 * d)], 1).astype(np.float32)
        shots.append((x0, nx, sou, rec))
    return vel, shots


def _desc(nz, nxm, nt, jdata=1, fsrf=0):
    import wavefield_imaging_gb300 as awe

    return awe.make_desc(2, (nz, nxm), (5.0, 5.0), (0.0, 0.0), nt, 0.005, nb=10, fdorder=8, dabc=1, expl=1,
                         jdata=jdata, fsrf=fsrf, precision=awe.FAST)


@pytest.mark.gpu
@pytest.mark.parametrize("jdata,fsrf", [(1, 0), (3, 1)])
def test_batch_matches_single_shot_runs_and_oracle(jdata, fsrf):
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    nz, nxm, nt = 60, 220, 240
    vel, shots = _survey(nz=nz, nxm=nxm)
    wav = ricker(nt, 0.005)
    with awe.Batch(_desc(nz, nxm, nt, jdata, fsrf), shots) as b:
        b.set_model(vel)
        dats = b.forward(wav)
        tile, grid = b.tune(steps=10)
        dats2 = b.forward(wav)
    for (x0, nx, sou, rec), dat, dat2 in zip(shots, dats, dats2):
        win = vel[x0:x0 + nx]
        o = (0.0, x0 * 5.0)
        desc = awe.make_desc(2, (nz, nx), (5.0, 5.0), o, nt, 0.005, nb=10, fdorder=8, dabc=1, expl=1, jdata=jdata,
                             fsrf=fsrf, precision=awe.FAST)
        with awe.Plan(desc) as p:
            p.set_model(win)
            p.set_geometry(sou, rec)
            single = p.forward(wav)
        assert rel_l2(dat, single) <= TOL
        assert rel_l2(dat2, single) <= TOL  # after autotuning (another tile shape)
        par = dict(n=[nz, nx], d=[5.0, 5.0], o=list(o), nb=10, nt=nt, dt=0.005, fdorder=8, dabc=1, expl=1,
                   fsrf=fsrf)
        ref, _ = oracle.cart_cpu(par, win, wav, sou, rec)
        assert rel_l2(dat, ref[::jdata]) <= TOL


def test_batch_rejects_bad_windows_without_a_device():
    import wavefield_imaging_gb300 as awe

    vel, shots = _survey()
    bad = [(200, 50, shots[0][2], shots[0][3])]  # 200 + 50 > 220 columns
    with pytest.raises(awe.AweError) as e:
        awe.Batch(_desc(60, 220, 10), bad)
    assert e.value.status == 1
    desc3 = awe.make_desc(3, (8, 8, 8), (5.0,) * 3, (0.0,) * 3, 10, 0.005, fdorder=8)
    with pytest.raises(awe.AweError) as e:
        awe.Batch(desc3, shots[:1])
    assert e.value.status == 4


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", [7, 32, 1000])
def test_column_march_equals_tile_kernel(chunk):
    """The column-march forward (whole columns streamed by bulk copies into a
    shared-memory ring, x neighbours from registers) performs the tile
    kernel's arithmetic in the same order: traces equal bit for bit, for
    chunks shorter than, comparable to and longer than the windows."""
    import wavefield_imaging_gb300 as awe

    nz, nxm, nt = 60, 220, 240
    vel, shots = _survey(nz=nz, nxm=nxm)
    wav = ricker(nt, 0.005)
    with awe.Batch(_desc(nz, nxm, nt, 3, 1), shots) as b:
        b.set_model(vel)
        b.select(0)
        ref = b.forward(wav)
        b.select(4, chunk=chunk)
        assert (b.info.tile_z, b.info.tile_x) == (nz + 20, chunk)
        col = b.forward(wav)
        col2 = b.forward(wav)  # graph replay
    for r, c, c2 in zip(ref, col, col2):
        assert np.abs(r).max() > 0
        np.testing.assert_array_equal(c, r)
        np.testing.assert_array_equal(c2, r)


@pytest.mark.gpu
def test_batch_gradient_with_column_march_forward():
    """The batched gradient's forward and recompute passes run the column
    march when it is selected; its levels equal the tile kernel's, so the
    misfit and the gradient are the same bit for bit."""
    import wavefield_imaging_gb300 as awe

    nz, nxm, nt = 60, 220, 160
    vel, shots = _survey(nz=nz, nxm=nxm)
    wav = ricker(nt, 0.005)
    with awe.Batch(_desc(nz, nxm, nt, 1, 0), shots) as b:
        b.set_model(vel)
        dobs = b.forward(wav)
        b.set_model((vel * 1.02).astype(np.float32))
        b.select(0)
        g0, J0 = b.gradient(wav, dobs, ckpt_format=awe.CKPT_FP32)
        b.select(4, chunk=24)
        g1, J1 = b.gradient(wav, dobs, ckpt_format=awe.CKPT_FP32)
    assert J0 > 0 and J1 == J0
    np.testing.assert_array_equal(g1, g0)


@pytest.mark.gpu
def test_batch_gradient_is_the_sum_of_per_shot_gradients():
    """The batch's misfit gradient against the FP64 oracle of every shot on
    its window, summed onto the model columns."""
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    nz, nxm, nt = 60, 220, 200
    vel, shots = _survey(nshots=4, nz=nz, nxm=nxm, seed=9)
    rng = np.random.default_rng(4)
    vtrue = (vel * (1 + 0.05 * rng.standard_normal(vel.shape))).astype(np.float32)
    wav = ricker(nt, 0.005)
    gsum = np.zeros(vel.shape, np.float64)
    Jsum = 0.0
    dobs = []
    for (x0, nx, sou, rec) in shots:
        par = dict(n=[nz, nx], d=[5.0, 5.0], o=[0.0, x0 * 5.0], nb=10, nt=nt, dt=0.005, fdorder=8, dabc=1, expl=1)
        d, _ = oracle.cart_cpu(par, vtrue[x0:x0 + nx], wav, sou, rec)
        dobs.append(d)
        g, J, _ = oracle.misfit_gradient(par, vel[x0:x0 + nx], wav, sou, rec, d)
        gsum[x0:x0 + nx] += g
        Jsum += J
    with awe.Batch(_desc(nz, nxm, nt), shots) as b:
        b.set_model(vel)
        g32, J32 = b.gradient(wav, dobs, ckpt_format=awe.CKPT_FP32)
        g16, J16 = b.gradient(wav, dobs, ckpt_format=awe.CKPT_BF16)
        gbf, Jbf = b.gradient(wav, dobs, ckpt_format=awe.CKPT_BFP16)
        b.tune(steps=5)
        g32b, _ = b.gradient(wav, dobs, ckpt_format=awe.CKPT_FP32)
    assert abs(J32 - Jsum) <= 1e-5 * Jsum
    assert J16 == J32
    assert rel_l2(g32, gsum) <= 1e-4
    assert rel_l2(g32b, gsum) <= 1e-4  # another tile shape after tuning
    assert rel_l2(g16, gsum) <= 3e-2
    assert Jbf == J32 and rel_l2(gbf, gsum) <= 1e-3  # block floating point checkpoints
