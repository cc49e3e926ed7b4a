"""Properties at the benchmark configurations' full grid sizes, where no CPU
oracle finishes in seconds: scaling the wavelet by 2 scales every trace by
2 (power-of-two scaling is exact in floating point; only the wavefront's
far tails below the normal range, 1.2e-38, which the kernels flush to zero
at one scale and not at the other, leave differences, at the rounding level
of the traces); a batched shot equals the same shot run alone; and the
gradient equals the difference of two Born images (linearity of the adjoint
in the data).  Time axes are shortened (the grids are not)."""
import numpy as np
import pytest

from helpers import rel_l2


def _twice(run, wav):
    d1 = run(wav)
    d2 = run(np.float32(2) * wav)
    return d1, d2


def _scaled(d2, d1):
    """d2 == 2 d1 up to the flushed subnormal tails."""
    d1 = np.asarray(d1, np.float64)
    d2 = np.asarray(d2, np.float64)
    assert rel_l2(d2, 2 * d1) <= 1e-6
    assert np.abs(d2 - 2 * d1).max() <= 1e-6 * np.abs(d1).max()


@pytest.mark.gpu
def test_3d_512_cube_traces_scale_with_the_wavelet():
    """512^3 (576^3 padded), nb=32, 8th order, dabc, 128x128
    receivers, on the TMA-staged step kernel."""
    import bench
    import wavefield_imaging_gb300 as awe

    w = bench.workload(nt=200)
    vel = bench.layered_model_3d(w)
    sou, rec = bench.geometry(w)
    wav = bench.ricker(w["nt"], w["dt"], w["f0"])
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], w["nt"], w["dt"], nb=w["nb"], fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)
    with awe.Plan(desc) as p:
        assert p.step_kernel == "tma3d"
        p.set_model(vel)
        p.set_geometry(sou, rec)
        d1, d2 = _twice(p.forward, wav)
    assert np.isfinite(d1).all() and np.abs(d1).max() > 0
    _scaled(d2, d1)


@pytest.mark.gpu
def test_256_shot_survey_scales_with_the_wavelet_and_shots_match_single_runs():
    """The survey: 256 shots on windows of 300-700 columns x nz 512 of a
    6000-column model, column-march kernel; two shots checked against
    single-shot plans."""
    import bench
    import wavefield_imaging_gb300 as awe

    nt, nz = 200, 512
    vel, shots = bench.batch_survey(nshots=256, nz=nz)
    wav = bench.ricker(nt, 0.005, 5.0)
    desc = awe.make_desc(2, (nz, vel.shape[0]), (5.0, 5.0), (0.0, 0.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)
    with awe.Batch(desc, shots) as b:
        b.set_model(vel)
        b.select(4, chunk=64)
        d1, d2 = _twice(b.forward, wav)
    _scaled(np.concatenate([c.ravel() for c in d2]), np.concatenate([a.ravel() for a in d1]))
    for k in (0, 171):
        x0, nx, sou, rec = shots[k]
        dk = awe.make_desc(2, (nz, nx), (5.0, 5.0), (0.0, x0 * 5.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                           precision=awe.FAST)
        with awe.Plan(dk) as p:
            p.set_model(vel[x0:x0 + nx])
            p.set_geometry(sou, rec)
            single = p.forward(wav)
        assert np.abs(single).max() > 0
        assert rel_l2(d1[k], single) <= 1e-5


@pytest.mark.gpu
def test_spherical_c4_grid_traces_scale_with_the_wavelet():
    """Spherical shell: r 700 x theta 512 x phi 512 (764 x 576 x 576 padded), one
    source and 64 x 64 receivers."""
    import bench
    import wavefield_imaging_gb300 as awe

    w = bench.spher_workload(100)
    vel = bench.spher_model(w)
    sou, rec = bench.spher_shots(w, 1)[0]
    wav = bench.ricker(w["nt"], w["dt"], w["f0"])
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], w["nt"], w["dt"], coords=awe.SPHER, scheme=awe.SCHEME_GPU,
                         nb=w["nb"], expl=0, precision=awe.FAST)
    with awe.Plan(desc) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        d1, d2 = _twice(p.forward, wav)
    assert np.isfinite(d1).all() and np.abs(d1).max() > 0
    _scaled(d2, d1)


@pytest.mark.gpu
def test_3d_512_cube_gradient_is_a_difference_of_born_images():
    """512^3 grid, a short time axis: the misfit gradient of dobs equals
    Born(dsyn) - Born(dobs) (the adjoint is linear in the data)."""
    import bench
    import wavefield_imaging_gb300 as awe

    w = bench.workload(nt=60)
    vtrue = bench.layered_model_3d(w)
    v0 = bench.smooth(vtrue, 100.0 / 5.0)
    sou, rec = bench.geometry(w)
    wav = bench.ricker(w["nt"], w["dt"], w["f0"])
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], w["nt"], w["dt"], nb=w["nb"], fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)
    with awe.Plan(desc) as p:
        p.set_geometry(sou, rec)
        p.set_model(vtrue)
        dobs = p.forward(wav)
        p.set_model(v0)
        g, J, dsyn = p.gradient(wav, dobs, ckpt_format=awe.CKPT_FP32, return_dsyn=True)
        bo = p.rtm(wav, dobs, condition=awe.IMAGE_BORN, ckpt_format=awe.CKPT_FP32)
        bs = p.rtm(wav, dsyn, condition=awe.IMAGE_BORN, ckpt_format=awe.CKPT_FP32)
    assert J > 0 and np.isfinite(g).all()
    assert rel_l2(bs - bo, g) <= 1e-3
