"""FP32 error of each configuration against an FP64 CPU run of the same
scheme (the engine's AWE_FAST traces against liboracle64 / the FP64
spherical restatement).  Sizes: the 2D configuration in full (512^2, nt=4000);
the 3D and spherical ones on their full grids with the time axis truncated
(576^3 padded, 60 steps; 764 x 576 x 576 padded, 40 steps, the Ricker peak
moved to 0.1 us so the wavefront forms inside the window) and on reduced
grids over longer runs (96^3 and 120 x 48 x 48, 300 steps).  The errors are
printed (pytest -s) and bounded at about ten times the measured value, so a
regression of the FP32 path shows.  The FP32 engine against the FP32 oracle
at the configurations' full grids is test_full_config_parity.py."""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu


def _report(name, err):
    print("\nFP64_ERROR %s rel_l2=%.3e" % (name, err))


def test_2d_full_config_against_fp64():
    import bench
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    nz = nx = 512
    nt = 4000
    w3 = dict(n=(nz, nx, 1), d=(5.0, 5.0, 5.0), seed=1)
    vel = bench.layered_model_3d(w3)[0]
    wav = bench.ricker(nt, 0.005, 5.0)
    sou = np.array([[0.5 * (nx - 1) * 5.0, 50.0]], np.float32)
    rec = np.stack([np.arange(nx) * 5.0, np.full(nx, 50.0)], 1).astype(np.float32)
    par = dict(n=[nz, nx], d=[5.0, 5.0], o=[0.0, 0.0], nb=40, nt=nt, dt=0.005, fdorder=8, dabc=1, expl=1,
               nthreads=0)
    desc = awe.make_desc(2, (nz, nx), (5.0, 5.0), (0.0, 0.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)
    with awe.Plan(desc) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        dat = p.forward(wav)
    ref, _ = oracle.cart_cpu(par, vel, wav, sou, rec, fp64=True)
    err = rel_l2(dat, ref)
    _report("2D 512^2 nt=4000 8th order (the 2D forward, survey and gradient grid)", err)
    assert err <= 1.5e-5  # measured 1.5e-6


def test_3d_reduced_config_against_fp64():
    import bench
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    w = bench.workload(300, 96)
    w["nb"] = 16
    vel = bench.layered_model_3d(w)
    sou, rec = bench.geometry(w)
    rec = rec[::64]
    wav = bench.ricker(w["nt"], w["dt"], w["f0"])
    par = dict(n=list(w["n"]), d=list(w["d"]), o=list(w["o"]), nb=16, nt=w["nt"], dt=w["dt"], fdorder=8, dabc=1,
               expl=1)
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], w["nt"], w["dt"], nb=16, fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)
    with awe.Plan(desc) as p:
        assert p.step_kernel == "tma3d"
        p.set_model(vel)
        p.set_geometry(sou, rec)
        dat = p.forward(wav)
    ref, _ = oracle.cart_cpu(par, vel, wav, sou, rec, fp64=True)
    err = rel_l2(dat, ref)
    _report("3D 96^3 nt=300 8th order, TMA kernel", err)
    assert err <= 2.5e-6  # measured 2.2e-7


def test_spherical_reduced_config_against_fp64():
    import bench
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    w = bench.spher_workload(300, nr=120, nang=48)
    w["nb"] = 10
    w["d"] = (0.005, 0.04 / 512, 0.04 / 512)
    vel = bench.spher_model(w)
    nr_, nth, nph = w["n"]
    rs = 3387.0 + 0.6 * nr_ * 0.005
    th0 = w["o"][1] + 0.5 * (nth - 1) * w["d"][1]
    ph0 = w["o"][2] + 0.5 * (nph - 1) * w["d"][2]
    sou = np.array([[rs, ph0, th0]], np.float32)
    rec = np.array([[rs + 0.02, ph0 + k * w["d"][2], th0] for k in range(-12, 13, 3)], np.float32)
    wav = bench.ricker(w["nt"], w["dt"], w["f0"])
    par = dict(n=list(w["n"]), d=list(w["d"]), o=list(w["o"]), nb=10, nt=w["nt"], dt=w["dt"])
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], w["nt"], w["dt"], coords=awe.SPHER, scheme=awe.SCHEME_GPU,
                         nb=10, precision=awe.FAST)
    with awe.Plan(desc) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        dat = p.forward(wav)
    ref = oracle.spher3d_fp64(par, vel, wav, sou, rec)
    err = rel_l2(dat, ref)
    _report("spherical shell 120x48x48 nt=300", err)
    assert err <= 4e-5  # measured 3.9e-6


def _ricker_at(nt, dt, f0, t0):
    t = np.arange(nt) * dt - t0
    a = (np.pi * f0 * t) ** 2
    r = (1 - 2 * a) * np.exp(-a)
    return (r / np.abs(r).max()).astype(np.float32)


def test_3d_full_grid_against_fp64():
    """The 512^3 grid (512^3, 576^3 padded, nb 32, 128 x 128 receivers), 60 steps:
    traces and the final padded wavefield against the FP64 oracle."""
    import bench
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    w = bench.workload(nt=60)
    vel = bench.layered_model_3d(w)
    sou, rec = bench.geometry(w)
    wav = _ricker_at(w["nt"], w["dt"], w["f0"], 0.1)
    js = w["nt"] - 1
    par = dict(n=list(w["n"]), d=list(w["d"]), o=list(w["o"]), nb=w["nb"], nt=w["nt"], dt=w["dt"], fdorder=8, dabc=1,
               expl=1, jsnap=js, bnds=1)
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], w["nt"], w["dt"], nb=w["nb"], fdorder=8, dabc=1, expl=1,
                         jsnap=js, bnds=1, precision=awe.FAST)
    with awe.Plan(desc) as p:
        assert p.step_kernel == "tma3d"
        p.set_model(vel)
        p.set_geometry(sou, rec)
        dat, snaps = p.forward(wav, snapshots=True)
    ref, ref_s = oracle.cart_cpu(par, vel, wav, sou, rec, fp64=True)
    assert np.abs(ref).max() > 0
    err, err_w = rel_l2(dat, ref), rel_l2(snaps[-1], ref_s[-1])
    _report("3D 512^3 (576^3 padded) nt=60 traces", err)
    _report("3D 512^3 (576^3 padded) nt=60 final wavefield", err_w)
    assert err <= 2.5e-6  # measured 2.2e-7
    assert err_w <= 3.5e-6  # measured 3.3e-7


def test_spherical_full_grid_against_fp64():
    """The spherical shell's full grid (764 x 576 x 576 padded, nb 32), one source of the track
    with 64 x 64 receivers and 8 more on its radius, 40 steps: traces against
    the FP64 spherical restatement."""
    import bench
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    nt = 40
    w = bench.spher_workload(nt)
    vel = bench.spher_model(w)
    sou, rec = bench.spher_shots(w, 1)[0]
    rs, ph, th = sou[0]
    near = np.array([[rs + k * w["d"][0], ph, th] for k in (-8, -6, -4, -2, 2, 4, 6, 8)], np.float32)
    rec = np.concatenate([rec, near])
    wav = _ricker_at(nt, w["dt"], w["f0"], 0.1)
    par = dict(n=list(w["n"]), d=list(w["d"]), o=list(w["o"]), nb=w["nb"], nt=nt, dt=w["dt"])
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], nt, w["dt"], coords=awe.SPHER, scheme=awe.SCHEME_GPU, nb=w["nb"],
                         expl=0, precision=awe.FAST)
    with awe.Plan(desc) as p:
        assert p.step_kernel == "tma_sph"
        p.set_model(vel)
        p.set_geometry(sou, rec)
        dat = p.forward(wav)
    ref = oracle.spher3d_fp64(dict(par, expl=0), vel, wav, sou, rec)
    assert np.abs(ref).max() > 0
    err = rel_l2(dat, ref)
    _report("spherical shell 764x576x576 padded nt=40 traces", err)
    assert err <= 3.5e-6  # measured 3.1e-7
