"""Parity at the benchmark configurations' own grids: the engine against the
reference-pinned FP32 oracle (oracle.cart_cpu, the restatement of
MAWEFDcart{2D,3D}cpu.c; oracle.gpu_scheme("spher3d"), the restatement of
MAWEFDspher3Dgpu.cu) on the full grids, with the time axis truncated where a
full run would take the oracle minutes.  Both the traces and the final
wavefield (the whole padded grid) are compared:

* AWE_EXACT: bit for bit;
* AWE_FAST: relative L2 <= 1e-5 (the FP32 parity bound), and, for the
  wavefield, <= 1e-4 in every 72^3 block that carries energy, so an error
  confined to one tile or one y-chunk cannot hide in the global norm.  One
  stated exception: the last frame of the full 4000-step 2D run, where the
  reference's own FP32 rounding noise (against FP64) exceeds 1e-5; there
  FAST is held to that noise instead (see the 2D test).

Truncated runs use the configuration's 5 MHz Ricker wavelet with its peak
moved to 0.1 us (step 20) so the wavefront is well formed inside the window.
The grid-scale workloads: 2D 512^2 (nt = 4000, the full run), the
256-shot survey (nt = 4000, three shots checked), 512^3 (576^3 padded,
nt = 60), the spherical shell 700 x 512 x 512 (764 x 576 x 576 padded,
nt = 40, the 16-shot track in one launch)."""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

BOUND = 1e-5  # rel-L2 parity bound, FP32 FAST vs the reference's FP32 order
BLOCK_BOUND = 1e-4


def ricker_at(nt, dt, f0, t0):
    t = np.arange(nt) * dt - t0
    a = (np.pi * f0 * t) ** 2
    r = (1 - 2 * a) * np.exp(-a)
    return (r / np.abs(r).max()).astype(np.float32)


def block_errors(a, b, shape, blk=72, floor=1e-3):
    """Largest rel-L2 over blocks of blk^3 cells whose oracle energy is at
    least `floor` of the largest block's."""
    a = np.asarray(a, np.float32).reshape(shape)
    b = np.asarray(b, np.float32).reshape(shape)
    norms, errs = [], []
    for i in range(0, shape[0], blk):
        for j in range(0, shape[1], blk):
            for k in range(0, shape[2], blk):
                sb = b[i:i + blk, j:j + blk, k:k + blk].astype(np.float64)
                sa = a[i:i + blk, j:j + blk, k:k + blk].astype(np.float64)
                n = np.linalg.norm(sb)
                norms.append(n)
                errs.append(np.linalg.norm(sa - sb) / n if n > 0 else 0.0)
    norms = np.array(norms)
    errs = np.array(errs)
    lit = norms >= floor * norms.max()
    return float(errs[lit].max()), int(lit.sum()), len(norms)


def _cart_desc(awe, w, nd, precision, jsnap, bnds):
    return awe.make_desc(nd, w["n"], w["d"], w["o"], w["nt"], w["dt"], nb=w["nb"], fdorder=8, dabc=1, expl=1,
                         jsnap=jsnap, bnds=bnds, precision=precision)


def _cart_par(w, jsnap, bnds):
    return dict(n=list(w["n"]), d=list(w["d"]), o=list(w["o"]), nb=w["nb"], nt=w["nt"], dt=w["dt"], fdorder=8,
                dabc=1, expl=1, jsnap=jsnap, bnds=bnds)


def _engine(awe, desc, vel, wav, sou, rec, shots=None):
    with awe.Plan(desc) as p:
        p.set_model(vel)
        if shots is None:
            p.set_geometry(sou, rec)
        else:
            p.set_shots(shots)
        if desc.jsnap > 0:
            dat, snaps = p.forward(wav, snapshots=True)
        else:
            dat, snaps = p.forward(wav), None
        kern = p.step_kernel
    return dat, snaps, kern


def test_2d_512_full_run_matches_the_oracle():
    """2D 512^2 at 5 m, nb 40, 8th order, dabc, nt = 4000 (the whole run),
    source at x = centre, z = 50 m, 512 receivers at z = 50 m, snapshots
    every 100 steps (interior)."""
    import bench
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    nz = nx = 512
    w = dict(n=(nz, nx), d=(5.0, 5.0), o=(0.0, 0.0), nt=4000, dt=0.005, nb=40)
    vel = bench.layered_model_3d(dict(n=(nz, nx, 1), d=(5.0, 5.0, 5.0), seed=1))[0]
    wav = bench.ricker(w["nt"], w["dt"], 5.0)
    sou = np.array([[0.5 * (nx - 1) * 5.0, 50.0]], np.float32)
    rec = np.stack([np.arange(nx) * 5.0, np.full(nx, 50.0)], 1).astype(np.float32)
    ref, ref_s = oracle.cart_cpu(_cart_par(w, 100, 0), vel, wav, sou, rec)
    assert np.abs(ref).max() > 0
    ex, ex_s, _ = _engine(awe, _cart_desc(awe, w, 2, awe.EXACT, 100, 0), vel, wav, sou, rec)
    assert np.array_equal(ex, ref)
    assert np.array_equal(ex_s, ref_s)
    fa, fa_s, _ = _engine(awe, _cart_desc(awe, w, 2, awe.FAST, 100, 0), vel, wav, sou, rec)
    assert rel_l2(fa, ref) <= BOUND
    assert rel_l2(fa_s, ref_s) <= BOUND
    # The last frame (step 3900) holds the late, partly absorbed field, where
    # the reference's own FP32 result is already ~1.6e-5 away from exact
    # (FP64) arithmetic.  There FAST must be as close to FP64 as the
    # reference is, and within the sum of the two rounding noises of it.
    _, r64_s = oracle.cart_cpu(_cart_par(w, 100, 0), vel, wav, sou, rec, fp64=True)
    ref_noise = rel_l2(ref_s[-1], r64_s[-1])
    fast_noise = rel_l2(fa_s[-1], r64_s[-1])
    diff = rel_l2(fa_s[-1], ref_s[-1])
    print("\nc0 final frame: reference vs FP64 %.2e, FAST vs FP64 %.2e, FAST vs reference %.2e" % (
        ref_noise, fast_noise, diff))
    assert fast_noise <= 1.5 * ref_noise
    assert diff <= max(BOUND, 2.0 * ref_noise)


def test_256_shot_survey_full_run_matches_the_oracle():
    """The survey: all 256 shots in one batched launch per step (column march),
    nt = 4000; shots 0, 128 and 255 against the oracle run on their windows."""
    import bench
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    nt, nz = 4000, 512
    vel, shots = bench.batch_survey(nshots=256, nz=nz)
    wav = bench.ricker(nt, 0.005, 5.0)
    desc = awe.make_desc(2, (nz, vel.shape[0]), (5.0, 5.0), (0.0, 0.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)
    with awe.Batch(desc, shots) as b:
        b.set_model(vel)
        b.select(4, chunk=64)
        dat = b.forward(wav)
    for k in (0, 128, 255):
        x0, nx, sou, rec = shots[k]
        par = dict(n=[nz, nx], d=[5.0, 5.0], o=[0.0, x0 * 5.0], nb=40, nt=nt, dt=0.005, fdorder=8, dabc=1, expl=1)
        ref, _ = oracle.cart_cpu(par, vel[x0:x0 + nx], wav, sou, rec)
        assert np.abs(ref).max() > 0
        assert rel_l2(dat[k], ref) <= BOUND, k


def _cube_case(lattice):
    import bench

    w = bench.workload(nt=60)
    vel = bench.layered_model_3d(w)
    sou, rec = bench.geometry(w)
    if lattice:
        # 8 x 8 x 8 sources, one at the centre of every 72^3 block of the padded
        # grid (padded index 36 + 72 k, 4 cells inside the model at the ends):
        # energy reaches every tile, y-chunk and the sponge band
        ax = [(4.0 + 72.0 * np.arange(8)) * d for d in w["d"]]
        Z, X, Y = np.meshgrid(ax[0], ax[1], ax[2], indexing="ij")
        sou = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1).astype(np.float32)
    wav = ricker_at(w["nt"], w["dt"], w["f0"], 0.1)
    return w, vel, sou, rec, wav


@pytest.mark.parametrize("lattice", [False, True], ids=["config_source", "source_lattice"])
def test_512_cube_matches_the_oracle(lattice):
    """512^3 at 5 m (576^3 padded), nb 32, 8th order, dabc, 128 x 128
    receivers at z = 50 m, nt = 60, on the TMA-staged step kernel; the final
    padded wavefield is compared whole and per 72^3 block."""
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    w, vel, sou, rec, wav = _cube_case(lattice)
    js = w["nt"] - 1  # frames at it = 0 and it = nt - 1
    ref, ref_s = oracle.cart_cpu(_cart_par(w, js, 1), vel, wav, sou, rec)
    assert np.abs(ref).max() > 0 and np.abs(ref_s[-1]).max() > 0
    ex, ex_s, kern = _engine(awe, _cart_desc(awe, w, 3, awe.EXACT, js, 1), vel, wav, sou, rec)
    assert kern == "tma3d"
    assert np.array_equal(ex, ref)
    assert np.array_equal(ex_s, ref_s)
    del ex_s
    fa, fa_s, kern = _engine(awe, _cart_desc(awe, w, 3, awe.FAST, js, 1), vel, wav, sou, rec)
    assert kern == "tma3d"
    assert rel_l2(fa, ref) <= BOUND
    assert rel_l2(fa_s[-1], ref_s[-1]) <= BOUND
    npad = tuple(n + 2 * w["nb"] for n in w["n"])[::-1]
    worst, lit, nblk = block_errors(fa_s[-1], ref_s[-1], npad)
    print("\n512^3 %s: %d of %d blocks lit, worst block rel-L2 %.2e" % ("lattice" if lattice else "config", lit, nblk,
                                                                   worst))
    assert worst <= BLOCK_BOUND
    if lattice:
        assert lit == nblk  # every block of the padded grid carries energy


def _shell_case(nt, nshots):
    import bench

    w = bench.spher_workload(nt)
    vel = bench.spher_model(w)
    shots = []
    for sou, rec in bench.spher_shots(w, nshots):
        # beside the 64 x 64 receivers, 8 on the radius through the source
        # (+-2, 4, 6, 8 cells), which the direct wave reaches within the window
        rs, ph, th = sou[0]
        near = np.array([[rs + k * w["d"][0], ph, th] for k in (-8, -6, -4, -2, 2, 4, 6, 8)], np.float32)
        shots.append((sou, np.concatenate([rec, near])))
    wav = ricker_at(nt, w["dt"], w["f0"], 0.1)
    return w, vel, shots, wav


def _spher_desc(awe, w, precision, jsnap=0, bnds=0):
    return awe.make_desc(3, w["n"], w["d"], w["o"], w["nt"], w["dt"], coords=awe.SPHER, scheme=awe.SCHEME_GPU,
                         nb=w["nb"], expl=0, jsnap=jsnap, bnds=bnds, precision=precision)


def test_spherical_shell_764x576x576_matches_the_oracle():
    """Spherical shell: r 700 x theta 512 x phi 512 (764 x 576 x 576 padded), nb 32,
    nt = 40.  The 16-shot track advances in one launch per step; shots 0 and
    15 are checked against oracle runs, shot 0 also alone in both precisions
    with its final padded wavefield."""
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    nt = 40
    w, vel, shots, wav = _shell_case(nt, 16)
    js = nt - 1
    par = dict(n=list(w["n"]), d=list(w["d"]), o=list(w["o"]), nb=w["nb"], nt=nt, dt=w["dt"], jsnap=js, bnds=1)
    ref0, ref0_s = oracle.gpu_scheme("spher3d", par, vel, wav, *shots[0])
    assert np.abs(ref0).max() > 0 and np.abs(ref0_s[-1]).max() > 0
    # shot 0 alone: EXACT bit for bit, FAST within the bound, traces and wavefield
    ex, ex_s, _ = _engine(awe, _spher_desc(awe, w, awe.EXACT, js, 1), vel, wav, *shots[0])
    assert np.array_equal(ex, ref0)
    assert np.array_equal(ex_s, ref0_s)
    del ex_s
    fa, fa_s, _ = _engine(awe, _spher_desc(awe, w, awe.FAST, js, 1), vel, wav, *shots[0])
    assert rel_l2(fa, ref0) <= BOUND
    assert rel_l2(fa_s[-1], ref0_s[-1]) <= BOUND
    npad = tuple(n + 2 * w["nb"] for n in w["n"])[::-1]
    worst, lit, nblk = block_errors(fa_s[-1], ref0_s[-1], npad)
    print("\nshell single shot: %d of %d blocks lit, worst block rel-L2 %.2e" % (lit, nblk, worst))
    assert worst <= BLOCK_BOUND
    del fa_s, ref0_s
    # the 16-shot track in one launch per step
    track, _, _ = _engine(awe, _spher_desc(awe, w, awe.FAST), vel, wav, None, None, shots=shots)
    nrs = [r.shape[0] for _, r in shots]
    cols = np.cumsum([0] + nrs)
    assert rel_l2(track[:, cols[0]:cols[1]], ref0) <= BOUND
    par15 = dict(par, jsnap=0, bnds=0)
    ref15, _ = oracle.gpu_scheme("spher3d", par15, vel, wav, *shots[15])
    assert np.abs(ref15).max() > 0
    assert rel_l2(track[:, cols[15]:cols[16]], ref15) <= BOUND
