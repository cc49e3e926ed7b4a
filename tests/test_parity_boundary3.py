"""The 3D step's boundary work in one launch (k_bnd3: one-way ABC of the six
faces, sponge of the shell the step kernel leaves unsponged, receiver
gather and, when no source touches that shell, injection): against the
oracle (EXACT bit for bit, FAST within rel-L2 1e-5), against the separate
boundary launches (AWE_BND3=0), with the line ends of the level the step
read taken from that level instead of the compact copy the previous launch
wrote (AWE_BND_ENDS=0), and run twice (results must not depend on the order
in which blocks run).  Grids at the edges of the block split (an
axis-1 length that is not a multiple of 64, an axis-2 length that is not a
multiple of 16), sources inside the shell, in the sponge band, on top of
each other and across tile edges, receivers on the faces and outside the
grid, a free surface, per-source wavelets, decimated traces, and the
one-thread-per-cell step kernel beside the TMA one."""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5
D = 5.0


def _case(n, nb, nt, seed, expl=1, shell_sources=True):
    """n = model (nz, nx, ny); points placed by padded index."""
    rng = np.random.default_rng(seed)
    nz, nx, ny = n
    pz, px, py = nz + 2 * nb, nx + 2 * nb, ny + 2 * nb
    vel = (168.0 + 20.0 * rng.random((ny, nx, nz))).astype(np.float32)
    vel[:, :, : nz // 5] = 300.0
    t = np.arange(nt) * 0.005 - 0.15
    a = (np.pi * 5.0 * t) ** 2
    wav = ((1 - 2 * a) * np.exp(-a)).astype(np.float32)

    def pt(iz, ix, iy):  # padded indices -> (x, y, z) model coordinates
        return [(ix - nb) * D, (iy - nb) * D, (iz - nb) * D]

    sou = [pt(0.45 * pz, 0.5 * px, 0.4 * py),   # interior
           pt(0.45 * pz, 0.5 * px, 0.4 * py),   # on top of the first one
           pt(63.5, 15.5, 0.5 * py)]            # corners in two tiles of axis 1 and axis 2
    if shell_sources:
        sou += [pt(3, 0.5 * px, 0.5 * py),      # inside the axis-1 ABC shell
                pt(0.6 * pz, 0.3 * px, py - 3),  # inside the high axis-3 shell
                pt(2, 2, 2),                     # a corner of the grid
                pt(pz - 2.5, px - 3.5, 5.5)]     # high faces of axes 1, 2, low of 3
    sou = np.array(sou, np.float32)
    gx, gy = np.meshgrid(np.linspace(0.1, 0.9, 4) * (nx - 1) * D, np.linspace(0.1, 0.9, 3) * (ny - 1) * D,
                         indexing="ij")
    rec = np.stack([gx.ravel(), gy.ravel(), np.full(gx.size, 0.3 * (nz - 1) * D)], 1)
    faces = np.array([pt(1, 0.5 * px, 0.5 * py), pt(pz - 2, 0.5 * px, 0.5 * py), pt(0.5 * pz, 1.5, 0.5 * py),
                      pt(0.5 * pz, px - 2, 0.5 * py), pt(0.5 * pz, 0.5 * px, 1), pt(0.5 * pz, 0.5 * px, py - 2),
                      [-1e4, -1e4, -1e4]])  # the last one outside the grid
    rec = np.concatenate([rec, faces]).astype(np.float32)
    if not expl:
        wav = np.stack([wav * (1 + 0.1 * k) for k in range(sou.shape[0])], 1).astype(np.float32)
    return vel, wav, sou, rec


# (model n, nb, nt, fsrf, jdata, expl, shell sources, step kernel): padded grids
# (136, 56, 44), (132, 42, 38) with nb = 4 (the ABC shell is wider than the
# sponge band), (128, 38, 44)
CASES = [
    ((120, 40, 28), 8, 80, 0, 1, 1, False, "tma"),
    ((120, 40, 28), 8, 80, 1, 3, 1, True, "tma"),
    ((112, 22, 28), 8, 70, 0, 1, 0, True, "tma"),
    ((124, 34, 30), 4, 70, 1, 2, 1, False, "tma"),
    ((120, 40, 28), 8, 60, 0, 1, 1, True, "simple"),
]


def _run(awe, n, nb, nt, fsrf, jdata, expl, precision, vel, wav, sou, rec):
    desc = awe.make_desc(3, n, (D, D, D), (0.0, 0.0, 0.0), nt, 0.005, nb=nb, fdorder=8, dabc=1, fsrf=fsrf,
                         expl=expl, jdata=jdata, jsnap=nt - 1, bnds=1, precision=precision)
    with awe.Plan(desc) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        dat, snaps = p.forward(wav, snapshots=True)
        return dat, snaps, p.last_launch_count()


@pytest.mark.parametrize("case", range(len(CASES)))
def test_boundary_launch_matches_oracle_and_separate_launches(monkeypatch, case):
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    n, nb, nt, fsrf, jdata, expl, shell_src, kern = CASES[case]
    if kern == "simple":
        monkeypatch.setenv("AWE_STEP_KERNEL", "simple")
    vel, wav, sou, rec = _case(n, nb, nt, seed=40 + case, expl=expl, shell_sources=shell_src)
    par = dict(n=list(n), d=[D] * 3, o=[0.0] * 3, nb=nb, nt=nt, dt=0.005, fdorder=8, dabc=1, fsrf=fsrf, expl=expl,
               jsnap=nt - 1, bnds=1)
    ref, rsnaps = oracle.cart_cpu(par, vel, wav, sou, rec)
    ref = ref[::jdata]
    assert np.abs(ref).max() > 0

    ex, ex_s, launches = _run(awe, n, nb, nt, fsrf, jdata, expl, awe.EXACT, vel, wav, sou, rec)
    # step + boundary launch per time step (+ the injection launch when a
    # source lies in the shell), plus the two snapshot copies
    assert launches == (3 if shell_src else 2) * nt + ex_s.shape[0]
    np.testing.assert_array_equal(ex, ref)
    np.testing.assert_array_equal(ex_s, rsnaps)
    again, again_s, _ = _run(awe, n, nb, nt, fsrf, jdata, expl, awe.EXACT, vel, wav, sou, rec)
    np.testing.assert_array_equal(again, ex)
    np.testing.assert_array_equal(again_s, ex_s)

    fa, fa_s, _ = _run(awe, n, nb, nt, fsrf, jdata, expl, awe.FAST, vel, wav, sou, rec)
    assert rel_l2(fa, ref) <= TOL
    assert rel_l2(fa_s[-1], rsnaps[-1]) <= TOL

    # the line ends of the level the step read taken from the level itself
    # instead of the compact copy the previous launch wrote (AWE_BND_ENDS=0):
    # the same values, so bit for bit in both precisions
    monkeypatch.setenv("AWE_BND_ENDS", "0")
    le, le_s, _ = _run(awe, n, nb, nt, fsrf, jdata, expl, awe.EXACT, vel, wav, sou, rec)
    np.testing.assert_array_equal(le, ex)
    np.testing.assert_array_equal(le_s, ex_s)
    lf, lf_s, _ = _run(awe, n, nb, nt, fsrf, jdata, expl, awe.FAST, vel, wav, sou, rec)
    np.testing.assert_array_equal(lf, fa)
    np.testing.assert_array_equal(lf_s, fa_s)
    monkeypatch.delenv("AWE_BND_ENDS")

    monkeypatch.setenv("AWE_BND3", "0")
    sep, sep_s, sep_launches = _run(awe, n, nb, nt, fsrf, jdata, expl, awe.EXACT, vel, wav, sou, rec)
    assert sep_launches > launches
    np.testing.assert_array_equal(sep, ex)
    np.testing.assert_array_equal(sep_s, ex_s)


def test_source_in_the_sponge_band_keeps_the_separate_launches():
    """A source node in the sponge band but outside the shell defers the
    whole sponge of the new level to after the injection: that run keeps the
    separate boundary launches, bit-exact all the same."""
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    n, nb, nt = (120, 40, 28), 8, 50
    vel, wav, sou, rec = _case(n, nb, nt, seed=50, shell_sources=False)
    sou = np.concatenate([sou, np.array([[(7 - nb) * D, 10 * D, 60 * D]], np.float32)])  # padded x = 7
    par = dict(n=list(n), d=[D] * 3, o=[0.0] * 3, nb=nb, nt=nt, dt=0.005, fdorder=8, dabc=1, expl=1)
    ref, _ = oracle.cart_cpu(par, vel, wav, sou, rec)
    desc = awe.make_desc(3, n, (D, D, D), (0.0, 0.0, 0.0), nt, 0.005, nb=nb, fdorder=8, dabc=1, expl=1,
                         precision=awe.EXACT)
    with awe.Plan(desc) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        dat = p.forward(wav)
        assert p.last_launch_count() > 3 * nt
    np.testing.assert_array_equal(dat, ref)
