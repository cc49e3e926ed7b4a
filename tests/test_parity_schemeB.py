"""CUDA path vs the reference's CPU-program scheme.

EXACT precision must reproduce the golden fixtures (written by the
reference's own MAWEFDcart{2D,3D}cpu programs) bit for bit; FAST precision
(fused multiply-adds) must stay within rel-L2 <= 1e-5 of them.  Larger
seeded cases compare with the oracle at the same tolerance."""
import numpy as np
import pytest

from helpers import desc_from_par, golden_paths, load_golden, rel_l2, run_engine

pytestmark = pytest.mark.gpu
TOL = 1e-5  # rel-L2, FP32 (the parity bound for FAST arithmetic)
GOLDEN = golden_paths()


@pytest.mark.parametrize("path", GOLDEN, ids=[p.split("/")[-1][:-4] for p in GOLDEN])
def test_exact_mode_bit_exact_vs_reference(path):
    par, a = load_golden(path)
    dat, snaps, launches = run_engine(par, a["vel"], a["wav"], a["sou"], a["rec"], den=a.get("den"), precision=1)
    assert launches > 0
    assert dat.shape == a["dat"].shape
    np.testing.assert_array_equal(dat, a["dat"])
    if "snaps" in a:
        np.testing.assert_array_equal(snaps.ravel(), a["snaps"])


@pytest.mark.parametrize("path", GOLDEN, ids=[p.split("/")[-1][:-4] for p in GOLDEN])
def test_fast_mode_within_tolerance(path):
    par, a = load_golden(path)
    dat, snaps, _ = run_engine(par, a["vel"], a["wav"], a["sou"], a["rec"], den=a.get("den"), precision=0)
    assert rel_l2(dat, a["dat"]) <= TOL
    if "snaps" in a:
        assert rel_l2(snaps.ravel(), a["snaps"]) <= TOL


def test_graph_replay_equals_direct_launches():
    """The CPU-program scheme's loop runs as a captured CUDA graph when no
    snapshots or profiling are requested; replays, re-captures after a
    geometry change, and the directly launched loop give the same traces."""
    import wavefield_imaging_gb300 as awe

    par, a = load_golden(golden_paths("c2d_o8_sponge.npz")[0])
    with awe.Plan(desc_from_par(par, precision=1)) as p:
        p.set_model(a["vel"])
        p.set_geometry(a["sou"], a["rec"])
        g1 = p.forward(a["wav"])  # captured
        g2 = p.forward(a["wav"])  # replayed
        p.profile(True)  # profiled runs launch directly
        d1 = p.forward(a["wav"])
        p.profile(False)
        p.set_geometry(a["sou"], a["rec"][::-1].copy())
        g3 = p.forward(a["wav"])  # re-captured with the new receivers
    np.testing.assert_array_equal(g1, a["dat"])
    np.testing.assert_array_equal(g2, g1)
    np.testing.assert_array_equal(d1, g1)
    np.testing.assert_array_equal(g3, g1[:, ::-1])


@pytest.mark.parametrize("precision", [1, 0], ids=["exact", "fast"])
def test_moving_geometry_per_step_equals_fixed_points(precision):
    """AWE_MOVE_PER_STEP on the CPU-program scheme (8th order, sponge, one
    wavelet per source): a moving receiver's sample at step it is the fixed
    receiver at that step's position, and one source that jumps between three
    positions equals a fixed run with a source at each position whose wavelet
    is zero outside its steps - bit for bit, in both precisions."""
    import wavefield_imaging_gb300 as awe

    par, a = load_golden(golden_paths("c2d_o8_sponge.npz")[0])
    nt = 150
    par = dict(par, nt=nt, expl=0, jsnap=0)
    wav = np.ascontiguousarray(a["wav"][:nt])
    pos = np.array([[110.0, 60.0], [150.5, 75.2], [200.0, 100.0]], np.float32)
    which = np.arange(nt) * 3 // nt  # source position of each step
    rx = (20.0 + 1.3 * np.arange(nt)).astype(np.float32)
    rec_moving = np.stack([np.stack([rx, np.full(nt, 40.3, np.float32)], 1),
                           np.tile(np.array([[250.0, 70.1]], np.float32), (nt, 1))], 1).reshape(-1, 2)
    with awe.Plan(desc_from_par(par, precision=precision)) as p:
        p.set_model(a["vel"])
        p.set_moving_geometry(pos[which], nt, rec_moving, nt, awe.MOVE_PER_STEP)
        dat = p.forward(wav)
        rec_fixed = np.concatenate([np.stack([rx, np.full(nt, 40.3, np.float32)], 1),
                                    np.array([[250.0, 70.1]], np.float32)])
        p.set_geometry(pos, rec_fixed)
        w3 = np.zeros((nt, 3), np.float32)
        w3[np.arange(nt), which] = wav
        ref = p.forward(w3)
    assert dat.shape == (nt, 2)
    np.testing.assert_array_equal(dat[:, 0], ref[np.arange(nt), np.arange(nt)])
    np.testing.assert_array_equal(dat[:, 1], ref[:, nt])
    assert np.abs(dat).max() > 0


@pytest.mark.parametrize("nd", [2, 3])
def test_captured_loop_follows_a_new_model_and_moved_points(nd):
    """The captured time loop is kept across awe_set_model (the model is
    refilled in place on the device) and across awe_set_geometry with the same
    point counts; its replay must equal a new plan's run on the new model and
    points, bit for bit (AWE_EXACT, the 8th-order sponge/ABC scheme)."""
    import wavefield_imaging_gb300 as awe

    name = "c2d_o8_sponge.npz" if nd == 2 else "c3d_o8_tma_shape.npz"
    par, a = load_golden(golden_paths(name)[0])
    par = dict(par, jsnap=0)
    vel2 = (a["vel"] * np.float32(1.07)).astype(np.float32)
    sou2 = (a["sou"] + np.float32(2.5)).astype(np.float32)
    with awe.Plan(desc_from_par(par, precision=1)) as p:
        p.set_model(a["vel"])
        p.set_geometry(a["sou"], a["rec"])
        first = p.forward(a["wav"])  # captured
        np.testing.assert_array_equal(first, a["dat"])
        p.set_model(vel2)
        p.set_geometry(sou2, a["rec"])
        kept = p.forward(a["wav"])
    with awe.Plan(desc_from_par(par, precision=1)) as q:
        q.set_model(vel2)
        q.set_geometry(sou2, a["rec"])
        fresh = q.forward(a["wav"])
    assert not np.array_equal(kept, first)
    np.testing.assert_array_equal(kept, fresh)
