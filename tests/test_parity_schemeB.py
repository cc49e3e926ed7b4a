"""CUDA path vs the reference's CPU-program scheme.

EXACT precision must reproduce the golden fixtures (written by the
reference's own MAWEFDcart{2D,3D}cpu programs) bit for bit; FAST precision
(fused multiply-adds) must stay within rel-L2 <= 1e-5 of them.  Larger
seeded cases compare with the oracle at the same tolerance."""
import numpy as np
import pytest

from helpers import desc_from_par, golden_paths, load_golden, rel_l2, run_engine

pytestmark = pytest.mark.gpu
TOL = 1e-5  # rel-L2, FP32 (the spec parity bound)
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
