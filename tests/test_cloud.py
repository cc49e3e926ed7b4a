"""Point-cloud windowing and merging (awe_cloud_window / awe_cloud_merge)
against fixtures written by the reference's own Mbycloudwin3d and
Mbycloudmerge3d (tests/golden/make_golden_cloud.py): the oracle restatement
on the CPU and the CUDA path on the GPU, bit for bit."""
import json

import numpy as np
import pytest

from helpers import golden_paths

CLOUD = golden_paths("pc_*.npz")


def load(path):
    z = np.load(path)
    par = json.loads(str(z["par"]))
    k = 0
    wins = []
    while "orbit%d" % k in z:
        wins.append((z["orbit%d" % k], z["win%d" % k], z["wdat%d" % k]))
        k += 1
    return par, z, wins


def window_data(par, z):
    """The reference windows complex data; the real case keeps the real part."""
    return z["data"].astype(np.complex64)


@pytest.mark.parametrize("path", CLOUD, ids=lambda p: p.split("/")[-1][:-4])
def test_oracle_matches_reference_programs(path):
    from oracle import oracle

    par, z, wins = load(path)
    merged_in = []
    for orb, win, wdat in wins:
        idx, pts, d = oracle.cloud_window(z["cloud"], orb, par["apt"], window_data(par, z))
        assert np.array_equal(pts, win)
        np.testing.assert_array_equal(d if par["complex"] else d.real, wdat)
        assert np.array_equal(z["cloud"][idx], win)
        merged_in.append((win, wdat))
    m = oracle.cloud_merge(z["cloud"], merged_in, norm=par["norm"])
    np.testing.assert_array_equal(m, z["merged"])


def test_fixtures_cover_overlap_and_both_types():
    kinds = set()
    for path in CLOUD:
        par, z, wins = load(path)
        kinds.add((par["complex"], par["norm"]))
        ids = [set(map(tuple, w[1][:, :3].tolist())) for w in wins]
        assert any(ids[i] & ids[j] for i in range(len(ids)) for j in range(i + 1, len(ids)))  # fold > 1 somewhere
    assert kinds == {(True, True), (False, False)}


@pytest.mark.gpu
@pytest.mark.parametrize("path", CLOUD, ids=lambda p: p.split("/")[-1][:-4])
def test_engine_matches_reference_programs(path):
    import wavefield_imaging_gb300 as awe

    par, z, wins = load(path)
    merged_in = []
    for orb, win, wdat in wins:
        idx, pts, d = awe.cloud_window(z["cloud"], orb, par["apt"], window_data(par, z))
        assert np.array_equal(pts, win)
        np.testing.assert_array_equal(d if par["complex"] else d.real, wdat)
        merged_in.append((win, wdat))
    m = awe.cloud_merge(z["cloud"], merged_in, norm=par["norm"])
    np.testing.assert_array_equal(m, z["merged"])


@pytest.mark.gpu
def test_engine_large_cloud_vs_oracle():
    """60k ground points, 40 orbit points, real data of 3 rows: indices,
    points and columns equal the oracle's; an orbit far away keeps nothing."""
    import wavefield_imaging_gb300 as awe
    from oracle import oracle

    rng = np.random.default_rng(7)
    ng = 60000
    th, ph = rng.uniform(-0.05, 0.05, ng), rng.uniform(-0.05, 0.05, ng)
    xyz = 3390.0 * np.stack([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), np.sin(th)], 1)
    g = np.zeros((ng, 9), np.float32)
    g[:, :3] = xyz
    g[:, 3:6] = xyz / 3390.0
    t = np.linspace(-0.03, 0.03, 40)
    orb = np.zeros((40, 9), np.float32)
    orb[:, 0], orb[:, 2] = 3690.0 * np.cos(t), 3690.0 * np.sin(t)
    data = rng.normal(size=(3, ng)).astype(np.float32)
    i1, p1, d1 = awe.cloud_window(g, orb, 4.0, data)
    i0, p0, d0 = oracle.cloud_window(g, orb, 4.0, data)
    assert 0 < i1.size < ng
    np.testing.assert_array_equal(i1, i0)
    np.testing.assert_array_equal(p1, p0)
    np.testing.assert_array_equal(d1, d0)
    far = orb.copy()
    far[:, 1] = 1e5
    i2, p2, d2 = awe.cloud_window(g, far, 1.0, data)
    assert i2.size == 0 and p2.shape == (0, 9) and d2.shape == (3, 0)


@pytest.mark.gpu
def test_merge_rejects_points_missing_from_the_cloud():
    import wavefield_imaging_gb300 as awe

    path = golden_paths("pc_real_fold.npz")[0]
    par, z, wins = load(path)
    win, wdat = wins[0][1].copy(), wins[0][2]
    win[0, :3] += 50.0
    with pytest.raises(awe.AweError, match="no full-cloud point"):
        awe.cloud_merge(z["cloud"], [(win, wdat)])


def _bindir():
    import wavefield_imaging_gb300 as awe
    from wavefield_imaging_gb300 import build as awe_build

    awe.lib()
    return awe_build.build_programs()


def test_cloud_programs_are_installed():
    import os

    from wavefield_imaging_gb300 import build as awe_build

    bindir = _bindir()
    for name in awe_build.CLOUD_PROGRAM_NAMES:
        assert os.access(os.path.join(bindir, name), os.X_OK), name


@pytest.mark.gpu
@pytest.mark.parametrize("path", CLOUD, ids=lambda p: p.split("/")[-1][:-4])
def test_cloud_programs_reproduce_reference_files(path, tmp_path):
    """sfbycloudwin3d per orbit stretch, then sfbycloudmerge3d over the
    windows, run as the reference's programs are run; files equal the
    fixtures bit for bit."""
    import os
    import subprocess

    from wavefield_imaging_gb300 import rsf

    bindir = _bindir()
    par, z, wins = load(path)
    cloud = z["cloud"]
    rsf.write(str(tmp_path / "cloud.rsf"), cloud, [(9, 0, 1), (cloud.shape[0], 0, 1)])
    data = window_data(par, z)
    rsf.write(str(tmp_path / "dat.rsf"), data, [(cloud.shape[0], 0, 1), (data.shape[0], 0, 1)])
    cws, dws = [], []
    for k, (orb, win, wdat) in enumerate(wins):
        rsf.write(str(tmp_path / ("oo%d.rsf" % k)), orb, [(9, 0, 1), (orb.shape[0], 0, 1)])
        cw, dw = tmp_path / ("cw%d.rsf" % k), tmp_path / ("dw%d.rsf" % k)
        with open(tmp_path / "cloud.rsf") as fi, open(cw, "w") as fo:
            r = subprocess.run([os.path.join(bindir, "sfbycloudwin3d"), "oo=%s" % (tmp_path / ("oo%d.rsf" % k)),
                                "dat=%s" % (tmp_path / "dat.rsf"), "dout=%s" % dw, "apt=%g" % par["apt"]],
                               stdin=fi, stdout=fo, stderr=subprocess.PIPE, timeout=120)
        assert r.returncode == 0, r.stderr.decode()
        c, hc = rsf.read(str(cw))
        d, hd = rsf.read(str(dw))
        np.testing.assert_array_equal(c, win)
        np.testing.assert_array_equal(d if par["complex"] else d.real, wdat)
        if not par["complex"]:
            rsf.write(str(dw), wdat, [(wdat.shape[1], 0, 1), (wdat.shape[0], 0, 1)])
        cws.append(str(cw))
        dws.append(str(dw))
    out = tmp_path / "merged.rsf"
    with open(out, "w") as fo:
        r = subprocess.run([os.path.join(bindir, "sfbycloudmerge3d"), *cws, *dws, "all=%s" % (tmp_path / "cloud.rsf"),
                            "norm=%s" % ("y" if par["norm"] else "n")], stdin=subprocess.DEVNULL, stdout=fo,
                           stderr=subprocess.PIPE, timeout=120)
    assert r.returncode == 0, r.stderr.decode()
    m, hm = rsf.read(str(out))
    np.testing.assert_array_equal(m, z["merged"])
    assert int(hm["n1"]) == cloud.shape[0]
