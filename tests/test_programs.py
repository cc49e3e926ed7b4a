"""The drop-in RSF programs (sfAWEFD{cart,spher}{2D,3D}gpu, sfAWEFDcart{2D,3D}cpu)
run as the reference's are run: RSF inputs on the command line and standard
input, data on standard output, wavefield to wfl=.  GPU cases feed each golden
fixture's inputs to the program with precision=exact and compare the written
data and wavefield files with the reference's outputs bit for bit; CPU cases
cover argument handling, which needs no device."""
import os
import subprocess

import numpy as np
import pytest

from helpers import golden_paths, load_golden

import wavefield_imaging_gb300 as awe
from wavefield_imaging_gb300 import rsf
from wavefield_imaging_gb300 import build as awe_build

PROGRAM_OF_KIND = {"cart2d": "sfAWEFDcart2Dgpu", "cart3d": "sfAWEFDcart3Dgpu", "polar2d": "sfAWEFDspher2Dgpu",
                   "spher3d": "sfAWEFDspher3Dgpu", "dyncart2d": "sfDYNAWEFDcart2Dgpu"}


@pytest.fixture(scope="module")
def bindir():
    awe.lib()  # builds libawe.so when missing
    return awe_build.build_programs()


def yn(v):
    return "y" if v else "n"


def write_inputs(tmp, par, a):
    nd = len(par["n"])
    rsf.write(str(tmp / "vel.rsf"), a["vel"], [(n, o, d) for n, o, d in zip(par["n"], par["o"], par["d"])])
    wav = a["wav"]
    ncs = 1 if wav.ndim == 1 else wav.shape[1]
    rsf.write(str(tmp / "wav.rsf"), wav.reshape(par["nt"], ncs), [(ncs, 0.0, 1.0), (par["nt"], 0.0, par["dt"])])
    if par.get("kind") == "dyncart2d":  # position tables: n2 points per step, n3 rows
        rsf.write(str(tmp / "sou.rsf"), a["sou"], [(nd, 0.0, 1.0), (par["ns"], 0.0, 1.0), (par["nst"], 0.0, 1.0)])
        rsf.write(str(tmp / "rec.rsf"), a["rec"], [(nd, 0.0, 1.0), (par["nr"], 0.0, 1.0), (par["nrt"], 0.0, 1.0)])
    else:
        rsf.write(str(tmp / "sou.rsf"), a["sou"], [(nd, 0.0, 1.0), (a["sou"].shape[0], 0.0, 1.0)])
        rsf.write(str(tmp / "rec.rsf"), a["rec"], [(nd, 0.0, 1.0), (a["rec"].shape[0], 0.0, 1.0)])
    args = ["vel=" + str(tmp / "vel.rsf"), "sou=" + str(tmp / "sou.rsf"), "rec=" + str(tmp / "rec.rsf")]
    for key in ("den", "rfl"):
        if key in a:
            rsf.write(str(tmp / (key + ".rsf")), a[key], [(n, o, d) for n, o, d in zip(par["n"], par["o"], par["d"])])
            args.append("%s=%s" % (key, tmp / (key + ".rsf")))
    return args


def run_program(bindir, name, tmp, args):
    out = tmp / "dat.rsf"
    with open(tmp / "wav.rsf", "rb") as fin, open(out, "wb") as fout:
        r = subprocess.run([os.path.join(bindir, name), *args, "wfl=" + str(tmp / "wfl.rsf")], stdin=fin,
                           stdout=fout, stderr=subprocess.PIPE, timeout=300)
    if r.returncode != 0:
        raise AssertionError("%s failed: %s" % (name, r.stderr.decode()))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("path", golden_paths("A_*.npz"), ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_program_matches_reference_outputs(bindir, tmp_path, path):
    par, a = load_golden(path)
    args = write_inputs(tmp_path, par, a)
    jsnap = par.get("jsnap", 0)
    args += ["nb=%d" % par["nb"], "jdata=%d" % par.get("jdata", 1), "snap=" + yn(jsnap > 0),
             "bnds=" + yn(par.get("bnds", 0)), "free=" + yn(par.get("fsrf", 0)), "expl=" + yn(par.get("expl", 0)),
             "precision=exact"]
    if jsnap > 0:
        args.append("jsnap=%d" % jsnap)
    if par["kind"] == "cart2d":
        args.append("refl=" + yn(par.get("refl", 0)))
    out = run_program(bindir, PROGRAM_OF_KIND[par["kind"]], tmp_path, args)
    dat, hdr = rsf.read(str(out))
    np.testing.assert_array_equal(dat.reshape(a["dat"].shape), a["dat"])
    assert int(hdr["n1"]) == a["dat"].shape[1]
    if "snaps" in a:
        wfl, _ = rsf.read(str(tmp_path / "wfl.rsf"))
        np.testing.assert_array_equal(wfl.ravel(), a["snaps"].ravel())


@pytest.mark.gpu
@pytest.mark.parametrize("path", golden_paths("c*.npz"), ids=lambda p: os.path.basename(p)[:-4])
def test_cpu_program_matches_reference_outputs(bindir, tmp_path, path):
    par, a = load_golden(path)
    args = write_inputs(tmp_path, par, a)
    jsnap = par.get("jsnap", 0)
    args += ["fdorder=%d" % par["fdorder"], "optfd=" + yn(par.get("optfd", 0)), "dabc=" + yn(par.get("dabc", 0)),
             "free=" + yn(par.get("fsrf", 0)), "hybridbc=" + yn(par.get("hybrid", 0)),
             "expl=" + yn(par.get("expl", 0)), "snap=" + yn(jsnap > 0), "bnds=" + yn(par.get("bnds", 0)),
             "precision=exact"]
    if par.get("nb", -1) >= 0:
        args.append("nb=%d" % par["nb"])
    if jsnap > 0:
        args.append("jsnap=%d" % jsnap)
    args += ["%s=%s" % (k, v) for k, v in par.get("win", {}).items()]  # snapshot window
    name = "sfAWEFDcart%dDcpu" % len(par["n"])
    out = run_program(bindir, name, tmp_path, args)
    dat, _ = rsf.read(str(out))
    np.testing.assert_array_equal(dat.reshape(a["dat"].shape), a["dat"])
    if "snaps" in a:
        wfl, _ = rsf.read(str(tmp_path / "wfl.rsf"))
        np.testing.assert_array_equal(wfl.ravel(), a["snaps"].ravel())


@pytest.mark.gpu
def test_cpu_program_snapshot_window_header_and_errors(bindir, tmp_path):
    """The window's axes in the wavefield header (sf_maxa(nq, oq, dq),
    MAWEFDcart2Dcpu.c:194-204), and a window that leaves the padded grid or
    an adj=y window whose size differs from the model's stops with an error."""
    par, a = load_golden(golden_paths("c2d_o8_window.npz")[0])
    base = write_inputs(tmp_path, par, a) + ["fdorder=8", "dabc=y", "expl=y", "nb=%d" % par["nb"], "snap=y",
                                             "jsnap=%d" % par["jsnap"]]
    run_program(bindir, "sfAWEFDcart2Dcpu", tmp_path, base + ["%s=%s" % kv for kv in par["win"].items()])
    _, hdr = rsf.read(str(tmp_path / "wfl.rsf"))
    w = par["win"]
    assert [int(hdr["n1"]), int(hdr["n2"]), int(hdr["n3"])] == [w["nqz"], w["nqx"], (par["nt"] - 1) // 50 + 1]
    assert [float(hdr["o1"]), float(hdr["o2"]), float(hdr["d1"]), float(hdr["d2"])] == [w["oqz"], w["oqx"], w["dqz"],
                                                                                        w["dqx"]]
    for bad, msg in ((["oqz=-100"], "outside the padded grid"), (["nqx=40", "dqx=15"], "outside the padded grid"),
                     (["adj=y", "kt=10", "nqz=20"], "must equal the model's")):
        with pytest.raises(AssertionError, match=msg):
            run_program(bindir, "sfAWEFDcart2Dcpu", tmp_path, base + bad)


def _run_bare(bindir, name, args):
    return subprocess.run([os.path.join(bindir, name), *args], stdin=subprocess.DEVNULL, capture_output=True,
                          timeout=60)


@pytest.mark.parametrize("name,arg,msg", [("sfAWEFDcart2Dgpu", "adj=y", "adj=y"),
                                          ("sfDYNAWEFDcart2Dgpu", "jdata=2", "jdata must be 1"),
                                          ("sfAWEFDcart2Dcpu", "sinc=y", "sinc=y")])
def test_unsupported_options_stop_with_an_error(bindir, name, arg, msg):
    r = _run_bare(bindir, name, [arg])
    assert r.returncode == 1
    assert msg in r.stderr.decode()


def test_missing_input_stops_with_an_error(bindir, tmp_path):
    r = _run_bare(bindir, "sfAWEFDspher2Dgpu", ["vel=" + str(tmp_path / "absent.rsf")])
    assert r.returncode == 1
    assert r.stderr


def test_every_program_name_is_installed(bindir):
    for name in awe_build.PROGRAM_NAMES:
        assert os.access(os.path.join(bindir, name), os.X_OK), name
    r = _run_bare(bindir, "awe_prog", [])
    assert r.returncode == 1


@pytest.mark.gpu
def test_cpu_program_adjoint_back_injection_image(bindir, tmp_path):
    """adj=y: the traces on standard input go back into the model at the
    receivers, reversed in time; the image is the wavefield at step nt-kt.
    Checked bit for bit (precision=exact) against the oracle run with the same
    back-injection (sources at the receivers, reversed traces, snapshot at
    nt-kt)."""
    from oracle import oracle

    par, a = load_golden(golden_paths("c2d_o8_sponge.npz")[0])
    nt, kt = par["nt"], 40
    data = a["dat"]  # [nt][nr] traces of the golden run, used as the recorded data
    nd = len(par["n"])
    rsf.write(str(tmp_path / "vel.rsf"), a["vel"], [(n, o, d) for n, o, d in zip(par["n"], par["o"], par["d"])])
    rsf.write(str(tmp_path / "sou.rsf"), a["sou"], [(nd, 0.0, 1.0), (a["sou"].shape[0], 0.0, 1.0)])
    rsf.write(str(tmp_path / "rec.rsf"), a["rec"], [(nd, 0.0, 1.0), (a["rec"].shape[0], 0.0, 1.0)])
    rsf.write(str(tmp_path / "wav.rsf"), data, [(data.shape[1], 0.0, 1.0), (nt, 0.0, par["dt"])])
    args = ["vel=" + str(tmp_path / "vel.rsf"), "sou=" + str(tmp_path / "sou.rsf"), "rec=" + str(tmp_path / "rec.rsf"),
            "adj=y", "kt=%d" % kt, "expl=n", "fdorder=8", "dabc=y", "nb=%d" % par["nb"], "precision=exact"]
    out = run_program(bindir, "sfAWEFDcart2Dcpu", tmp_path, args)
    img, hdr = rsf.read(str(out))
    assert (int(hdr["n1"]), int(hdr["n2"])) == (par["n"][0], par["n"][1])
    steps = nt - kt + 1
    back = np.ascontiguousarray(data[::-1][:steps])
    p2 = dict(par, nt=steps, jsnap=nt - kt, expl=0, bnds=0)
    _, snaps = oracle.cart_cpu(p2, a["vel"], back, a["rec"], a["rec"][:1])
    np.testing.assert_array_equal(img.ravel(), snaps[-1].ravel())


@pytest.mark.gpu
def test_cpu_program_adjoint_expl_snapshots(bindir, tmp_path):
    """sfAWEFDcart2Dcpu adj=y expl=y snap=y bnds=y: the one-component wavelet,
    reversed in time, goes in at the sources; the padded frames of the steps
    it % jsnap == 0 up to the image step go to wfl and the image is the model
    window of step nt-kt (here not a multiple of jsnap, so the engine delivers
    every frame).  Bit for bit against the oracle."""
    from oracle import oracle

    par, a = load_golden(golden_paths("c2d_o8_sponge.npz")[0])
    nt, kt, jsnap = par["nt"], 37, 11
    args = write_inputs(tmp_path, par, a)
    args += ["adj=y", "kt=%d" % kt, "expl=y", "snap=y", "bnds=y", "jsnap=%d" % jsnap, "fdorder=8", "dabc=y",
             "nb=%d" % par["nb"], "precision=exact"]
    out = run_program(bindir, "sfAWEFDcart2Dcpu", tmp_path, args)
    img, hdr = rsf.read(str(out))
    wfl, whdr = rsf.read(str(tmp_path / "wfl.rsf"))
    img_it = nt - kt
    assert img_it % jsnap != 0
    steps = img_it + 1
    back = np.ascontiguousarray(a["wav"][::-1][:steps])
    _, frames = oracle.cart_cpu(dict(par, nt=steps, jsnap=jsnap, expl=1, bnds=1), a["vel"], back, a["sou"],
                                a["rec"][:1])
    assert int(whdr["n3"]) == frames.shape[0] == img_it // jsnap + 1
    np.testing.assert_array_equal(wfl.ravel(), frames.ravel())
    _, last = oracle.cart_cpu(dict(par, nt=steps, jsnap=img_it, expl=1, bnds=0), a["vel"], back, a["sou"],
                              a["rec"][:1])
    assert (int(hdr["n1"]), int(hdr["n2"])) == (par["n"][0], par["n"][1])
    np.testing.assert_array_equal(img.ravel(), last[-1].ravel())


@pytest.mark.gpu
@pytest.mark.parametrize("fixture", ["c3d_o8_sponge.npz", "c3d_o4_free_den.npz"])
def test_cpu3d_program_adjoint_is_reversed_forward(bindir, tmp_path, fixture):
    """sfAWEFDcart3Dcpu adj=y injects the wavelet reversed in time at the
    sources and otherwise runs as forward (traces on standard output): the
    outputs equal those of adj=n on the reversed wavelet, bit for bit."""
    par, a = load_golden(golden_paths(fixture)[0])
    common = ["expl=%s" % yn(par["expl"]), "fdorder=%d" % par["fdorder"], "dabc=%s" % yn(par["dabc"]),
              "free=%s" % yn(par["fsrf"]), "nb=%d" % par["nb"], "precision=exact"]
    fwd_dir, adj_dir = tmp_path / "fwd", tmp_path / "adj"
    fwd_dir.mkdir()
    adj_dir.mkdir()
    args = write_inputs(adj_dir, par, a) + common
    adj_out = run_program(bindir, "sfAWEFDcart3Dcpu", adj_dir, args + ["adj=y"])
    rev = dict(a, wav=np.ascontiguousarray(a["wav"][::-1]))
    args = write_inputs(fwd_dir, par, rev) + common
    fwd_out = run_program(bindir, "sfAWEFDcart3Dcpu", fwd_dir, args)
    d_adj, h_adj = rsf.read(str(adj_out))
    d_fwd, h_fwd = rsf.read(str(fwd_out))
    assert int(h_adj["n2"]) == par["nt"]
    np.testing.assert_array_equal(d_adj, d_fwd)
    assert np.abs(d_adj).max() > 0


def _spher_adj_inputs(tmp, par, a):
    rsf.write(str(tmp / "vel.rsf"), a["vel"], [(n, o, d) for n, o, d in zip(par["n"], par["o"], par["d"])])
    rsf.write(str(tmp / "sou.rsf"), a["sou"], [(3, 0.0, 1.0), (a["sou"].shape[0], 0.0, 1.0)])
    rsf.write(str(tmp / "rec.rsf"), a["rec"], [(3, 0.0, 1.0), (a["rec"].shape[0], 0.0, 1.0)])
    data = a["data"]
    rsf.write(str(tmp / "wav.rsf"), data, [(data.shape[1], 0.0, 1.0), (par["nt"], 0.0, par["dt"])])
    return ["vel=" + str(tmp / "vel.rsf"), "sou=" + str(tmp / "sou.rsf"), "rec=" + str(tmp / "rec.rsf")]


@pytest.mark.gpu
@pytest.mark.parametrize("path", golden_paths("Aadj_*.npz"), ids=lambda p: os.path.basename(p)[:-4])
def test_spherical_program_adjoint_matches_reference_outputs(bindir, tmp_path, path):
    """sfAWEFDspher3Dgpu adj=y: the traces on standard input go back in at the
    receivers, reversed in time; the image (model window after step nt-kt)
    and the frames of snap=y equal, bit for bit, what the reference's own
    kernels give through the host emulation of the program's adj branch."""
    par, a = load_golden(path)
    jsnap = par.get("jsnap", 0)
    args = _spher_adj_inputs(tmp_path, par, a)
    args += ["adj=y", "kt=%d" % par["kt"], "nb=%d" % par["nb"], "snap=" + yn(jsnap > 0),
             "bnds=" + yn(par.get("bnds", 0)), "free=" + yn(par.get("fsrf", 0)), "precision=exact"]
    if jsnap > 0:
        args.append("jsnap=%d" % jsnap)
    out = run_program(bindir, "sfAWEFDspher3Dgpu", tmp_path, args)
    img, hdr = rsf.read(str(out))
    assert [int(hdr["n%d" % k]) for k in (1, 2, 3)] == list(par["n"])
    np.testing.assert_array_equal(img.ravel(), a["image"].ravel())
    if "snaps" in a:
        wfl, whdr = rsf.read(str(tmp_path / "wfl.rsf"))
        assert int(whdr["n4"]) == a["snaps"].shape[0]
        np.testing.assert_array_equal(wfl.ravel(), a["snaps"].ravel())


def test_spherical_program_adjoint_needs_a_reachable_image_step(bindir, tmp_path):
    par, a = load_golden(golden_paths("Aadj_spher3d_snap.npz")[0])
    args = _spher_adj_inputs(tmp_path, par, a) + ["adj=y", "kt=0", "nb=%d" % par["nb"]]
    with open(tmp_path / "wav.rsf", "rb") as fin:
        r = subprocess.run([os.path.join(bindir, "sfAWEFDspher3Dgpu"), *args], stdin=fin, capture_output=True,
                           timeout=60)
    assert r.returncode == 1
    assert b"kt must be in [1, nt]" in r.stderr
