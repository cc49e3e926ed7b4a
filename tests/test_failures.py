"""Failure detection.  The reference stops with sf_error and checks every CUDA
call (sf_check_gpu_error, MAWEFDcart2Dgpu.cu:23-27); the engine returns a
status instead, and the drop-in programs print it and exit 1.  Failures are
made on the host or by a limit, never by faulting the GPU:

* CPU: truncated, missing or empty RSF inputs make the programs exit 1
  with the reason, before any device work;
* GPU: a per-plan device-memory cap (AWE_DEVICE_BYTES_LIMIT) turns plan
  creation into AWE_ERR_NOMEM and leaks nothing; a pipeline wait limit of
  zero polls (AWE_PIPELINE_SPIN_LIMIT) makes every first wait of the TMA
  step kernel give up, which the run reports as AWE_ERR_CUDA, and the GPU
  stays usable for the next plan."""
import os
import subprocess
import sys

import numpy as np
import pytest

import wavefield_imaging_gb300 as awe
from wavefield_imaging_gb300 import build as awe_build
from wavefield_imaging_gb300 import rsf

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bindir():
    awe.lib()
    return awe_build.build_programs()


def _inputs(tmp, nz=40, nx=44, nt=50):
    vel = np.full((nx, nz), 168.0, np.float32)
    rsf.write(str(tmp / "vel.rsf"), vel, [(nz, 0.0, 5.0), (nx, 0.0, 5.0)])
    wav = np.sin(np.arange(nt) * 0.3).astype(np.float32).reshape(nt, 1)
    rsf.write(str(tmp / "wav.rsf"), wav, [(1, 0.0, 1.0), (nt, 0.0, 0.005)])
    sou = np.array([[100.0, 60.0]], np.float32)
    rec = np.array([[50.0, 50.0], [120.0, 50.0]], np.float32)
    rsf.write(str(tmp / "sou.rsf"), sou, [(2, 0.0, 1.0), (1, 0.0, 1.0)])
    rsf.write(str(tmp / "rec.rsf"), rec, [(2, 0.0, 1.0), (2, 0.0, 1.0)])
    return ["vel=" + str(tmp / "vel.rsf"), "sou=" + str(tmp / "sou.rsf"), "rec=" + str(tmp / "rec.rsf"),
            "fdorder=8", "nb=8"]


def _run(bindir, tmp, args, stdin_name="wav.rsf"):
    with open(tmp / stdin_name, "rb") as fin, open(tmp / "dat.rsf", "wb") as fout:
        return subprocess.run([os.path.join(bindir, "sfAWEFDcart2Dcpu"), *args], stdin=fin, stdout=fout,
                              stderr=subprocess.PIPE, timeout=120)


def _truncate(path, keep):
    with open(path, "r+b") as f:
        f.truncate(keep)


def test_truncated_velocity_stops_with_short_read(bindir, tmp_path):
    args = _inputs(tmp_path)
    _truncate(str(tmp_path / "vel.rsf") + "@", 4 * 100)
    r = _run(bindir, tmp_path, args)
    assert r.returncode == 1
    assert b"short read (vel)" in r.stderr


def test_truncated_wavelet_stops_with_short_read(bindir, tmp_path):
    args = _inputs(tmp_path)
    _truncate(str(tmp_path / "wav.rsf") + "@", 4 * 7)
    r = _run(bindir, tmp_path, args)
    assert r.returncode == 1
    assert b"short read (wavelet)" in r.stderr


def test_truncated_receivers_stop_with_short_read(bindir, tmp_path):
    args = _inputs(tmp_path)
    _truncate(str(tmp_path / "rec.rsf") + "@", 4 * 3)
    r = _run(bindir, tmp_path, args)
    assert r.returncode == 1
    assert b"short read (rec)" in r.stderr


def test_missing_velocity_file_is_an_error(bindir, tmp_path):
    args = _inputs(tmp_path)
    os.remove(tmp_path / "vel.rsf")
    r = _run(bindir, tmp_path, args)
    assert r.returncode == 1
    assert r.stderr


def test_empty_standard_input_is_an_error(bindir, tmp_path):
    args = _inputs(tmp_path)
    (tmp_path / "empty.rsf").write_bytes(b"")
    r = _run(bindir, tmp_path, args, stdin_name="empty.rsf")
    assert r.returncode == 1
    assert r.stderr


def _probe(code, env):
    """Run `code` in a fresh interpreter with extra environment variables (the
    limits are read when a plan is created) and return its last output line."""
    e = dict(os.environ, **env)
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=e, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout.strip().splitlines()[-1]


_CAP_CODE = r'''
import sys; sys.path.insert(0, ".")
import torch, wavefield_imaging_gb300 as awe
torch.cuda.init()
desc = awe.make_desc(3, (200, 200, 200), (5.0, 5.0, 5.0), (0.0, 0.0, 0.0), 10, 0.005, nb=16, fdorder=8, dabc=1)
try:  # one attempt first, so one-time context set-up is not counted
    awe.Plan(desc).close()
except awe.AweError:
    pass
free0 = torch.cuda.mem_get_info()[0]
codes = []
for _ in range(20):
    try:
        awe.Plan(desc).close()
        codes.append(0)
    except awe.AweError as e:
        codes.append(e.status)
        msg = str(e)
free1 = torch.cuda.mem_get_info()[0]
print(codes[0], codes[-1], free0 - free1, "AWE_DEVICE_BYTES_LIMIT" in msg)
'''


@pytest.mark.gpu
def test_device_memory_cap_gives_nomem_and_leaks_nothing():
    # one 232^3 field is 50 MB: a 64 MB cap fails at the second field
    out = _probe(_CAP_CODE, {"AWE_DEVICE_BYTES_LIMIT": str(64 << 20)})
    first, last, leaked, named = out.split()
    assert int(first) == 3 and int(last) == 3  # AWE_ERR_NOMEM
    assert named == "True"
    assert abs(int(leaked)) < (8 << 20)  # twenty failed creations hold nothing


_TIMEOUT_CODE = r'''
import os, sys; sys.path.insert(0, ".")
import numpy as np, wavefield_imaging_gb300 as awe
n, nt = (72, 40, 40), 30
vel = np.full(n[::-1], 168.0, np.float32)
wav = np.sin(np.arange(nt) * 0.3).astype(np.float32)
sou = np.array([[100.0, 100.0, 150.0]], np.float32)
rec = np.array([[60.0, 60.0, 50.0]], np.float32)
desc = awe.make_desc(3, n, (5.0, 5.0, 5.0), (0.0, 0.0, 0.0), nt, 0.005, nb=8, fdorder=8, dabc=1, expl=1)
status, msg = 0, ""
with awe.Plan(desc) as p:
    assert p.step_kernel == "tma3d"
    p.set_model(vel); p.set_geometry(sou, rec)
    try:
        p.forward(wav)
    except awe.AweError as e:
        status, msg = e.status, str(e)
os.environ.pop("AWE_PIPELINE_SPIN_LIMIT")
with awe.Plan(desc) as p:
    p.set_model(vel); p.set_geometry(sou, rec)
    d = p.forward(wav)
print(status, "timed out" in msg, bool(np.isfinite(d).all() and np.abs(d).max() > 0))
'''


@pytest.mark.gpu
def test_pipeline_wait_timeout_is_reported_and_the_gpu_stays_usable():
    out = _probe(_TIMEOUT_CODE, {"AWE_PIPELINE_SPIN_LIMIT": "0"})
    status, named, ok = out.split()
    assert int(status) == 2  # AWE_ERR_CUDA
    assert named == "True"
    assert ok == "True"  # a new plan without the limit runs normally


_SPH_TIMEOUT_CODE = r'''
import os, sys; sys.path.insert(0, ".")
import numpy as np, wavefield_imaging_gb300 as awe
n, nt = (40, 30, 28), 40
d = (0.005, 1.5e-6, 1.5e-6)
o = (3387.0, np.pi / 2 - 15 * d[1], -14 * d[2])
vel = np.full(n[::-1], 0.168, np.float32)
wav = np.sin(np.arange(nt) * 0.3).astype(np.float32)
sou = np.array([[o[0] + 25 * d[0], o[2] + 14 * d[2], o[1] + 15 * d[1]]], np.float32)
rec = np.array([[o[0] + 28 * d[0], o[2] + 10 * d[2], o[1] + 12 * d[1]]], np.float32)
desc = awe.make_desc(3, n, d, o, nt, 0.005, coords=awe.SPHER, scheme=awe.SCHEME_GPU, nb=6, precision=awe.FAST)
res = []
with awe.Plan(desc) as p:
    assert p.step_kernel == "tma_sph"
    p.set_model(vel); p.set_geometry(sou, rec)
    for call in ("forward", "gradient"):
        try:
            if call == "forward":
                p.forward(wav)
            else:
                p.gradient(wav, np.zeros((nt, 1), np.float32))
            res.append("0")
        except awe.AweError as e:
            res.append("%d:%s" % (e.status, "timed out" in str(e)))
os.environ.pop("AWE_PIPELINE_SPIN_LIMIT")
with awe.Plan(desc) as p:
    p.set_model(vel); p.set_geometry(sou, rec)
    dat = p.forward(wav)
    g, J = p.gradient(wav, np.zeros((nt, 1), np.float32))
print(" ".join(res), bool(np.isfinite(dat).all() and np.abs(dat).max() > 0), bool(np.isfinite(g).all() and J > 0))
'''


@pytest.mark.gpu
def test_spherical_pipeline_wait_timeouts_are_reported():
    """The TMA-staged spherical step and adjoint kernels under a zero wait
    limit: the forward and the gradient both report AWE_ERR_CUDA with the
    timeout message (their CTAs drain their copies in flight and leave), and
    a new plan without the limit runs both normally."""
    out = _probe(_SPH_TIMEOUT_CODE, {"AWE_PIPELINE_SPIN_LIMIT": "0"})
    fwd, grad, ok_fwd, ok_grad = out.split()
    assert fwd == "2:True" and grad == "2:True"
    assert ok_fwd == "True" and ok_grad == "True"
