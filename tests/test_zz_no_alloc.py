"""awe_forward2d_noalloc: 2D forward modelling for callers that cannot
allocate device memory (a framework-owned memory pool, graph capture, a
plug-in with a fixed device footprint).  Its scratch is one static device
array; these tests call it through the C-ABI with caller-owned device
buffers and compare with awe_forward, which allocates its own.

Collected last (file name) so a run that stops at the first failure has run
every other test first."""
import ctypes as C

import numpy as np
import pytest

import wavefield_imaging_gb300 as awe
from helpers import rel_l2

TOL = 1e-5  # rel-L2, the tolerance of the other parity tests


def _case(seed=5):
    rng = np.random.default_rng(seed)
    nz, nx, nt = 120, 150, 500
    vel = np.full((nx, nz), 168.0, np.float32)
    vel[:, :30] = 300.0
    vel[:, 90:] = 110.0 + 4.0 * rng.random((nx, nz - 90)).astype(np.float32)
    t = np.arange(nt) * 0.005 - 0.3
    a = (np.pi * 5.0 * t) ** 2
    wav = ((1 - 2 * a) * np.exp(-a)).astype(np.float32)
    sou = np.array([[0.5 * (nx - 1) * 5.0, 160.0]], np.float32)
    rec = np.stack([np.linspace(10.0, (nx - 2) * 5.0, 40), np.full(40, 150.0)], 1).astype(np.float32)
    desc = awe.make_desc(2, (nz, nx), (5.0, 5.0), (0.0, 0.0), nt, 0.005, nb=24, fdorder=8, dabc=1, expl=1)
    return desc, vel, wav, sou, rec


def _fp(t):
    return C.c_void_p(t.data_ptr())


def _lib():
    L = awe.lib()
    L.awe_forward2d_noalloc.argtypes = [C.POINTER(awe.Desc), C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                        C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.awe_forward2d_noalloc.restype = C.c_int
    return L


def test_noalloc_rejects_sizes_beyond_the_static_scratch():
    L = _lib()
    desc = awe.make_desc(2, (1200, 1200), (5.0, 5.0), (0.0, 0.0), 10, 0.005, nb=20, fdorder=8, dabc=1)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    st = L.awe_forward2d_noalloc(C.byref(desc), dummy, dummy, 1, 1, dummy, 1, dummy, dummy, None)
    assert st == 1
    assert b"static scratch" in L.awe_last_error()


@pytest.mark.gpu
def test_noalloc_matches_awe_forward_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    L = _lib()
    desc, vel, wav, sou, rec = _case()
    with awe.Plan(desc) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        ref = p.forward(wav)

    d_vel = torch.from_numpy(vel).cuda()
    d_wav = torch.from_numpy(wav).cuda()
    d_sou = torch.from_numpy(sou).cuda()
    d_rec = torch.from_numpy(rec).cuda()
    for call in range(2):
        d_dat = torch.full(ref.shape, float("nan"), dtype=torch.float32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        st = L.awe_forward2d_noalloc(C.byref(desc), _fp(d_vel), _fp(d_wav), 1, sou.shape[0], _fp(d_sou),
                                     rec.shape[0], _fp(d_rec), _fp(d_dat), C.c_void_p(stream))
        assert st == 0, L.awe_last_error()
        torch.cuda.synchronize()
        out = d_dat.cpu().numpy()
        assert np.isfinite(out).all(), "call %d left unwritten samples" % call
        assert rel_l2(out, ref) <= TOL, "call %d" % call
        assert np.abs(out).max() > 0
