"""awe_forward2d_noalloc: 2D forward modelling for callers that cannot
allocate device memory (a framework-owned memory pool, graph capture, a
plug-in with a fixed device footprint).  Its scratch is one static device
array; these tests call it through the C-ABI with caller-owned device
buffers and compare with awe_forward, which allocates its own.

Collected last (file name) so a run that stops at the first failure has run
every other test first.  Besides the basic comparison, the options of the
path are each compared once: free surface, one wavelet per source, decimated
traces, no sponge, a source inside the sponge band, receivers on the edge and
outside the grid; under AWE_EXACT the output must equal awe_forward's bit for
bit."""
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


def _variant(kind):
    rng = np.random.default_rng(11)
    nz, nx, nt = 96, 110, 300
    vel = (160.0 + 20.0 * rng.random((nx, nz))).astype(np.float32)
    vel[:, :20] = 300.0
    t = np.arange(nt) * 0.005 - 0.2
    a = (np.pi * 5.0 * t) ** 2
    wav = ((1 - 2 * a) * np.exp(-a)).astype(np.float32)
    sou = np.array([[0.5 * (nx - 1) * 5.0, 140.0]], np.float32)
    rec = np.stack([np.linspace(10.0, (nx - 2) * 5.0, 30), np.full(30, 120.0)], 1).astype(np.float32)
    opts = dict(nb=20, fdorder=8, dabc=1, expl=1, precision=awe.EXACT)
    ncs = 1
    if kind == "free_surface":
        opts["fsrf"] = 1
    elif kind == "wavelet_per_source":
        sou = np.array([[100.0, 140.0], [300.0, 200.0], [420.0, 90.0]], np.float32)
        wav = np.stack([wav, 0.5 * wav, -wav], 1).astype(np.float32)
        opts["expl"] = 0
        ncs = 3
    elif kind == "decimated":
        opts["jdata"] = 3
    elif kind == "no_sponge":
        opts["dabc"] = 0
    elif kind == "source_in_band":
        sou = np.array([[-40.0, 150.0]], np.float32)  # 8 cells outside the model, inside the 20-cell band
    elif kind == "edge_receivers":
        rec = np.concatenate([rec, np.array([[0.0, 0.0], [(nx - 1) * 5.0, (nz - 1) * 5.0], [-1e4, 50.0],
                                             [50.0, 1e4]], np.float32)])
    elif kind == "fast":
        opts["precision"] = awe.FAST
    desc = awe.make_desc(2, (nz, nx), (5.0, 5.0), (0.0, 0.0), nt, 0.005, **opts)
    return desc, vel, wav, ncs, sou, rec


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["free_surface", "wavelet_per_source", "decimated", "no_sponge", "source_in_band",
                                  "edge_receivers", "fast"])
def test_noalloc_options_match_awe_forward(kind):
    torch = pytest.importorskip("torch")
    L = _lib()
    desc, vel, wav, ncs, sou, rec = _variant(kind)
    with awe.Plan(desc) as p:
        p.set_model(vel)
        p.set_geometry(sou, rec)
        ref = p.forward(wav)
    assert np.abs(ref).max() > 0
    d_vel, d_wav = torch.from_numpy(vel).cuda(), torch.from_numpy(wav).cuda()
    d_sou, d_rec = torch.from_numpy(sou).cuda(), torch.from_numpy(rec).cuda()
    for call in range(2):
        d_dat = torch.full(ref.shape, float("nan"), dtype=torch.float32, device="cuda")
        st = L.awe_forward2d_noalloc(C.byref(desc), _fp(d_vel), _fp(d_wav), ncs, sou.shape[0], _fp(d_sou),
                                     rec.shape[0], _fp(d_rec), _fp(d_dat),
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == 0, L.awe_last_error()
        torch.cuda.synchronize()
        out = d_dat.cpu().numpy()
        if desc.precision == awe.EXACT:
            np.testing.assert_array_equal(out, ref, err_msg="%s, call %d" % (kind, call))
        else:
            assert rel_l2(out, ref) <= TOL, "call %d" % call


def test_noalloc_rejects_what_it_leaves_out():
    L = _lib()
    dummy = C.c_void_p(16)  # never dereferenced: the checks come first
    for field, value, status in (("jdata", -1, 1), ("precision", 7, 1), ("bnds", 1, 4), ("refl", 1, 4),
                                 ("hybrid", 1, 4), ("ndim", 3, 4)):
        desc = awe.make_desc(2, (60, 60), (5.0, 5.0), (0.0, 0.0), 10, 0.005, nb=8, fdorder=8, dabc=1)
        setattr(desc, field, value)
        if field == "ndim":
            desc.n[2] = 10
        st = L.awe_forward2d_noalloc(C.byref(desc), dummy, dummy, 1, 1, dummy, 1, dummy, dummy, None)
        assert st == status, (field, st, L.awe_last_error())
