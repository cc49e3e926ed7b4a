"""Python front end of libawe.so (include/awe.h) over ctypes.

The engine runs only on the GPU through its own CUDA kernels; there is no CPU
fallback.  Importing works without a GPU; creating a plan without one raises
``AweError`` (status AWE_ERR_NODEVICE).  A missing library raises
immediately with the build command.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libawe.so")

CART, SPHER = 0, 1
SCHEME_GPU, SCHEME_CPU = 0, 1
FAST, EXACT = 0, 1

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "unsupported",
          5: "no CUDA device", 6: "call out of order"}


class AweError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class Desc(C.Structure):
    _fields_ = [
        ("coords", C.c_int), ("scheme", C.c_int), ("ndim", C.c_int),
        ("n", C.c_int * 3), ("d", C.c_float * 3), ("o", C.c_float * 3),
        ("nb", C.c_int), ("nt", C.c_int), ("dt", C.c_float),
        ("fdorder", C.c_int), ("optfd", C.c_int), ("dabc", C.c_int), ("hybrid", C.c_int),
        ("fsrf", C.c_int), ("expl", C.c_int), ("refl", C.c_int), ("jdata", C.c_int),
        ("jsnap", C.c_int), ("bnds", C.c_int), ("precision", C.c_int),
    ]


class Info(C.Structure):
    _fields_ = [("npad", C.c_int * 3), ("nbpad", C.c_int), ("nsmp", C.c_int), ("nsnap", C.c_int),
                ("snap_elems", C.c_size_t), ("device_bytes", C.c_size_t), ("step_kernel", C.c_int)]


class Shot(C.Structure):
    _fields_ = [("x0", C.c_int), ("nx", C.c_int), ("ns", C.c_int), ("nr", C.c_int),
                ("sou", C.POINTER(C.c_float)), ("rec", C.POINTER(C.c_float))]


class BatchInfo(C.Structure):
    _fields_ = [("nshots", C.c_int), ("nsmp", C.c_int), ("total_samples", C.c_longlong), ("cells", C.c_longlong),
                ("tile_z", C.c_int), ("tile_x", C.c_int), ("grid", C.c_int), ("work_items", C.c_int),
                ("launches_per_forward", C.c_int)]


class GradOpts(C.Structure):
    _fields_ = [("ckpt_every", C.c_int), ("ckpt_format", C.c_int)]


CKPT_BF16, CKPT_FP32, CKPT_FP16, CKPT_BFP16 = 0, 1, 2, 3
# awe_move_mode: one row of positions per step / sfDYNAWEFDcart2Dgpu's entry k*(it+1)
MOVE_PER_STEP, MOVE_DYN = 0, 1
# awe_image_condition: zero-lag cross-correlation / Born adjoint
IMAGE_XCORR, IMAGE_BORN = 0, 1

SNAP_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_size_t)

_lib = None


def lib():
    """Load libawe.so (built in-tree by wavefield_imaging_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libawe.so not built: run `python -m wavefield_imaging_gb300.build` (%s)" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        vp, fp = C.c_void_p, C.POINTER(C.c_float)
        L.awe_version.restype = C.c_char_p
        L.awe_last_error.restype = C.c_char_p
        L.awe_status_string.restype = C.c_char_p
        L.awe_status_string.argtypes = [C.c_int]
        L.awe_plan_create.argtypes = [C.POINTER(Desc), C.c_int, C.POINTER(vp)]
        L.awe_plan_destroy.argtypes = [vp]
        L.awe_plan_info.argtypes = [vp, C.POINTER(Info)]
        L.awe_set_model.argtypes = [vp, fp, fp, fp]
        L.awe_set_geometry.argtypes = [vp, C.c_int, fp, C.c_int, fp]
        L.awe_forward.argtypes = [vp, fp, C.c_int, fp, fp]
        L.awe_forward_device.argtypes = [vp, vp, C.c_int, vp, vp, vp]
        L.awe_set_snapshot_callback.argtypes = [vp, SNAP_FN, vp]
        L.awe_synchronize.argtypes = [vp]
        L.awe_last_launch_count.argtypes = [vp]
        L.awe_last_launch_count.restype = C.c_longlong
        L.awe_profile_enable.argtypes = [vp, C.c_int]
        L.awe_profile_read.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
        L.awe_profile_read_kinds.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
        L.awe_batch_create.argtypes = [C.POINTER(Desc), C.c_int, C.POINTER(Shot), C.c_int, C.POINTER(vp)]
        L.awe_batch_destroy.argtypes = [vp]
        L.awe_batch_set_model.argtypes = [vp, fp]
        L.awe_batch_forward.argtypes = [vp, fp, fp]
        L.awe_batch_forward_device.argtypes = [vp, vp, vp, vp]
        L.awe_batch_tune.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.awe_batch_select.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.awe_batch_select.restype = C.c_int
        L.awe_batch_info.argtypes = [vp, C.POINTER(BatchInfo)]
        L.awe_batch_gradient.argtypes = [vp, fp, fp, C.POINTER(GradOpts), C.POINTER(C.c_double),
                                         C.POINTER(C.c_double)]
        for name in ("awe_batch_create", "awe_batch_destroy", "awe_batch_set_model", "awe_batch_forward",
                     "awe_batch_forward_device", "awe_batch_tune", "awe_batch_info", "awe_batch_gradient"):
            getattr(L, name).restype = C.c_int
        ip = C.POINTER(C.c_int)
        L.awe_set_shots.argtypes = [vp, C.c_int, ip, fp, ip, fp]
        L.awe_set_shots.restype = C.c_int
        L.awe_set_moving_geometry.argtypes = [vp, C.c_int, C.c_int, fp, C.c_int, C.c_int, fp, C.c_int]
        L.awe_set_moving_geometry.restype = C.c_int
        L.awe_rtm.argtypes = [vp, fp, C.c_int, fp, C.POINTER(GradOpts), C.c_int, C.POINTER(C.c_double)]
        L.awe_rtm.restype = C.c_int
        lp = C.POINTER(C.c_longlong)
        ll = C.c_longlong
        L.awe_cloud_window.argtypes = [C.c_int, fp, ll, fp, ll, C.c_float, ll, C.c_int, fp, lp, lp, fp, fp]
        L.awe_cloud_window.restype = C.c_int
        L.awe_cloud_merge.argtypes = [C.c_int, fp, ll, C.c_int, lp, fp, fp, ll, C.c_int, C.c_int, C.c_float, fp]
        L.awe_cloud_merge.restype = C.c_int
        L.awe_rtm_device.argtypes = [vp, vp, C.c_int, vp, C.POINTER(GradOpts), C.c_int, vp, vp]
        L.awe_rtm_device.restype = C.c_int
        dp = C.POINTER(C.c_double)
        L.awe_gradient.argtypes = [vp, fp, C.c_int, fp, C.POINTER(GradOpts), dp, dp, fp]
        L.awe_gradient_device.argtypes = [vp, vp, C.c_int, vp, C.POINTER(GradOpts), vp, dp, vp, vp]
        for name in ("awe_plan_create", "awe_plan_destroy", "awe_plan_info", "awe_set_model", "awe_set_geometry",
                     "awe_forward", "awe_forward_device", "awe_set_snapshot_callback", "awe_synchronize",
                     "awe_profile_enable", "awe_profile_read", "awe_profile_read_kinds", "awe_gradient",
                     "awe_gradient_device"):
            getattr(L, name).restype = C.c_int
        _lib = L
    return _lib


def _check(status: int):
    if status != 0:
        raise AweError(status, lib().awe_last_error().decode())


def _fp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def make_desc(ndim, n, d, o, nt, dt, coords=CART, scheme=SCHEME_CPU, nb=-1, fdorder=0, optfd=0, dabc=0,
              hybrid=0, fsrf=0, expl=0, refl=0, jdata=1, jsnap=0, bnds=0, precision=FAST) -> Desc:
    q = Desc()
    q.coords, q.scheme, q.ndim = coords, scheme, ndim
    n = list(n) + [1] * (3 - len(n))
    d = list(d) + [1.0] * (3 - len(d))
    o = list(o) + [0.0] * (3 - len(o))
    for a in range(3):
        q.n[a], q.d[a], q.o[a] = n[a], d[a], o[a]
    q.nb, q.nt, q.dt = nb, nt, dt
    q.fdorder, q.optfd, q.dabc, q.hybrid, q.fsrf = fdorder, int(optfd), int(dabc), int(hybrid), int(fsrf)
    q.expl, q.refl, q.jdata, q.jsnap, q.bnds, q.precision = int(expl), int(refl), jdata, jsnap, int(bnds), precision
    return q


class Plan:
    """One modelling set-up on one GPU: padded grid, model, geometry."""

    def __init__(self, desc: Desc, device: int = 0):
        self._h = C.c_void_p()
        _check(lib().awe_plan_create(C.byref(desc), device, C.byref(self._h)))
        self.desc = desc
        info = Info()
        _check(lib().awe_plan_info(self._h, C.byref(info)))
        self.npad = tuple(info.npad)
        self.nbpad = info.nbpad
        self.nsmp = info.nsmp
        self.nsnap = info.nsnap
        self.snap_elems = info.snap_elems
        self.step_kernel = {1: "tma3d", 2: "tma_sph"}.get(info.step_kernel, "simple")
        self._cb = None
        self.ns = self.nr = 0

    @property
    def handle(self):
        return self._h

    def device_bytes(self) -> int:
        info = Info()
        _check(lib().awe_plan_info(self._h, C.byref(info)))
        return info.device_bytes

    def set_model(self, vel, den=None, rfl=None):
        vel = np.ascontiguousarray(vel, np.float32)
        den = None if den is None else np.ascontiguousarray(den, np.float32)
        rfl = None if rfl is None else np.ascontiguousarray(rfl, np.float32)
        _check(lib().awe_set_model(self._h, _fp(vel), _fp(den), _fp(rfl)))

    def set_geometry(self, sou, rec):
        nd = self.desc.ndim
        sou = np.ascontiguousarray(sou, np.float32).reshape(-1, nd)
        rec = np.ascontiguousarray(rec, np.float32).reshape(-1, nd)
        self.ns, self.nr = sou.shape[0], rec.shape[0]
        _check(lib().awe_set_geometry(self._h, self.ns, _fp(sou), self.nr, _fp(rec)))

    def set_moving_geometry(self, sou, nst: int, rec, nrt: int, mode: int = MOVE_PER_STEP):
        """sou: ns*nst points, rec: nr*nrt points (awe_set_geometry's
        coordinate order); at each step ns sources and nr receivers use the
        entries `mode` selects (awe_set_moving_geometry)."""
        nd = self.desc.ndim
        sou = np.ascontiguousarray(sou, np.float32).reshape(-1, nd)
        rec = np.ascontiguousarray(rec, np.float32).reshape(-1, nd)
        if sou.shape[0] % nst or rec.shape[0] % nrt:
            raise ValueError("tables must hold ns*nst and nr*nrt points")
        self.ns, self.nr = sou.shape[0] // nst, rec.shape[0] // nrt
        _check(lib().awe_set_moving_geometry(self._h, self.ns, nst, _fp(sou), self.nr, nrt, _fp(rec), mode))

    def set_shots(self, shots):
        """shots: list of (sou [ns][3], rec [nr][3]) advanced together (spherical 3D)."""
        nd = self.desc.ndim
        sou = [np.ascontiguousarray(s_, np.float32).reshape(-1, nd) for s_, _ in shots]
        rec = [np.ascontiguousarray(r_, np.float32).reshape(-1, nd) for _, r_ in shots]
        ns = (C.c_int * len(shots))(*[a.shape[0] for a in sou])
        nr = (C.c_int * len(shots))(*[a.shape[0] for a in rec])
        S, R = np.ascontiguousarray(np.concatenate(sou)), np.ascontiguousarray(np.concatenate(rec))
        self.ns, self.nr = S.shape[0], R.shape[0]
        _check(lib().awe_set_shots(self._h, len(shots), ns, _fp(S), nr, _fp(R)))

    def forward(self, wav, snapshots: bool = False):
        """wav: [nt] or [nt][ncs].  Returns dat [nsmp][nr] (and snaps
        [nsnap][snap_elems] when snapshots=True)."""
        wav = np.ascontiguousarray(wav, np.float32)
        ncs = 1 if wav.ndim == 1 else wav.shape[1]
        dat = np.zeros((self.nsmp, self.nr), np.float32)
        wfl = np.zeros((self.nsnap, self.snap_elems), np.float32) if snapshots and self.nsnap else None
        _check(lib().awe_forward(self._h, _fp(wav), ncs, _fp(dat), _fp(wfl)))
        return (dat, wfl) if snapshots else dat

    def gradient(self, wav, dobs, ckpt_every: int = 0, ckpt_format: int = CKPT_BFP16, return_dsyn: bool = False):
        """Misfit J = 0.5 ||d - dobs||^2 and dJ/dm (m = 1/v^2) on the model
        grid (float64, model shape).  Returns (grad, J[, dsyn])."""
        wav = np.ascontiguousarray(wav, np.float32)
        ncs = 1 if wav.ndim == 1 else wav.shape[1]
        dobs = np.ascontiguousarray(dobs, np.float32).reshape(self.nsmp, self.nr)
        n = list(self.desc.n)[: self.desc.ndim]
        grad = np.zeros(n[::-1], np.float64)
        dsyn = np.zeros((self.nsmp, self.nr), np.float32) if return_dsyn else None
        J = C.c_double()
        opts = GradOpts(ckpt_every, ckpt_format)
        _check(lib().awe_gradient(self._h, _fp(wav), ncs, _fp(dobs), C.byref(opts),
                                  grad.ctypes.data_as(C.POINTER(C.c_double)), C.byref(J), _fp(dsyn)))
        return (grad, J.value, dsyn) if return_dsyn else (grad, J.value)

    def rtm(self, wav, data, condition: int = IMAGE_XCORR, ckpt_every: int = 0, ckpt_format: int = CKPT_BFP16):
        """Reverse-time migration image of the recorded traces `data`
        [nsmp][nr] on the exact adjoint (awe_rtm): model shape, float64."""
        wav = np.ascontiguousarray(wav, np.float32)
        ncs = 1 if wav.ndim == 1 else wav.shape[1]
        data = np.ascontiguousarray(data, np.float32).reshape(self.nsmp, self.nr)
        img = np.zeros(list(self.desc.n)[: self.desc.ndim][::-1], np.float64)
        opts = GradOpts(ckpt_every, ckpt_format)
        _check(lib().awe_rtm(self._h, _fp(wav), ncs, _fp(data), C.byref(opts), condition,
                             img.ctypes.data_as(C.POINTER(C.c_double))))
        return img

    def gradient_device(self, d_wav: int, ncs: int, d_dobs: int, d_grad: int, ckpt_every: int = 0,
                        ckpt_format: int = CKPT_BFP16, d_dsyn: int = 0, stream: int = 0) -> float:
        """Device-pointer variant; returns J (the call synchronizes)."""
        J = C.c_double()
        opts = GradOpts(ckpt_every, ckpt_format)
        _check(lib().awe_gradient_device(self._h, C.c_void_p(d_wav), ncs, C.c_void_p(d_dobs), C.byref(opts),
                                         C.c_void_p(d_grad), C.byref(J), C.c_void_p(d_dsyn or None),
                                         C.c_void_p(stream or None)))
        return J.value

    def forward_device(self, d_wav: int, ncs: int, d_dat: int, d_wfl: int = 0, stream: int = 0):
        """Device-resident run: arguments are raw device pointers (ints)."""
        _check(lib().awe_forward_device(self._h, C.c_void_p(d_wav), ncs, C.c_void_p(d_dat),
                                        C.c_void_p(d_wfl) if d_wfl else None,
                                        C.c_void_p(stream) if stream else None))

    def set_snapshot_callback(self, fn):
        """fn(isnap, it, frame: np.ndarray) called per snapshot (host copy)."""
        if fn is None:
            self._cb = None
            _check(lib().awe_set_snapshot_callback(self._h, SNAP_FN(), None))
            return

        def tramp(_user, isnap, it, ptr, n):
            fn(isnap, it, np.ctypeslib.as_array(ptr, shape=(n,)).copy())

        self._cb = SNAP_FN(tramp)
        _check(lib().awe_set_snapshot_callback(self._h, self._cb, None))

    def synchronize(self):
        _check(lib().awe_synchronize(self._h))

    def profile(self, on: bool = True):
        _check(lib().awe_profile_enable(self._h, int(on)))

    def profile_read_kinds(self):
        """{"step": (ms, launches), "adjoint": (ms, launches)} of the runs since
        profiling was enabled or last read: step kernels (forward and the
        gradient's recompute) and the gradient's adjoint step kernels."""
        ms, n = (C.c_double * 2)(), (C.c_longlong * 2)()
        _check(lib().awe_profile_read_kinds(self._h, ms, n))
        return {"step": (ms[0], n[0]), "adjoint": (ms[1], n[1])}

    def profile_read(self):
        """(summed step-kernel milliseconds, step-kernel launches) of the last run."""
        ms, n = C.c_double(), C.c_longlong()
        _check(lib().awe_profile_read(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def last_launch_count(self) -> int:
        return lib().awe_last_launch_count(self._h)

    def close(self):
        if self._h:
            lib().awe_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Batch:
    """Many 2D shots, each on its own window [x0, x0 + nx) of one model,
    advanced together (awe_batch_*).  shots: list of (x0, nx, sou [ns][2],
    rec [nr][2]) with points in model coordinates."""

    def __init__(self, desc: Desc, shots, device: int = 0):
        self._keep = []
        arr = (Shot * len(shots))()
        self.nr = []
        for i, (x0, nx, sou, rec) in enumerate(shots):
            sou = np.ascontiguousarray(sou, np.float32).reshape(-1, 2)
            rec = np.ascontiguousarray(rec, np.float32).reshape(-1, 2)
            self._keep += [sou, rec]
            arr[i] = Shot(int(x0), int(nx), sou.shape[0], rec.shape[0], _fp(sou), _fp(rec))
            self.nr.append(rec.shape[0])
        self._h = C.c_void_p()
        _check(lib().awe_batch_create(C.byref(desc), len(shots), arr, device, C.byref(self._h)))
        self.desc = desc
        self.info = self._info()

    def _info(self):
        info = BatchInfo()
        _check(lib().awe_batch_info(self._h, C.byref(info)))
        return info

    def set_model(self, vel):
        vel = np.ascontiguousarray(vel, np.float32)
        _check(lib().awe_batch_set_model(self._h, _fp(vel)))

    def forward(self, wav):
        """Returns a list of per-shot traces [nsmp][nr_s]."""
        wav = np.ascontiguousarray(wav, np.float32).reshape(-1)
        dat = np.zeros(self.info.total_samples, np.float32)
        _check(lib().awe_batch_forward(self._h, _fp(wav), _fp(dat)))
        out, off = [], 0
        for nr in self.nr:
            n = self.info.nsmp * nr
            out.append(dat[off:off + n].reshape(self.info.nsmp, nr))
            off += n
        return out

    def forward_device(self, d_wav: int, d_dat: int, stream: int = 0):
        _check(lib().awe_batch_forward_device(self._h, C.c_void_p(d_wav), C.c_void_p(d_dat),
                                              C.c_void_p(stream or None)))

    def gradient(self, wav, dobs, ckpt_every: int = 0, ckpt_format: int = CKPT_BFP16):
        """dobs: list of per-shot traces [nsmp][nr_s].  Returns (dJ/dm on the
        whole model [n2][n1], float64; J)."""
        wav = np.ascontiguousarray(wav, np.float32).reshape(-1)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(d, np.float32).ravel() for d in dobs]))
        if flat.size != self.info.total_samples:
            raise ValueError("dobs has %d samples, the batch %d" % (flat.size, self.info.total_samples))
        grad = np.zeros((self.desc.n[1], self.desc.n[0]), np.float64)
        J = C.c_double()
        opts = GradOpts(ckpt_every, ckpt_format)
        _check(lib().awe_batch_gradient(self._h, _fp(wav), _fp(flat), C.byref(opts),
                                        grad.ctypes.data_as(C.POINTER(C.c_double)), C.byref(J)))
        return grad, J.value

    def select(self, kernel: int, chunk: int = 32, grid: int = 0):
        """Forward kernel without timing (awe_batch_select): 0-3 tile shapes,
        4 = the column march with `chunk` columns per item."""
        _check(lib().awe_batch_select(self._h, kernel, chunk, grid))
        self.info = self._info()

    def tune(self, steps: int = 20):
        t, g = C.c_int(), C.c_int()
        _check(lib().awe_batch_tune(self._h, steps, C.byref(t), C.byref(g)))
        self.info = self._info()
        return (self.info.tile_z, self.info.tile_x), g.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().awe_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()



def cloud_window(ground, orbit, apt: float, data=None, device: int = 0):
    """Ground points [ng][9] whose aperture cone (apt degrees about the normal)
    holds an orbit point (orbit [no][9]), in input order (awe_cloud_window).
    data [nf][ng] (complex64 or float32) is optional.  Returns (index [nw],
    points [nw][9], data [nf][nw] or None)."""
    g = np.ascontiguousarray(ground, np.float32).reshape(-1, 9)
    o = np.ascontiguousarray(orbit, np.float32).reshape(-1, 9)
    ng = g.shape[0]
    nf, ncomp, dflat = 0, 2, None
    if data is not None:
        ncomp = 2 if np.iscomplexobj(data) else 1
        d = np.ascontiguousarray(data, np.complex64 if ncomp == 2 else np.float32)
        nf = d.shape[0]
        dflat = d.view(np.float32).reshape(-1)
    index = np.zeros(max(ng, 1), np.int64)
    win = np.zeros((max(ng, 1), 9), np.float32)
    wd = np.zeros(max(nf * ng * ncomp, 1), np.float32)
    nw = C.c_longlong()
    _check(lib().awe_cloud_window(device, _fp(g), ng, _fp(o), o.shape[0], apt, nf, ncomp, _fp(dflat), C.byref(nw),
                                  index.ctypes.data_as(C.POINTER(C.c_longlong)), _fp(win), _fp(wd)))
    n = nw.value
    wdat = None
    if data is not None:
        wdat = wd[: nf * n * ncomp].view(np.complex64 if ncomp == 2 else np.float32).reshape(nf, n).copy()
    return index[:n].copy(), win[:n].copy(), wdat


def cloud_merge(all_pts, windows, norm: bool = True, hashscale: float = 2.0, device: int = 0):
    """Sum windows [(points [nw][9], data [nf][nw]), ...] onto the full cloud
    all_pts [na][9], fold-normalised with norm (awe_cloud_merge).  Returns
    [nf][na] in the windows' dtype (complex64 or float32)."""
    a = np.ascontiguousarray(all_pts, np.float32).reshape(-1, 9)
    na = a.shape[0]
    ncomp = 2 if np.iscomplexobj(windows[0][1]) else 1
    dt = np.complex64 if ncomp == 2 else np.float32
    nf = np.asarray(windows[0][1]).shape[0]
    nwp = np.array([np.asarray(w[0]).reshape(-1, 9).shape[0] for w in windows], np.int64)
    pts = np.ascontiguousarray(np.concatenate([np.asarray(w[0], np.float32).reshape(-1, 9) for w in windows]))
    dat = np.ascontiguousarray(np.concatenate([np.asarray(w[1], dt).reshape(-1) for w in windows])).view(np.float32)
    out = np.zeros(max(nf * na * ncomp, 1), np.float32)
    _check(lib().awe_cloud_merge(device, _fp(a), na, len(windows), nwp.ctypes.data_as(C.POINTER(C.c_longlong)),
                                 _fp(pts), _fp(dat), nf, ncomp, int(norm), hashscale, _fp(out)))
    return out[: nf * na * ncomp].view(dt).reshape(nf, na)
