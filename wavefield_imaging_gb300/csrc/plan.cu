// C-ABI of the engine (include/awe.h): plan lifetime, model and geometry
// upload, and the forward time loop.  The loop issues, per time step, the
// fused step kernel and the few small kernels the reference's step order
// needs around it (injection, boundary passes, receiver gather, snapshot).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <climits>
#include <cstring>
#include <vector>

#include "awe_internal.h"
#include "plan_impl.h"

namespace awe {
const char *last_error();
}

using namespace awe;

#define CUDA_TRY(expr)                                                                            \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return AWE_ERR_CUDA;                                                                  \
        }                                                                                         \
    } while (0)

#define AWE_TRY_SNAP(expr)           \
    do {                             \
        awe_status s_ = (expr);      \
        if (s_ != AWE_OK) return s_; \
    } while (0)

namespace awe {

// Fixed (mode < 0) or moving points.  sfDYNAWEFDcart2Dgpu applies the free
// surface only with free=y (MDYNAWEFDcart2Dgpu.cu:393-396) where
// sfAWEFDcart2Dgpu applies it always (MAWEFDcart2Dgpu.cu:424).
static void set_move_mode(awe_plan *p, int mode, int src_rows, int rec_rows) {
    p->move_mode = mode;
    p->src_rows = src_rows;
    p->rec_rows = rec_rows;
    if (p->d.scheme == AWE_SCHEME_GPU && p->pa.geom == 0) p->pa.mask = (mode == AWE_MOVE_DYN && !p->d.fsrf) ? 0 : 1;
}

void plan_graph_drop(awe_plan *p) {
    plan_gradient_graph_drop(p);
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    p->gexec = nullptr;
    p->g_wav = nullptr;
    p->g_dat = nullptr;
    p->g_ncs = 0;
}

// Optional cap on the device memory one plan may hold (AWE_DEVICE_BYTES_LIMIT,
// bytes): a plan that would exceed it fails with AWE_ERR_NOMEM as if the
// device were full, which lets callers keep a footprint and lets tests take
// the out-of-memory paths without exhausting a shared GPU.
static size_t device_bytes_limit() {
    static const size_t lim = [] {
        const char *e = std::getenv("AWE_DEVICE_BYTES_LIMIT");
        return e && *e ? (size_t)std::strtoull(e, nullptr, 10) : (size_t)0;
    }();
    return lim;
}

awe_status dev_alloc(awe_plan *p, void **ptr, size_t bytes) {
    if (bytes == 0) bytes = 16;
    const size_t lim = device_bytes_limit();
    if (lim && p->device_bytes + bytes > lim) {
        *ptr = nullptr;
        set_error("device memory limit: %zu bytes held + %zu requested > AWE_DEVICE_BYTES_LIMIT %zu",
                  p->device_bytes, bytes, lim);
        return AWE_ERR_NOMEM;
    }
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
        set_error("cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
        return AWE_ERR_NOMEM;
    }
    p->allocs.push_back({*ptr, bytes});
    p->device_bytes += bytes;
    return AWE_OK;
}

void dev_free(awe_plan *p, void *ptr) {
    if (!ptr) return;
    for (auto it = p->allocs.begin(); it != p->allocs.end(); ++it)
        if (it->first == ptr) {
            p->device_bytes -= it->second;
            p->allocs.erase(it);
            break;
        }
    cudaFree(ptr);
}

// Snapshot frames stream to the callback through two pinned host buffers:
// frame k is copied (cudaMemcpyAsync, event) while the host hands frame k-1,
// whose copy finished long before, to the callback - the host never waits on
// the GPU for the frame it just queued, and the GPU never waits on the
// callback (disk writes overlap the following time steps).
static awe_status snap_deliver_pending(awe_plan *p) {
    if (p->snap_pending < 0) return AWE_OK;
    const int b = p->snap_pending_isnap & 1;
    CUDA_TRY(cudaEventSynchronize(p->snap_ev[b]));
    p->snap_cb(p->snap_user, p->snap_pending_isnap, p->snap_pending_it, p->snap_host[b], p->snap_elems);
    p->snap_pending = -1;
    return AWE_OK;
}

awe_status deliver_snapshot(awe_plan *p, const float *d_frame, int isnap, int it, cudaStream_t s) {
    if (!p->snap_cb) return AWE_OK;
    const size_t bytes = p->snap_elems * sizeof(float);
    if (p->snap_host_bytes < bytes) {
        AWE_TRY_SNAP(snap_deliver_pending(p));
        for (int b = 0; b < 2; b++) {
            if (p->snap_host[b]) cudaFreeHost(p->snap_host[b]);
            p->snap_host[b] = nullptr;
            if (cudaMallocHost((void **)&p->snap_host[b], bytes) != cudaSuccess) {
                set_error("pinned snapshot buffers (2 x %zu bytes) failed", bytes);
                return AWE_ERR_NOMEM;
            }
            if (!p->snap_ev[b]) CUDA_TRY(cudaEventCreateWithFlags(&p->snap_ev[b], cudaEventDisableTiming));
        }
        p->snap_host_bytes = bytes;
    }
    const int b = isnap & 1;
    CUDA_TRY(cudaMemcpyAsync(p->snap_host[b], d_frame, bytes, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaEventRecord(p->snap_ev[b], s));
    AWE_TRY_SNAP(snap_deliver_pending(p));
    p->snap_pending = 1;
    p->snap_pending_isnap = isnap;
    p->snap_pending_it = it;
    return AWE_OK;
}

awe_status flush_snapshots(awe_plan *p) { return p->snap_cb ? snap_deliver_pending(p) : AWE_OK; }

void prof_begin(awe_plan *p, cudaStream_t s, int kind) {
    if (!p->profile) return;
    const size_t need = 2 * (size_t)(p->prof_n + 1);
    if (p->prof_kind.size() < (size_t)p->prof_n + 1) p->prof_kind.resize((size_t)p->prof_n + 1);
    p->prof_kind[(size_t)p->prof_n] = kind;
    while (p->prof_ev.size() < need) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) {
            p->profile = false;
            return;
        }
        p->prof_ev.push_back(e);
    }
    cudaEventRecord(p->prof_ev[2 * p->prof_n], s);
}

void prof_end(awe_plan *p, cudaStream_t s) {
    if (!p->profile || p->prof_ev.size() < 2 * (size_t)(p->prof_n + 1)) return;
    cudaEventRecord(p->prof_ev[2 * p->prof_n + 1], s);
    p->prof_n++;
}

}  // namespace awe

// The pipelined step kernels bound every wait and raise a device flag instead
// of hanging; surface it as a CUDA error once the stream has drained.
static awe_status check_pipeline(awe_plan *p) {
    if (!p->d_err) return AWE_OK;
    int h = 0;
    CUDA_TRY(cudaMemcpy(&h, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        cudaMemset(p->d_err, 0, sizeof(int));
        set_error("a pipeline wait in the step kernel timed out; this run's results are invalid");
        return AWE_ERR_CUDA;
    }
    return AWE_OK;
}

awe_status awe::check_desc(const awe_desc *d) {
    if (!d) {
        set_error("null descriptor");
        return AWE_ERR_INVALID;
    }
    if (d->ndim != 2 && d->ndim != 3) {
        set_error("ndim must be 2 or 3 (got %d)", d->ndim);
        return AWE_ERR_INVALID;
    }
    for (int a = 0; a < d->ndim; a++) {
        if (d->n[a] < 1) {
            set_error("axis %d has n=%d", a + 1, d->n[a]);
            return AWE_ERR_INVALID;
        }
        if (!(d->d[a] > 0.f)) {
            set_error("axis %d has spacing %g", a + 1, (double)d->d[a]);
            return AWE_ERR_INVALID;
        }
    }
    if (d->nt < 1 || !(d->dt > 0.f)) {
        set_error("need nt >= 1 and dt > 0 (nt=%d dt=%g)", d->nt, (double)d->dt);
        return AWE_ERR_INVALID;
    }
    if (d->scheme != AWE_SCHEME_CPU && d->scheme != AWE_SCHEME_GPU) {
        set_error("unknown scheme %d", d->scheme);
        return AWE_ERR_INVALID;
    }
    if (d->coords != AWE_CART && d->coords != AWE_SPHER) {
        set_error("unknown coordinate system %d", d->coords);
        return AWE_ERR_INVALID;
    }
    if (d->scheme == AWE_SCHEME_CPU) {
        if (d->coords != AWE_CART) {
            set_error("the 2N-order CPU scheme is cartesian only (as MAWEFDcart*cpu.c)");
            return AWE_ERR_UNSUPPORTED;
        }
        int fo = d->fdorder ? d->fdorder : 4;
        if (fo < 2 || fo > 2 * kMaxNop || (fo & 1)) {
            set_error("fdorder must be even in [2, %d] (got %d)", 2 * kMaxNop, fo);
            return AWE_ERR_INVALID;
        }
    } else {
        if (d->fdorder != 0 && d->fdorder != 2) {
            set_error("the GPU programs' scheme is second order (fdorder=%d)", d->fdorder);
            return AWE_ERR_UNSUPPORTED;
        }
    }
    if (d->jsnap < 0 || d->jdata < 0) {
        set_error("jsnap and jdata must be >= 0");
        return AWE_ERR_INVALID;
    }
    if (d->precision != AWE_FAST && d->precision != AWE_EXACT) {
        set_error("unknown precision %d", d->precision);
        return AWE_ERR_INVALID;
    }
    return AWE_OK;
}

extern "C" {

const char *awe_version(void) { return "awe-gb300 1.0 (sm_103a)"; }
const char *awe_last_error(void) { return awe::last_error(); }

const char *awe_status_string(awe_status s) {
    switch (s) {
        case AWE_OK: return "ok";
        case AWE_ERR_INVALID: return "invalid argument";
        case AWE_ERR_CUDA: return "CUDA error";
        case AWE_ERR_NOMEM: return "out of memory";
        case AWE_ERR_UNSUPPORTED: return "unsupported";
        case AWE_ERR_NODEVICE: return "no CUDA device";
        case AWE_ERR_STATE: return "call out of order";
    }
    return "unknown";
}

awe_status awe_plan_create(const awe_desc *desc, int device, awe_plan **out) {
    if (!out) {
        set_error("null output pointer");
        return AWE_ERR_INVALID;
    }
    *out = nullptr;
    awe_status st = check_desc(desc);
    if (st != AWE_OK) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device visible");
        return AWE_ERR_NODEVICE;
    }
    if (device < 0 || device >= ndev) {
        set_error("device %d out of range (%d devices)", device, ndev);
        return AWE_ERR_INVALID;
    }
    CUDA_TRY(cudaSetDevice(device));
    awe_plan *p = new awe_plan();
    p->d = *desc;
    p->device = device;
    if (p->d.jdata <= 0) p->d.jdata = 1;
    if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete p;
        set_error("cudaStreamCreate failed");
        return AWE_ERR_CUDA;
    }
    st = (p->d.scheme == AWE_SCHEME_CPU) ? planB_init(p) : planA_init(p);
    if (st != AWE_OK) {
        awe_plan_destroy(p);
        return st;
    }
    *out = p;
    return AWE_OK;
}

awe_status awe_plan_destroy(awe_plan *p) {
    if (!p) return AWE_OK;
    cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    plan_graph_drop(p);
    plan_gradient_free(p);
    for (auto &a : p->allocs) cudaFree(a.first);
    p->allocs.clear();
    for (int b = 0; b < 2; b++) {
        if (p->snap_host[b]) cudaFreeHost(p->snap_host[b]);
        if (p->snap_ev[b]) cudaEventDestroy(p->snap_ev[b]);
    }
    for (cudaEvent_t e : p->prof_ev) cudaEventDestroy(e);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
    return AWE_OK;
}

awe_status awe_plan_info(const awe_plan *p, awe_info *info) {
    if (!p || !info) {
        set_error("null argument");
        return AWE_ERR_INVALID;
    }
    info->npad[0] = p->g.n1;
    info->npad[1] = p->g.n2;
    info->npad[2] = p->g.n3;
    info->nbpad = p->nbd;
    info->nsmp = p->nsmp;
    info->nsnap = p->nsnap;
    info->snap_elems = p->snap_elems;
    info->device_bytes = p->device_bytes;
    info->step_kernel = p->use_tma ? 1 : (p->sph_tma ? 2 : 0);
    return AWE_OK;
}

awe_status awe_set_model(awe_plan *p, const float *vel, const float *den, const float *rfl) {
    if (!p || !vel) {
        set_error("null plan or velocity");
        return AWE_ERR_INVALID;
    }
    // The captured time loop of the CPU-program scheme reads the model through
    // its device buffers, which a new model refills in place: the loop is kept
    // unless a buffer moved (the first model, or a density added).
    const bool cpu = p->d.scheme == AWE_SCHEME_CPU;
    const void *before[8] = {p->vel, p->den, p->abc[0], p->abc[1], p->abc[2], p->abc[3], p->abc[4], p->abc[5]};
    if (cpu) plan_gradient_graph_drop(p);
    else plan_graph_drop(p);
    CUDA_TRY(cudaSetDevice(p->device));
    awe_status st = cpu ? planB_model(p, vel, den) : planA_model(p, vel, rfl);
    if (cpu) {
        const void *after[8] = {p->vel, p->den, p->abc[0], p->abc[1], p->abc[2], p->abc[3], p->abc[4], p->abc[5]};
        if (st != AWE_OK || std::memcmp(before, after, sizeof before) != 0) plan_graph_drop(p);
    }
    if (st == AWE_OK) p->model_set = true;
    return st;
}

// back to one shot after awe_set_shots: one field per time level
static awe_status single_shot(awe_plan *p, int ns, int nr) {
    p->shot_ns.assign(1, ns);
    p->shot_nr.assign(1, nr);
    if (p->pa.nshot <= 1) return AWE_OK;
    const size_t bytes = (size_t)p->g.cells() * sizeof(float);
    for (int k = 0; k < 2; k++) {
        dev_free(p, p->u[k]);
        p->u[k] = nullptr;
        const awe_status st = dev_alloc(p, (void **)&p->u[k], bytes);
        if (st != AWE_OK) return st;
    }
    p->pa.nshot = 1;
    return AWE_OK;
}

awe_status awe_set_geometry(awe_plan *p, int ns, const float *sou, int nr, const float *rec) {
    if (!p || ns < 0 || nr < 0 || (ns > 0 && !sou) || (nr > 0 && !rec)) {
        set_error("bad geometry arguments");
        return AWE_ERR_INVALID;
    }
    // the captured time loop baked in the point buffers, their counts and the
    // flags the points set; it is kept when none of them changes (the same
    // acquisition run again, or points that only moved within their buffers)
    auto key = [&](long long *k) {
        k[0] = (long long)(uintptr_t)p->src;
        k[1] = (long long)(uintptr_t)p->rec;
        k[2] = p->ns;
        k[3] = p->nr;
        k[4] = p->move_mode;
        k[5] = p->src_rows;
        k[6] = p->rec_rows;
        k[7] = p->sponge_deferred;
        k[8] = p->src_in_shell;
        k[9] = p->pa.nshot;
    };
    long long before[10], after[10];
    key(before);
    plan_gradient_graph_drop(p);  // its per-cell point lists follow the geometry
    CUDA_TRY(cudaSetDevice(p->device));
    set_move_mode(p, -1, 1, 1);
    awe_status st = set_geometry_common(p, ns, sou, nr, rec);
    if (st == AWE_OK) st = single_shot(p, ns, nr);
    key(after);
    if (st != AWE_OK || std::memcmp(before, after, sizeof before) != 0) plan_graph_drop(p);
    if (st == AWE_OK) p->geom_set = true;
    return st;
}

awe_status awe_set_moving_geometry(awe_plan *p, int ns, int nst, const float *sou, int nr, int nrt,
                                   const float *rec, int mode) {
    if (!p || ns < 0 || nr < 0 || nst < 1 || nrt < 1 || (ns > 0 && !sou) || (nr > 0 && !rec)) {
        set_error("bad moving-geometry arguments (ns, nr >= 0; nst, nrt >= 1; coordinates for every entry)");
        return AWE_ERR_INVALID;
    }
    const awe_desc &d = p->d;
    if (mode != AWE_MOVE_PER_STEP && mode != AWE_MOVE_DYN) {
        set_error("unknown moving-geometry mode %d", mode);
        return AWE_ERR_INVALID;
    }
    if (mode == AWE_MOVE_DYN && !(d.scheme == AWE_SCHEME_GPU && d.coords == AWE_CART && d.ndim == 2)) {
        set_error("AWE_MOVE_DYN follows sfDYNAWEFDcart2Dgpu: cartesian 2D, AWE_SCHEME_GPU");
        return AWE_ERR_UNSUPPORTED;
    }
    if (d.scheme == AWE_SCHEME_GPU && (d.expl || d.refl)) {
        set_error("moving geometry on the GPU-program scheme needs expl = 0 (unscaled injection)");
        return AWE_ERR_UNSUPPORTED;
    }
    if (mode == AWE_MOVE_DYN) {
        // the entries the run selects: k*(it+1) for k < n, it < nt
        const long long last_s = (long long)(ns > 0 ? ns - 1 : 0) * d.nt, last_r = (long long)(nr > 0 ? nr - 1 : 0) * d.nt;
        if ((ns > 0 && last_s >= (long long)ns * nst) || (nr > 0 && last_r >= (long long)nr * nrt)) {
            set_error("AWE_MOVE_DYN reads entry (n-1)*nt of each table: need (ns-1)*nt < ns*nst and "
                      "(nr-1)*nt < nr*nrt (ns=%d nst=%d nr=%d nrt=%d nt=%d)",
                      ns, nst, nr, nrt, d.nt);
            return AWE_ERR_INVALID;
        }
    }
    if ((long long)ns * nst > INT_MAX || (long long)nr * nrt > INT_MAX) {
        set_error("moving-geometry tables too large");
        return AWE_ERR_INVALID;
    }
    plan_graph_drop(p);  // the captured time loop baked in the old state
    CUDA_TRY(cudaSetDevice(p->device));
    awe_status st = set_geometry_common(p, ns * nst, sou, nr * nrt, rec);
    if (st != AWE_OK) return st;
    p->ns = ns;
    p->nr = nr;
    set_move_mode(p, mode, nst, nrt);
    st = single_shot(p, ns, nr);
    if (st != AWE_OK) return st;
    p->geom_set = true;
    return AWE_OK;
}

awe_status awe_set_shots(awe_plan *p, int nshots, const int *ns, const float *sou, const int *nr, const float *rec) {
    if (!p || nshots < 1 || !ns || !nr) {
        set_error("bad shot arguments");
        return AWE_ERR_INVALID;
    }
    plan_graph_drop(p);  // the captured time loop baked in the old state
    const awe_desc &d = p->d;
    if (nshots > 1 && !(d.scheme == AWE_SCHEME_GPU && d.coords == AWE_SPHER && d.ndim == 3 &&
                        d.precision == AWE_FAST && d.jsnap == 0)) {
        set_error("awe_set_shots: several shots need the spherical 3D GPU-program scheme, AWE_FAST, no snapshots");
        return AWE_ERR_UNSUPPORTED;
    }
    int NS = 0, NR = 0;
    for (int s = 0; s < nshots; s++) {
        if (ns[s] < 0 || nr[s] < 0) {
            set_error("negative point count for shot %d", s);
            return AWE_ERR_INVALID;
        }
        NS += ns[s];
        NR += nr[s];
    }
    if ((NS > 0 && !sou) || (NR > 0 && !rec)) {
        set_error("null source or receiver coordinates");
        return AWE_ERR_INVALID;
    }
    CUDA_TRY(cudaSetDevice(p->device));
    set_move_mode(p, -1, 1, 1);
    awe_status st = set_geometry_common(p, NS, sou, NR, rec);
    if (st != AWE_OK) return st;
    // points of shot s address field s
    const long long cells = p->g.cells();
    int a = 0, b = 0;
    for (int s = 0; s < nshots; s++) {
        for (int i = 0; i < ns[s]; i++) p->h_src[a++].base += s * cells;
        for (int i = 0; i < nr[s]; i++) p->h_rec[b++].base += s * cells;
    }
    if (NS) CUDA_TRY(cudaMemcpy(p->src, p->h_src.data(), NS * sizeof(GeoPoint), cudaMemcpyHostToDevice));
    if (NR) CUDA_TRY(cudaMemcpy(p->rec, p->h_rec.data(), NR * sizeof(GeoPoint), cudaMemcpyHostToDevice));
    p->shot_ns.assign(ns, ns + nshots);
    p->shot_nr.assign(nr, nr + nshots);
    if (nshots != p->pa.nshot) {
        for (int k = 0; k < 2; k++) {
            dev_free(p, p->u[k]);
            p->u[k] = nullptr;
            st = dev_alloc(p, (void **)&p->u[k], (size_t)nshots * cells * sizeof(float));
            if (st != AWE_OK) return st;
        }
        p->pa.nshot = nshots;
    }
    p->geom_set = true;
    return AWE_OK;
}

awe_status awe_set_snapshot_callback(awe_plan *p, awe_snap_fn fn, void *user) {
    if (!p) {
        set_error("null plan");
        return AWE_ERR_INVALID;
    }
    plan_graph_drop(p);  // the captured time loop baked in the old state
    p->snap_cb = fn;
    p->snap_user = user;
    return AWE_OK;
}

awe_status awe_synchronize(awe_plan *p) {
    if (!p) return AWE_ERR_INVALID;
    CUDA_TRY(cudaSetDevice(p->device));
    CUDA_TRY(cudaStreamSynchronize(p->stream));
    return check_pipeline(p);
}

long long awe_last_launch_count(const awe_plan *p) { return p ? p->launches : -1; }

awe_status awe_profile_enable(awe_plan *p, int on) {
    if (!p) return AWE_ERR_INVALID;
    plan_graph_drop(p);  // profiled runs bracket kernels with host-side events: no graph
    p->profile = on != 0;
    p->prof_n = 0;
    return AWE_OK;
}

awe_status awe_profile_read_kinds(awe_plan *p, double *ms, long long *n) {
    if (!p || !ms || !n) return AWE_ERR_INVALID;
    CUDA_TRY(cudaSetDevice(p->device));
    for (int k = 0; k < AWE_PROF_KINDS; k++) {
        ms[k] = 0.0;
        n[k] = 0;
    }
    for (long long i = 0; i < p->prof_n; i++) {
        float t = 0.f;
        CUDA_TRY(cudaEventSynchronize(p->prof_ev[2 * i + 1]));
        CUDA_TRY(cudaEventElapsedTime(&t, p->prof_ev[2 * i], p->prof_ev[2 * i + 1]));
        const int k = p->prof_kind[(size_t)i];
        ms[k] += t;
        n[k]++;
    }
    p->prof_n = 0;
    return AWE_OK;
}

awe_status awe_profile_read(awe_plan *p, double *ms, long long *n) {
    if (!p || !ms || !n) return AWE_ERR_INVALID;
    double mk[AWE_PROF_KINDS];
    long long nk[AWE_PROF_KINDS];
    const awe_status st = awe_profile_read_kinds(p, mk, nk);
    if (st != AWE_OK) return st;
    *ms = mk[AWE_PROF_STEP];
    *n = nk[AWE_PROF_STEP];
    return AWE_OK;
}

awe_status awe_forward_device(awe_plan *p, const float *d_wav, int ncs, float *d_dat, float *d_wfl, void *stream) {
    if (!p || !d_wav || !d_dat) {
        set_error("null plan, wavelet or data pointer");
        return AWE_ERR_INVALID;
    }
    if (!p->model_set || !p->geom_set) {
        set_error("awe_set_model and awe_set_geometry must precede awe_forward");
        return AWE_ERR_STATE;
    }
    if (ncs != 1 && ncs != p->ns) {
        set_error("wavelet has %d components; need 1 or ns=%d", ncs, p->ns);
        return AWE_ERR_INVALID;
    }
    CUDA_TRY(cudaSetDevice(p->device));
    cudaStream_t s = stream ? (cudaStream_t)stream : p->stream;
    // the CPU-program scheme's loop is pure stream work without snapshots and
    // profiling: capture it once as a CUDA graph and replay it (one launch per
    // run instead of several per time step - what matters for small 2D grids)
    const bool graph = p->d.scheme == AWE_SCHEME_CPU && !(p->nsnap > 0 && (d_wfl || p->snap_cb)) && !p->profile;
    awe_status st = AWE_OK;
    if (graph) {
        if (!p->gexec || p->g_wav != d_wav || p->g_dat != d_dat || p->g_ncs != ncs) {
            plan_graph_drop(p);
            cudaStream_t cs;
            CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
            cudaGraph_t gr = nullptr;
            cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                st = planB_run(p, d_wav, ncs, d_dat, nullptr, cs);
                e = cudaStreamEndCapture(cs, &gr);
            }
            if (st == AWE_OK && e == cudaSuccess) e = cudaGraphInstantiate(&p->gexec, gr, 0);
            if (gr) cudaGraphDestroy(gr);
            cudaStreamDestroy(cs);
            if (st != AWE_OK) return st;
            if (e != cudaSuccess) {
                plan_graph_drop(p);
                set_error("CUDA graph capture of the time loop failed: %s", cudaGetErrorString(e));
                return AWE_ERR_CUDA;
            }
            p->g_wav = d_wav;
            p->g_dat = d_dat;
            p->g_ncs = ncs;
            p->g_launches = p->launches;
        }
        CUDA_TRY(cudaGraphLaunch(p->gexec, s));
        p->launches = p->g_launches;
    } else {
        st = (p->d.scheme == AWE_SCHEME_CPU) ? planB_run(p, d_wav, ncs, d_dat, d_wfl, s)
                                             : planA_run(p, d_wav, ncs, d_dat, d_wfl, s);
    }
    if (st != AWE_OK) return st;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("kernel launch failed: %s", cudaGetErrorString(e));
        return AWE_ERR_CUDA;
    }
    return AWE_OK;
}

awe_status awe_forward(awe_plan *p, const float *wav, int ncs, float *dat, float *wfl) {
    if (!p || !wav || !dat) {
        set_error("null plan, wavelet or data pointer");
        return AWE_ERR_INVALID;
    }
    if (!p->model_set || !p->geom_set) {
        set_error("awe_set_model and awe_set_geometry must precede awe_forward");
        return AWE_ERR_STATE;
    }
    CUDA_TRY(cudaSetDevice(p->device));
    const size_t wav_bytes = (size_t)p->d.nt * ncs * sizeof(float);
    const size_t dat_bytes = (size_t)p->nsmp * p->nr * sizeof(float);
    // staging buffers kept across calls (stable pointers keep the captured time loop valid)
    awe_status st = AWE_OK;
    auto stage = [&](float **buf, size_t &have, size_t need) {
        if (have >= need && *buf) return AWE_OK;
        dev_free(p, *buf);
        *buf = nullptr;
        have = 0;
        awe_status r = dev_alloc(p, (void **)buf, need);
        if (r == AWE_OK) have = need;
        return r;
    };
    st = stage(&p->stage_wav, p->stage_wav_bytes, wav_bytes);
    if (st == AWE_OK) st = stage(&p->stage_dat, p->stage_dat_bytes, dat_bytes);
    float *d_wav = p->stage_wav, *d_dat = p->stage_dat, *d_wfl = nullptr;
    if (st == AWE_OK && wfl && p->nsnap > 0) st = dev_alloc(p, (void **)&d_wfl, p->nsnap * p->snap_elems * sizeof(float));
    if (st == AWE_OK) {
        cudaError_t e = cudaMemcpyAsync(d_wav, wav, wav_bytes, cudaMemcpyHostToDevice, p->stream);
        if (e != cudaSuccess) {
            set_error("wavelet upload failed: %s", cudaGetErrorString(e));
            st = AWE_ERR_CUDA;
        }
    }
    if (st == AWE_OK) st = awe_forward_device(p, d_wav, ncs, d_dat, d_wfl, nullptr);
    if (st == AWE_OK) {
        cudaError_t e = cudaMemcpyAsync(dat, d_dat, dat_bytes, cudaMemcpyDeviceToHost, p->stream);
        if (e == cudaSuccess && d_wfl)
            e = cudaMemcpyAsync(wfl, d_wfl, p->nsnap * p->snap_elems * sizeof(float), cudaMemcpyDeviceToHost,
                                p->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
        if (e != cudaSuccess) {
            set_error("result download failed: %s", cudaGetErrorString(e));
            st = AWE_ERR_CUDA;
        }
    }
    cudaStreamSynchronize(p->stream);
    dev_free(p, d_wfl);
    if (st == AWE_OK) st = check_pipeline(p);
    return st;
}

static awe_status gradient_or_image(awe_plan *p, const float *d_wav, int ncs, const float *d_dobs,
                                    const awe_grad_opts *opts, double *d_grad, double *misfit, float *d_dsyn,
                                    void *stream, int image);

awe_status awe_rtm_device(awe_plan *p, const float *d_wav, int ncs, const float *d_data, const awe_grad_opts *opts,
                          int condition, double *d_image, void *stream) {
    if (condition != AWE_IMAGE_XCORR && condition != AWE_IMAGE_BORN) {
        set_error("awe_rtm: unknown imaging condition %d", condition);
        return AWE_ERR_INVALID;
    }
    double unused = 0;
    return gradient_or_image(p, d_wav, ncs, d_data, opts, d_image, &unused, nullptr, stream, condition);
}

awe_status awe_gradient_device(awe_plan *p, const float *d_wav, int ncs, const float *d_dobs,
                               const awe_grad_opts *opts, double *d_grad, double *misfit, float *d_dsyn,
                               void *stream) {
    return gradient_or_image(p, d_wav, ncs, d_dobs, opts, d_grad, misfit, d_dsyn, stream, -1);
}

static awe_status gradient_or_image(awe_plan *p, const float *d_wav, int ncs, const float *d_dobs,
                                    const awe_grad_opts *opts, double *d_grad, double *misfit, float *d_dsyn,
                                    void *stream, int image) {
    if (!p || !d_wav || !d_dobs || !d_grad || !misfit) {
        set_error("null plan, wavelet, data, gradient or misfit pointer");
        return AWE_ERR_INVALID;
    }
    if (!p->model_set || !p->geom_set) {
        set_error("awe_set_model and awe_set_geometry must precede awe_gradient");
        return AWE_ERR_STATE;
    }
    if (p->move_mode >= 0) {
        set_error("awe_gradient: the misfit gradient needs fixed sources and receivers (awe_set_geometry)");
        return AWE_ERR_UNSUPPORTED;
    }
    if (ncs != 1 && ncs != p->ns) {
        set_error("wavelet has %d components; need 1 or ns=%d", ncs, p->ns);
        return AWE_ERR_INVALID;
    }
    awe_grad_opts o{0, AWE_CKPT_BFP16};
    if (opts) o = *opts;
    CUDA_TRY(cudaSetDevice(p->device));
    cudaStream_t s = stream ? (cudaStream_t)stream : p->stream;
    awe_status st = plan_gradient(p, d_wav, ncs, d_dobs, o, d_grad, misfit, d_dsyn, s, image);
    if (st != AWE_OK) return st;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("kernel launch failed: %s", cudaGetErrorString(e));
        return AWE_ERR_CUDA;
    }
    return check_pipeline(p);
}

static awe_status gradient_or_image_host(awe_plan *p, const float *wav, int ncs, const float *dobs,
                                         const awe_grad_opts *opts, double *grad, double *misfit, float *dsyn,
                                         int image);

awe_status awe_gradient(awe_plan *p, const float *wav, int ncs, const float *dobs, const awe_grad_opts *opts,
                        double *grad, double *misfit, float *dsyn) {
    return gradient_or_image_host(p, wav, ncs, dobs, opts, grad, misfit, dsyn, -1);
}

awe_status awe_rtm(awe_plan *p, const float *wav, int ncs, const float *data, const awe_grad_opts *opts,
                   int condition, double *image) {
    if (condition != AWE_IMAGE_XCORR && condition != AWE_IMAGE_BORN) {
        set_error("awe_rtm: unknown imaging condition %d", condition);
        return AWE_ERR_INVALID;
    }
    double unused = 0;
    return gradient_or_image_host(p, wav, ncs, data, opts, image, &unused, nullptr, condition);
}

static awe_status gradient_or_image_host(awe_plan *p, const float *wav, int ncs, const float *dobs,
                                         const awe_grad_opts *opts, double *grad, double *misfit, float *dsyn,
                                         int image) {
    if (!p || !wav || !dobs || !grad || !misfit) {
        set_error("null plan, wavelet, data, gradient or misfit pointer");
        return AWE_ERR_INVALID;
    }
    CUDA_TRY(cudaSetDevice(p->device));
    const awe_desc &d = p->d;
    const size_t wav_bytes = (size_t)d.nt * ncs * sizeof(float);
    const size_t dat_bytes = (size_t)p->nsmp * p->nr * sizeof(float);
    const size_t grad_bytes = (size_t)d.n[0] * d.n[1] * (d.ndim == 3 ? d.n[2] : 1) * sizeof(double);
    // staging buffers kept across calls (stable pointers keep a captured gradient valid)
    auto stage = [&](void **buf, size_t &have, size_t need) {
        if (need == 0) need = 16;
        if (have >= need && *buf) return AWE_OK;
        dev_free(p, *buf);
        *buf = nullptr;
        have = 0;
        awe_status r = dev_alloc(p, buf, need);
        if (r == AWE_OK) have = need;
        return r;
    };
    awe_status st = stage((void **)&p->stage_wav, p->stage_wav_bytes, wav_bytes);
    if (st == AWE_OK) st = stage((void **)&p->stage_dat, p->stage_dat_bytes, dat_bytes);
    if (st == AWE_OK && dsyn) st = stage((void **)&p->stage_dsyn, p->stage_dsyn_bytes, dat_bytes);
    if (st == AWE_OK) st = stage((void **)&p->stage_grad, p->stage_grad_bytes, grad_bytes);
    if (st != AWE_OK) return st;
    float *d_wav = p->stage_wav, *d_dobs = p->stage_dat, *d_dsyn = dsyn ? p->stage_dsyn : nullptr;
    double *d_grad = p->stage_grad;
    if (st == AWE_OK) {
        cudaError_t e = cudaMemcpyAsync(d_wav, wav, wav_bytes, cudaMemcpyHostToDevice, p->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_dobs, dobs, dat_bytes, cudaMemcpyHostToDevice, p->stream);
        if (e != cudaSuccess) {
            set_error("input upload failed: %s", cudaGetErrorString(e));
            st = AWE_ERR_CUDA;
        }
    }
    if (st == AWE_OK) st = gradient_or_image(p, d_wav, ncs, d_dobs, opts, d_grad, misfit, d_dsyn, nullptr, image);
    if (st == AWE_OK) {
        cudaError_t e = cudaMemcpyAsync(grad, d_grad, grad_bytes, cudaMemcpyDeviceToHost, p->stream);
        if (e == cudaSuccess && dsyn) e = cudaMemcpyAsync(dsyn, d_dsyn, dat_bytes, cudaMemcpyDeviceToHost, p->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
        if (e != cudaSuccess) {
            set_error("result download failed: %s", cudaGetErrorString(e));
            st = AWE_ERR_CUDA;
        }
    }
    cudaStreamSynchronize(p->stream);
    return st;
}

}  // extern "C"
