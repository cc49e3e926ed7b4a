// Host side of the batched 2D forward (awe_batch_*): many shots along a
// track, each on its own window of one model (the c1-style survey of
// byrne_awe.py, one sfAWEFDcart2Dcpu run per window), advanced together.
//
// All shots' padded fields live in three concatenated arrays; every time step
// is one launch of k_batch2d over the flat (shot, tile) + (shot, receiver
// block) item list; the nt launches are captured once into a CUDA graph and
// replayed.  The autotuner times each tile shape and grid size on a few steps
// and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "awe_internal.h"

using namespace awe;

struct awe_batch {
    awe_desc d{};
    int device = 0;
    cudaStream_t stream = nullptr;
    int nop = 4, nb = 0, n1 = 0;  // padded rows
    Coef k{};
    std::vector<awe_shot> shots_in;
    std::vector<BatchShot> shots;
    std::vector<float> h_wz, h_wx;
    std::vector<int4> items;
    int ntile_items = 0;
    long long cells = 0, ndat = 0;
    int nsmp = 0;
    std::vector<void *> allocs;
    float *u[2] = {nullptr, nullptr}, *vel = nullptr, *wz = nullptr, *wx = nullptr, *wav = nullptr, *dat = nullptr;
    BatchShot *d_shots = nullptr;
    int4 *d_items = nullptr;
    GeoPoint *src = nullptr, *rec = nullptr;
    bool model_set = false;
    int tile = 0, grid = 0, sms = 1;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
    std::vector<GeoPoint> h_rec;
    // misfit gradient state
    int gT = 0, gseg = 0, gfmt = -1;
    long long gscale_per = 0;  // checkpoint scales per level: one per shot, or per 64-cell block (BFP16)
    float *slots = nullptr, *gX = nullptr, *gY = nullptr, *res = nullptr, *scales = nullptr, *dobs = nullptr;
    void *ckpt = nullptr;
    float2 *G = nullptr;  // gradient accumulators (compensated pairs)
    double *part = nullptr, *grad = nullptr;
    // receiver cells of the adjoint's residual term (-1: not built yet)
    BatchRecCell *rec_cells = nullptr;
    BatchRecW *rec_ws = nullptr;
    int nrec_cells = -1;
    int2 *win = nullptr;
    // column-march forward (k_batch2d_col): chunk length (0 = the tile kernels), its items and grid
    int colL = 0, col_grid = 0, ncol_items = 0;
    std::vector<int4> col_items;
    int4 *d_col_items = nullptr;
    int *d_err = nullptr;  // set by a bulk-copy wait that timed out
    int col_adj_grid = 0;  // column-march adjoint's grid (0: the tile adjoint)
};

#define CUDA_TRY(expr)                                                                            \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return AWE_ERR_CUDA;                                                                  \
        }                                                                                         \
    } while (0)

static awe_status balloc(awe_batch *b, void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        set_error("cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
        return AWE_ERR_NOMEM;
    }
    b->allocs.push_back(*p);
    return AWE_OK;
}

static void drop_graph(awe_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

static void build_items(awe_batch *b) {
    const int TZ = kBatchTiles[b->tile][0], TX = kBatchTiles[b->tile][1];
    b->items.clear();
    for (int s = 0; s < (int)b->shots.size(); s++)
        for (int x0 = 0; x0 < b->shots[s].n2; x0 += TX)
            for (int z0 = 0; z0 < b->n1; z0 += TZ) b->items.push_back(make_int4(s, z0, x0, 0));
    b->ntile_items = (int)b->items.size();
    for (int s = 0; s < (int)b->shots.size(); s++)
        for (int r = 0; r < b->shots[s].nr; r += kBatchRecBlock) b->items.push_back(make_int4(s, r, 0, 1));
}

static awe_status upload_items(awe_batch *b) {
    if (b->d_items) {
        cudaFree(b->d_items);
        b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), (void *)b->d_items));
        b->d_items = nullptr;
    }
    awe_status st = balloc(b, (void **)&b->d_items, b->items.size() * sizeof(int4));
    if (st != AWE_OK) return st;
    CUDA_TRY(cudaMemcpy(b->d_items, b->items.data(), b->items.size() * sizeof(int4), cudaMemcpyHostToDevice));
    return AWE_OK;
}

// column items (shot, x0) for chunks of L columns, then the receiver items
static awe_status build_col_items(awe_batch *b, int L) {
    b->col_items.clear();
    for (int s = 0; s < (int)b->shots.size(); s++)
        for (int x0 = 0; x0 < b->shots[s].n2; x0 += L) b->col_items.push_back(make_int4(s, 0, x0, 0));
    b->ncol_items = (int)b->col_items.size();
    for (int s = 0; s < (int)b->shots.size(); s++)
        for (int r = 0; r < b->shots[s].nr; r += kBatchRecBlock) b->col_items.push_back(make_int4(s, r, 0, 1));
    if (b->d_col_items) {
        cudaFree(b->d_col_items);
        b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), (void *)b->d_col_items));
        b->d_col_items = nullptr;
    }
    awe_status st = balloc(b, (void **)&b->d_col_items, b->col_items.size() * sizeof(int4));
    if (st != AWE_OK) return st;
    CUDA_TRY(cudaMemcpy(b->d_col_items, b->col_items.data(), b->col_items.size() * sizeof(int4),
                        cudaMemcpyHostToDevice));
    b->colL = L;
    return AWE_OK;
}

static BatchStep step_params(const awe_batch *b, int it) {
    BatchStep p{};
    // level it lives in u[it & 1] (cur); the new level overwrites u[(it + 1) & 1]
    p.cur = b->u[it & 1];
    p.nxt = b->u[(it + 1) & 1];
    p.vel = b->vel;
    p.wz = b->wz;
    p.wx = b->wx;
    p.sponge = b->d.dabc ? 1 : 0;
    p.n1 = b->n1;
    p.c0 = b->k.c0;
    for (int i = 0; i <= kMaxNop; i++) {
        p.cz[i] = b->k.c[0][i];
        p.cx[i] = b->k.c[1][i];
    }
    p.src = b->src;
    p.rec = b->rec;
    p.wav = b->wav;
    p.it = it;
    p.dat = b->dat;
    p.row = (it % b->d.jdata == 0) ? it / b->d.jdata : -1;
    return p;
}

// one forward step with the chosen kernel; without receivers: the column or
// tile items alone (the gradient's recompute)
static void launch_fwd(awe_batch *b, const BatchStep &p, cudaStream_t s, bool receivers) {
    if (b->colL > 0)
        launch_batch2d_col(b->d_shots, b->d_col_items, receivers ? (int)b->col_items.size() : b->ncol_items,
                           b->col_grid, b->colL, p, b->d_err, s);
    else
        launch_batch2d(b->nop, b->tile, b->d_shots, b->d_items, receivers ? (int)b->items.size() : b->ntile_items,
                       b->grid, p, s);
}

static void launch_range(awe_batch *b, int it0, int it1, cudaStream_t s) {
    for (int it = it0; it < it1; it++) {
        const BatchStep p = step_params(b, it);
        if (b->colL > 0)
            launch_batch2d_col(b->d_shots, b->d_col_items, (int)b->col_items.size(), b->col_grid, b->colL, p,
                               b->d_err, s);
        else
            launch_batch2d(b->nop, b->tile, b->d_shots, b->d_items, (int)b->items.size(), b->grid, p, s);
    }
}

static awe_status run_all(awe_batch *b, cudaStream_t s) {
    const size_t bytes = (size_t)b->cells * sizeof(float);
    CUDA_TRY(cudaMemsetAsync(b->u[0], 0, bytes, s));
    CUDA_TRY(cudaMemsetAsync(b->u[1], 0, bytes, s));
    CUDA_TRY(cudaMemsetAsync(b->d_err, 0, sizeof(int), s));
    if (!b->exec) {
        // capture the nt step launches once; replays reuse the same buffers
        cudaStream_t cs;
        CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            launch_range(b, 0, b->d.nt, cs);
            e = cudaStreamEndCapture(cs, &b->graph);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess) {
            drop_graph(b);
            set_error("CUDA graph capture of the batched time loop failed: %s", cudaGetErrorString(e));
            return AWE_ERR_CUDA;
        }
    }
    CUDA_TRY(cudaGraphLaunch(b->exec, s));
    b->launches = b->d.nt;
    return AWE_OK;
}

extern "C" {

awe_status awe_batch_create(const awe_desc *desc, int nshots, const awe_shot *shots, int device, awe_batch **out) {
    if (!desc || !shots || !out || nshots <= 0) {
        set_error("null descriptor, shots or output, or no shots");
        return AWE_ERR_INVALID;
    }
    *out = nullptr;
    const awe_desc &d = *desc;
    if (d.scheme != AWE_SCHEME_CPU || d.coords != AWE_CART || d.ndim != 2) {
        set_error("awe_batch: 2D cartesian, scheme AWE_SCHEME_CPU only");
        return AWE_ERR_UNSUPPORTED;
    }
    if (d.hybrid || d.precision != AWE_FAST || d.jsnap > 0) {
        set_error("awe_batch: no hybrid ABC, no snapshots, AWE_FAST only");
        return AWE_ERR_UNSUPPORTED;
    }
    const int fdorder = d.fdorder ? d.fdorder : 4;
    if (fdorder < 2 || fdorder > 16 || fdorder % 2 || d.nt < 1 || d.dt <= 0 || d.n[0] < 1 || d.n[1] < 1 ||
        d.jdata < 1) {
        set_error("awe_batch: bad descriptor (fdorder 2..16 even, nt >= 1, dt > 0, jdata >= 1)");
        return AWE_ERR_INVALID;
    }
    for (int s = 0; s < nshots; s++) {
        const awe_shot &sh = shots[s];
        if (sh.x0 < 0 || sh.nx < 1 || sh.x0 + sh.nx > d.n[1] || sh.ns < 0 || sh.nr < 0 ||
            (sh.ns > 0 && !sh.sou) || (sh.nr > 0 && !sh.rec)) {
            set_error("awe_batch: shot %d: window [%d, %d) outside the model's %d columns or bad points", s, sh.x0,
                      sh.x0 + sh.nx, d.n[1]);
            return AWE_ERR_INVALID;
        }
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        set_error("no CUDA device %d", device);
        return AWE_ERR_NODEVICE;
    }
    awe_batch *b = new awe_batch();
    b->d = d;
    b->d.fdorder = fdorder;
    b->device = device;
    b->nop = fdorder / 2;
    int nb = d.nb;
    if (nb < b->nop) nb = b->nop;  // MAWEFDcart2Dcpu.c:211
    b->nb = nb;
    b->n1 = d.n[0] + 2 * nb;
    if (b->n1 % 4) {
        delete b;
        set_error("awe_batch: nz + 2 nb must be a multiple of 4 (16-byte rows)");
        return AWE_ERR_UNSUPPORTED;
    }
    float dd[3] = {d.d[0], d.d[1], 1.f};
    fd_coefficients(b->nop, 2, dd, d.optfd, b->k);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device);
    b->grid = 4 * std::max(b->sms, 1);
    b->shots_in.assign(shots, shots + nshots);
    cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);

    // layout: shot s occupies (nx_s + 2 nb) columns of n1 floats
    std::vector<float> w;
    if (d.dabc) sponge_weights(nb, w);
    auto table = [&](int n) {
        std::vector<float> t(n, 1.f);
        if (d.dabc)
            for (int i = 0; i < nb && i < n; i++) t[i] = t[n - 1 - i] = w[nb - i - 1];
        return t;
    };
    b->h_wz = table(b->n1);
    long long off = 0, doff = 0;
    b->nsmp = (d.nt - 1) / d.jdata + 1;
    std::vector<GeoPoint> hs, hr;
    for (int s = 0; s < nshots; s++) {
        const awe_shot &in = shots[s];
        BatchShot sh{};
        sh.off = off;
        sh.n2 = in.nx + 2 * nb;
        sh.wx_off = (int)b->h_wx.size();
        std::vector<float> tx = table(sh.n2);
        b->h_wx.insert(b->h_wx.end(), tx.begin(), tx.end());
        // the window's padded origin (fdutil_init on the cropped axes)
        const float oz = d.o[0] - nb * d.d[0], ox = d.o[1] + in.x0 * d.d[1] - nb * d.d[1];
        FdmAxes f{oz, ox, 0.f, d.d[0], d.d[1], 1.f, b->n1, sh.n2, 1};
        auto point = [&](const float *xz) {
            Lint l = lint_make(2, xz[0], 0.f, xz[1], f);
            GeoPoint g{};
            g.base = (long long)l.jx * b->n1 + l.jz;
            for (int c = 0; c < 4; c++) g.w[c] = l.w[c];
            return g;
        };
        sh.ns = in.ns;
        sh.src0 = (int)hs.size();
        for (int i = 0; i < in.ns; i++) hs.push_back(point(in.sou + 2 * i));
        sh.nr = in.nr;
        sh.rec0 = (int)hr.size();
        for (int i = 0; i < in.nr; i++) hr.push_back(point(in.rec + 2 * i));
        sh.dat_off = doff;
        doff += (long long)b->nsmp * in.nr;
        off += (long long)sh.n2 * b->n1;
        b->shots.push_back(sh);
    }
    b->cells = off;
    b->ndat = doff;
    b->h_rec = hr;
    awe_status st = AWE_OK;
    const size_t cb = (size_t)off * sizeof(float);
    for (void **p : {(void **)&b->u[0], (void **)&b->u[1], (void **)&b->vel})
        if (st == AWE_OK) st = balloc(b, p, cb);
    if (st == AWE_OK) st = balloc(b, (void **)&b->wz, b->h_wz.size() * sizeof(float));
    if (st == AWE_OK) st = balloc(b, (void **)&b->wx, b->h_wx.size() * sizeof(float));
    if (st == AWE_OK) st = balloc(b, (void **)&b->wav, (size_t)d.nt * sizeof(float));
    if (st == AWE_OK) st = balloc(b, (void **)&b->dat, (size_t)std::max(doff, 1LL) * sizeof(float));
    if (st == AWE_OK) st = balloc(b, (void **)&b->d_shots, b->shots.size() * sizeof(BatchShot));
    if (st == AWE_OK) st = balloc(b, (void **)&b->src, std::max<size_t>(hs.size(), 1) * sizeof(GeoPoint));
    if (st == AWE_OK) st = balloc(b, (void **)&b->rec, std::max<size_t>(hr.size(), 1) * sizeof(GeoPoint));
    if (st == AWE_OK) st = balloc(b, (void **)&b->d_err, sizeof(int));
    if (st == AWE_OK && cudaMemset(b->d_err, 0, sizeof(int)) != cudaSuccess) st = AWE_ERR_CUDA;
    if (st == AWE_OK) {
        cudaMemcpy(b->wz, b->h_wz.data(), b->h_wz.size() * sizeof(float), cudaMemcpyHostToDevice);
        cudaMemcpy(b->wx, b->h_wx.data(), b->h_wx.size() * sizeof(float), cudaMemcpyHostToDevice);
        cudaMemcpy(b->d_shots, b->shots.data(), b->shots.size() * sizeof(BatchShot), cudaMemcpyHostToDevice);
        if (!hs.empty()) cudaMemcpy(b->src, hs.data(), hs.size() * sizeof(GeoPoint), cudaMemcpyHostToDevice);
        if (!hr.empty()) cudaMemcpy(b->rec, hr.data(), hr.size() * sizeof(GeoPoint), cudaMemcpyHostToDevice);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("batch upload failed: %s", cudaGetErrorString(e));
            st = AWE_ERR_CUDA;
        }
    }
    if (st == AWE_OK) {
        build_items(b);
        st = upload_items(b);
    }
    if (st != AWE_OK) {
        awe_batch_destroy(b);
        return st;
    }
    *out = b;
    return AWE_OK;
}

awe_status awe_batch_destroy(awe_batch *b) {
    if (!b) return AWE_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    for (void *p : b->allocs) cudaFree(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return AWE_OK;
}

awe_status awe_batch_set_model(awe_batch *b, const float *vel) {
    if (!b || !vel) {
        set_error("null batch or model");
        return AWE_ERR_INVALID;
    }
    CUDA_TRY(cudaSetDevice(b->device));
    const awe_desc &d = b->d;
    const int nz = d.n[0];
    std::vector<float> all((size_t)b->cells);
    const float dt2 = d.dt * d.dt;
    for (size_t s = 0; s < b->shots.size(); s++) {
        const awe_shot &in = b->shots_in[s];
        const BatchShot &sh = b->shots[s];
        // window, padded by edge replication (expand2d, fdutil.c:435-458), then v^2 dt^2
        const int n[2] = {nz, in.nx};
        expand_model(2, vel + (size_t)in.x0 * nz, all.data() + sh.off, b->nb, n);
        float *v = all.data() + sh.off;
        for (long long i = 0; i < (long long)sh.n2 * b->n1; i++) v[i] *= v[i] * dt2;  // MAWEFDcart2Dcpu.c:290
        if (d.fsrf)
            for (int x = 0; x < sh.n2; x++)
                for (int z = 0; z < b->nb + 1 && z < b->n1; z++) v[(size_t)x * b->n1 + z] = 0.f;  // :292-295
    }
    CUDA_TRY(cudaMemcpy(b->vel, all.data(), all.size() * sizeof(float), cudaMemcpyHostToDevice));
    b->model_set = true;
    return AWE_OK;
}

awe_status awe_batch_forward_device(awe_batch *b, const float *d_wav, float *d_dat, void *stream) {
    if (!b || !d_wav || !d_dat) {
        set_error("null batch, wavelet or data pointer");
        return AWE_ERR_INVALID;
    }
    if (!b->model_set) {
        set_error("awe_batch_set_model must precede awe_batch_forward");
        return AWE_ERR_STATE;
    }
    CUDA_TRY(cudaSetDevice(b->device));
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    CUDA_TRY(cudaMemcpyAsync(b->wav, d_wav, (size_t)b->d.nt * sizeof(float), cudaMemcpyDeviceToDevice, s));
    awe_status st = run_all(b, s);
    if (st != AWE_OK) return st;
    CUDA_TRY(cudaMemcpyAsync(d_dat, b->dat, (size_t)b->ndat * sizeof(float), cudaMemcpyDeviceToDevice, s));
    return AWE_OK;
}

awe_status awe_batch_forward(awe_batch *b, const float *wav, float *dat) {
    if (!b || !wav || !dat) {
        set_error("null batch, wavelet or data pointer");
        return AWE_ERR_INVALID;
    }
    if (!b->model_set) {
        set_error("awe_batch_set_model must precede awe_batch_forward");
        return AWE_ERR_STATE;
    }
    CUDA_TRY(cudaSetDevice(b->device));
    CUDA_TRY(cudaMemcpyAsync(b->wav, wav, (size_t)b->d.nt * sizeof(float), cudaMemcpyHostToDevice, b->stream));
    awe_status st = run_all(b, b->stream);
    if (st != AWE_OK) return st;
    CUDA_TRY(cudaMemcpyAsync(dat, b->dat, (size_t)b->ndat * sizeof(float), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    int bad = 0;
    CUDA_TRY(cudaMemcpy(&bad, b->d_err, sizeof bad, cudaMemcpyDeviceToHost));
    if (bad) {
        set_error("awe_batch_forward: a bulk-copy wait of the column kernel timed out; results are invalid");
        return AWE_ERR_CUDA;
    }
    return AWE_OK;
}

awe_status awe_batch_tune(awe_batch *b, int steps, int *tile_out, int *grid_out) {
    if (!b || steps < 1) {
        set_error("null batch or steps < 1");
        return AWE_ERR_INVALID;
    }
    if (!b->model_set) {
        set_error("awe_batch_set_model must precede awe_batch_tune");
        return AWE_ERR_STATE;
    }
    CUDA_TRY(cudaSetDevice(b->device));
    steps = std::min(steps, b->d.nt);
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_tile = b->tile, best_grid = b->grid;
    const size_t bytes = (size_t)b->cells * sizeof(float);
    for (int t = 0; t < kBatchNumTiles; t++) {
        b->tile = t;
        build_items(b);
        awe_status st = upload_items(b);
        if (st != AWE_OK) return st;
        for (int mult : {2, 4, 8, 16}) {
            b->grid = mult * b->sms;
            cudaMemsetAsync(b->u[0], 0, bytes, b->stream);
            cudaMemsetAsync(b->u[1], 0, bytes, b->stream);
            launch_range(b, 0, 1, b->stream);  // warm
            cudaEventRecord(e0, b->stream);
            launch_range(b, 0, steps, b->stream);
            cudaEventRecord(e1, b->stream);
            CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                best_tile = t;
                best_grid = b->grid;
            }
        }
    }
    // the column-march kernel: chunk lengths x (1, 2) persistent waves
    b->tile = best_tile;
    b->grid = best_grid;
    int best_col = 0, best_col_grid = 0;
    const int cpsm = batch2d_col_shape(b->nop, b->n1, nullptr) ? batch2d_col_ctas_per_sm(b->n1) : 0;
    for (int L : {16, 32, 64}) {
        if (cpsm <= 0) break;
        awe_status st = build_col_items(b, L);
        if (st != AWE_OK) return st;
        for (int mult : {1, 2}) {
            b->col_grid = mult * cpsm * b->sms;
            cudaMemsetAsync(b->u[0], 0, bytes, b->stream);
            cudaMemsetAsync(b->u[1], 0, bytes, b->stream);
            launch_range(b, 0, 1, b->stream);  // warm
            cudaEventRecord(e0, b->stream);
            launch_range(b, 0, steps, b->stream);
            cudaEventRecord(e1, b->stream);
            CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                best_col = L;
                best_col_grid = b->col_grid;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->colL = 0;
    if (best_col > 0) {
        awe_status st = build_col_items(b, best_col);
        if (st != AWE_OK) return st;
        b->col_grid = best_col_grid;
    }
    int bad = 0;
    CUDA_TRY(cudaMemcpy(&bad, b->d_err, sizeof bad, cudaMemcpyDeviceToHost));
    if (bad) {
        set_error("awe_batch_tune: a bulk-copy wait of the column kernel timed out");
        return AWE_ERR_CUDA;
    }
    build_items(b);
    awe_status st = upload_items(b);
    if (st != AWE_OK) return st;
    drop_graph(b);  // recaptured with the chosen shape on the next forward
    CUDA_TRY(cudaGetLastError());
    if (tile_out) *tile_out = b->colL > 0 ? kBatchNumTiles : best_tile;
    if (grid_out) *grid_out = b->colL > 0 ? b->col_grid : best_grid;
    return AWE_OK;
}

// receiver cells of every shot (cells the adjoint injects residuals into),
// each with its corners in (receiver, corner) order
static awe_status build_rec_cells(awe_batch *b) {
    std::vector<BatchRecCell> cells;
    std::vector<BatchRecW> ws;
    for (size_t s = 0; s < b->shots.size(); s++) {
        const BatchShot &sh = b->shots[s];
        std::map<long long, std::vector<BatchRecW>> per;
        for (int r = 0; r < sh.nr; r++) {
            const GeoPoint &g = b->h_rec[sh.rec0 + r];
            for (int c = 0; c < 4; c++) {
                const long long node = g.base + (c & 1) + (c >> 1) * (long long)b->n1;
                if (node < 0 || node >= (long long)sh.n2 * b->n1) continue;
                per[node].push_back(BatchRecW{r, g.w[c]});
            }
        }
        for (const auto &kv : per) {
            const int e0 = (int)ws.size();
            ws.insert(ws.end(), kv.second.begin(), kv.second.end());
            cells.push_back(BatchRecCell{sh.off + kv.first, (int)s, (int)(kv.first / b->n1), (int)(kv.first % b->n1),
                                         e0, (int)ws.size(), 0});
        }
    }
    for (void *q : {(void *)b->rec_cells, (void *)b->rec_ws}) {
        if (!q) continue;
        cudaFree(q);
        b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), q));
    }
    b->rec_cells = nullptr;
    b->rec_ws = nullptr;
    awe_status st = balloc(b, (void **)&b->rec_cells, std::max<size_t>(cells.size(), 1) * sizeof(BatchRecCell));
    if (st == AWE_OK) st = balloc(b, (void **)&b->rec_ws, std::max<size_t>(ws.size(), 1) * sizeof(BatchRecW));
    if (st != AWE_OK) return st;
    if (!cells.empty()) {
        CUDA_TRY(cudaMemcpy(b->rec_cells, cells.data(), cells.size() * sizeof(BatchRecCell), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(b->rec_ws, ws.data(), ws.size() * sizeof(BatchRecW), cudaMemcpyHostToDevice));
    }
    b->nrec_cells = (int)cells.size();
    return AWE_OK;
}

static awe_status grad_alloc(awe_batch *b, int T, int fmt) {
    if (b->gT == T && b->gfmt == fmt) return AWE_OK;
    for (void *q : {(void *)b->slots, b->ckpt, (void *)b->scales}) {
        if (!q) continue;
        cudaFree(q);
        b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), q));
    }
    b->slots = nullptr;
    b->ckpt = nullptr;
    b->scales = nullptr;
    const int nseg = (b->d.nt + T - 1) / T;
    const size_t es = fmt == AWE_CKPT_FP32 ? 4 : 2;
    awe_status st = balloc(b, (void **)&b->slots, (size_t)(T + 1) * b->cells * sizeof(float));
    if (st == AWE_OK) st = balloc(b, &b->ckpt, (size_t)2 * nseg * b->cells * es);
    b->gscale_per = fmt == AWE_CKPT_BFP16 ? (b->cells + kBfpBlock - 1) / kBfpBlock : (long long)b->shots.size();
    if (st == AWE_OK) st = balloc(b, (void **)&b->scales, (size_t)2 * nseg * b->gscale_per * sizeof(float));
    if (st != AWE_OK) return st;
    if (!b->gX) {
        const size_t cb = (size_t)b->cells * sizeof(float);
        const size_t nd = (size_t)std::max(b->ndat, 1LL);
        for (void **q : {(void **)&b->gX, (void **)&b->gY})
            if (st == AWE_OK) st = balloc(b, q, cb);
        if (st == AWE_OK) st = balloc(b, (void **)&b->G, (size_t)b->cells * sizeof(float2));
        if (st == AWE_OK) st = balloc(b, (void **)&b->res, nd * sizeof(float));
        if (st == AWE_OK) st = balloc(b, (void **)&b->dobs, nd * sizeof(float));
        if (st == AWE_OK) st = balloc(b, (void **)&b->part, ((nd + 1023) / 1024) * sizeof(double));
        if (st == AWE_OK) st = balloc(b, (void **)&b->grad, (size_t)b->d.n[0] * b->d.n[1] * sizeof(double));
        if (st == AWE_OK) st = balloc(b, (void **)&b->win, b->shots.size() * sizeof(int2));
        if (st != AWE_OK) return st;
        std::vector<int2> w(b->shots.size());
        for (size_t s = 0; s < w.size(); s++) w[s] = make_int2(b->shots_in[s].x0, b->shots_in[s].nx);
        CUDA_TRY(cudaMemcpy(b->win, w.data(), w.size() * sizeof(int2), cudaMemcpyHostToDevice));
    }
    b->gT = T;
    b->gfmt = fmt;
    b->gseg = nseg;
    return AWE_OK;
}

static BatchAdj adj_params(const awe_batch *b, int it, const float *V) {
    BatchAdj p{};
    p.V = V;
    p.vel = b->vel;
    p.G = b->G;
    p.wz = b->wz;
    p.wx = b->wx;
    p.sponge = b->d.dabc ? 1 : 0;
    p.n1 = b->n1;
    p.c0 = b->k.c0;
    for (int i = 0; i <= kMaxNop; i++) {
        p.cz[i] = b->k.c[0][i];
        p.cx[i] = b->k.c[1][i];
    }
    p.src = b->src;
    p.wav = b->wav;
    p.it = it;
    p.res = b->res;
    p.row = (it % b->d.jdata == 0) ? it / b->d.jdata : -1;
    return p;
}

// the whole gradient as one launch sequence on stream s (capturable)
static awe_status grad_sequence(awe_batch *b, cudaStream_t s) {
    const long long cells = b->cells;
    const size_t cb = (size_t)cells * sizeof(float);
    const int T = b->gT, ns = (int)b->shots.size();
    const size_t es = b->gfmt == AWE_CKPT_FP32 ? 4 : 2;
    auto ck = [&](int idx) { return (void *)((char *)b->ckpt + (size_t)idx * cells * es); };
    auto sc = [&](int idx) { return b->scales + (size_t)idx * b->gscale_per; };
    // forward with checkpoints of both levels at every segment start
    CUDA_TRY(cudaMemsetAsync(b->d_err, 0, sizeof(int), s));
    CUDA_TRY(cudaMemsetAsync(b->u[0], 0, cb, s));
    CUDA_TRY(cudaMemsetAsync(b->u[1], 0, cb, s));
    for (int it = 0; it < b->d.nt; it++) {
        BatchStep p = step_params(b, it);
        if (it % T == 0) {
            const int seg = it / T;
            launch_batch_ckpt(true, b->gfmt, b->d_shots, ns, p.nxt, ck(2 * seg), sc(2 * seg), b->n1, cells, s);
            launch_batch_ckpt(true, b->gfmt, b->d_shots, ns, (float *)p.cur, ck(2 * seg + 1), sc(2 * seg + 1), b->n1,
                              cells, s);
        }
        launch_fwd(b, p, s, true);
    }
    launch_residual_flat(b->dat, b->dobs, b->res, b->ndat, b->part, s);
    // adjoint sweep, last segment first
    CUDA_TRY(cudaMemsetAsync(b->gX, 0, cb, s));
    CUDA_TRY(cudaMemsetAsync(b->gY, 0, cb, s));
    CUDA_TRY(cudaMemsetAsync(b->G, 0, (size_t)cells * sizeof(float2), s));
    float *X = b->gX, *Y = b->gY;
    for (int seg = b->gseg - 1; seg >= 0; seg--) {
        const int k0 = seg * T, k1 = std::min(k0 + T, b->d.nt);
        launch_batch_ckpt(false, b->gfmt, b->d_shots, ns, b->slots, ck(2 * seg), sc(2 * seg), b->n1, cells, s);
        launch_batch_ckpt(false, b->gfmt, b->d_shots, ns, b->slots + cells, ck(2 * seg + 1), sc(2 * seg + 1), b->n1,
                          cells, s);
        for (int k = k0; k <= k1 - 2; k++) {
            const int j = k - k0;
            BatchStep p = step_params(b, k);
            p.prv = b->slots + (size_t)j * cells;
            p.cur = b->slots + (size_t)(j + 1) * cells;
            p.nxt = b->slots + (size_t)(j + 2) * cells;
            p.row = -1;
            launch_fwd(b, p, s, false);
        }
        for (int k = k1 - 1; k >= k0; k--) {
            BatchAdj p = adj_params(b, k, b->slots + (size_t)(k - k0 + 1) * cells);
            p.X = X;
            p.Y = Y;
            if (b->colL > 0 && b->col_adj_grid > 0)
                launch_batch2d_col_adj(b->d_shots, b->d_col_items, b->ncol_items, b->col_adj_grid, b->colL, p,
                                       b->d_err, s);
            else
                launch_batch2d_adj(b->nop, b->tile, b->d_shots, b->d_items, b->ntile_items, b->grid, p, s);
            launch_batch_rec_adj(b->rec_cells, b->nrec_cells, b->rec_ws, b->d_shots, p, s);
            std::swap(X, Y);
        }
    }
    launch_batch_grad_fold(b->d_shots, b->win, ns, b->G, b->vel, b->d.dt, b->n1, b->nb, b->d.n[0], b->d.n[1],
                           b->grad, s);
    return AWE_OK;
}

awe_status awe_batch_gradient(awe_batch *b, const float *wav, const float *dobs, const awe_grad_opts *opts,
                              double *grad, double *misfit) {
    if (!b || !wav || !dobs || !grad || !misfit) {
        set_error("null batch, wavelet, data, gradient or misfit pointer");
        return AWE_ERR_INVALID;
    }
    if (!b->model_set) {
        set_error("awe_batch_set_model must precede awe_batch_gradient");
        return AWE_ERR_STATE;
    }
    awe_grad_opts o{0, AWE_CKPT_BFP16};
    if (opts) o = *opts;
    if (o.ckpt_format != AWE_CKPT_BF16 && o.ckpt_format != AWE_CKPT_FP32 && o.ckpt_format != AWE_CKPT_FP16 &&
        o.ckpt_format != AWE_CKPT_BFP16) {
        set_error("awe_batch_gradient: unknown checkpoint format %d", o.ckpt_format);
        return AWE_ERR_INVALID;
    }
    CUDA_TRY(cudaSetDevice(b->device));
    int T = o.ckpt_every > 0 ? o.ckpt_every : (int)std::ceil(std::sqrt((double)b->d.nt));
    T = std::max(1, std::min(T, b->d.nt));
    awe_status st = grad_alloc(b, T, o.ckpt_format);
    if (st == AWE_OK && b->nrec_cells < 0) st = build_rec_cells(b);
    if (st == AWE_OK) {
        const int cpsm = b->colL > 0 ? batch2d_col_adj_ctas_per_sm(b->n1) : 0;
        b->col_adj_grid = cpsm > 0 ? cpsm * b->sms : 0;
    }
    if (st != AWE_OK) return st;
    cudaStream_t s = b->stream;
    CUDA_TRY(cudaMemcpyAsync(b->wav, wav, (size_t)b->d.nt * sizeof(float), cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(b->dobs, dobs, (size_t)b->ndat * sizeof(float), cudaMemcpyHostToDevice, s));
    st = grad_sequence(b, s);
    if (st != AWE_OK) return st;
    const size_t nparts = (size_t)((b->ndat + 1023) / 1024);
    std::vector<double> parts(nparts);
    if (nparts) CUDA_TRY(cudaMemcpyAsync(parts.data(), b->part, nparts * sizeof(double), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(grad, b->grad, (size_t)b->d.n[0] * b->d.n[1] * sizeof(double), cudaMemcpyDeviceToHost,
                             s));
    CUDA_TRY(cudaStreamSynchronize(s));
    CUDA_TRY(cudaGetLastError());
    int bad = 0;
    CUDA_TRY(cudaMemcpy(&bad, b->d_err, sizeof bad, cudaMemcpyDeviceToHost));
    if (bad) {
        set_error("awe_batch_gradient: a bulk-copy wait of the column kernel timed out; results are invalid");
        return AWE_ERR_CUDA;
    }
    double J = 0;
    for (double v : parts) J += 0.5 * v;
    *misfit = J;
    return AWE_OK;
}

awe_status awe_batch_select(awe_batch *b, int kernel, int chunk, int grid) {
    if (!b || kernel < 0 || kernel > kBatchNumTiles) {
        set_error("awe_batch_select: kernel must be 0-%d", kBatchNumTiles);
        return AWE_ERR_INVALID;
    }
    CUDA_TRY(cudaSetDevice(b->device));
    drop_graph(b);
    if (kernel < kBatchNumTiles) {
        b->tile = kernel;
        b->grid = grid > 0 ? grid : 4 * std::max(b->sms, 1);
        b->colL = 0;
        build_items(b);
        return upload_items(b);
    }
    if (chunk < 1 || !batch2d_col_shape(b->nop, b->n1, nullptr)) {
        set_error("awe_batch_select: the column march needs 8th order, nz + 2 nb <= 2048 and chunk >= 1");
        return AWE_ERR_UNSUPPORTED;
    }
    const int cpsm = batch2d_col_ctas_per_sm(b->n1);
    if (cpsm < 1) {
        set_error("awe_batch_select: the column march does not fit on this device");
        return AWE_ERR_UNSUPPORTED;
    }
    awe_status st = build_col_items(b, chunk);
    if (st != AWE_OK) return st;
    b->col_grid = grid > 0 ? grid : cpsm * b->sms;
    return AWE_OK;
}

awe_status awe_batch_info(const awe_batch *b, awe_batch_info_t *info) {
    if (!b || !info) {
        set_error("null argument");
        return AWE_ERR_INVALID;
    }
    info->nshots = (int)b->shots.size();
    info->nsmp = b->nsmp;
    info->total_samples = b->ndat;
    info->cells = b->cells;
    if (b->colL > 0) {  // column march: whole columns, chunks of colL
        info->tile_z = b->n1;
        info->tile_x = b->colL;
        info->grid = b->col_grid;
        info->work_items = (int)b->col_items.size();
    } else {
        info->tile_z = kBatchTiles[b->tile][0];
        info->tile_x = kBatchTiles[b->tile][1];
        info->grid = b->grid;
        info->work_items = (int)b->items.size();
    }
    info->launches_per_forward = b->d.nt;
    return AWE_OK;
}

}  // extern "C"
