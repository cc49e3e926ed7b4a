// Misfit gradient of the CPU-program scheme: forward pass with checkpoints,
// then, segment by segment from the last, recompute of the forward levels
// from the segment's checkpoint and the adjoint sweep over them.
//
// Memory (cells = padded grid): 2 forward levels + vel (the plan's), segment
// levels (ckpt_every + 1) x 4 B, checkpoints 2 x ceil(nt / ckpt_every) x 2 B
// (BF16, FP16) or 4 B, adjoint 2 x 4 B, ABC transpose scratch 4 B (3D), gradient 8 B.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "awe_internal.h"
#include "plan_impl.h"

namespace awe {

#define CUDA_TRY(expr)                                                                            \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return AWE_ERR_CUDA;                                                                  \
        }                                                                                         \
    } while (0)
#define AWE_TRY(expr)                \
    do {                             \
        awe_status s_ = (expr);      \
        if (s_ != AWE_OK) return s_; \
    } while (0)

struct GradState {
    int T = 0, nseg = 0, fmt = -1;
    // generic path: (T + 1) segment levels V_k; TMA path: T slots of L(V_k)
    float *slots = nullptr;
    void *ckpt = nullptr;    // 2 * nseg levels
    float *scales = nullptr; // 2 * nseg (BF16/FP16), 2 * nseg * blocks (block floating point)
    long long nblk = 0;      // scale blocks per level (block floating point)
    unsigned int *amax = nullptr;
    float *X = nullptr, *Y = nullptr, *kap = nullptr;
    float2 *G = nullptr;  // gradient / image accumulators (compensated pairs)
    float *dat = nullptr, *r = nullptr;
    double *row_sum = nullptr;
    // TMA path (3D, 8th order): three rolling forward levels, I vel2 nu, and
    // the tensor maps of every buffer the TMA kernels read
    bool tma = false;
    float *vr = nullptr, *gbuf = nullptr;
    CUtensorMap vr_halo[3], vr_tile[3], g_halo, x_tile, y_tile;
    // TMA path of the spherical scheme (AWE_FAST): halo and tile maps of the
    // T + 1 recompute slots stacked along phi, halo maps of X, Y and v
    bool sph = false;
    CUtensorMap sl_halo, sl_tile, xy_halo[2], xy_tile[2], v_halo, g_tile;
    // receiver / source corners by padded cell for the fused adjoint step
    int *rc_start = nullptr, *sc_start = nullptr;
    int2 *rc_ent = nullptr, *sc_ent = nullptr;
    size_t rc_cap = 0, sc_cap = 0;
    bool lists_ok = false;  // cleared when the geometry changes
    size_t nd_cap = 0;      // trace samples dat and r hold
    // misfit rows (pinned, written by the stream) and the captured gradient
    double *h_rows = nullptr;
    size_t h_rows_n = 0;
    cudaGraphExec_t gexec = nullptr;
    // settings of the captured graph, or of the last direct run (captured when
    // a second call repeats them: a one-off call pays no capture)
    const void *g_key[4] = {nullptr, nullptr, nullptr, nullptr};
    int g_ncs = 0, g_image = -2;
    bool g_seen = false;
    long long g_launches = 0;
};

void plan_gradient_graph_drop(awe_plan *p) {
    if (!p->grad) return;
    GradState *st = p->grad;
    if (st->gexec) cudaGraphExecDestroy(st->gexec);
    st->gexec = nullptr;
    st->g_seen = false;
    st->lists_ok = false;
}

void plan_gradient_free(awe_plan *p) {
    if (!p->grad) return;
    plan_gradient_graph_drop(p);
    GradState *st = p->grad;
    if (st->h_rows) cudaFreeHost(st->h_rows);
    for (void *ptr : {(void *)st->slots, st->ckpt, (void *)st->scales, (void *)st->amax, (void *)st->X, (void *)st->Y,
                      (void *)st->kap, (void *)st->G, (void *)st->dat, (void *)st->r, (void *)st->row_sum,
                      (void *)st->vr, (void *)st->gbuf, (void *)st->rc_start, (void *)st->sc_start,
                      (void *)st->rc_ent, (void *)st->sc_ent})
        if (ptr) dev_free(p, ptr);
    delete st;
    p->grad = nullptr;
}

static awe_status grad_alloc(awe_plan *p, int T, int fmt) {
    const size_t nd = (size_t)p->nsmp * (p->nr > 0 ? p->nr : 1);
    if (p->grad && p->grad->T == T && p->grad->fmt == fmt && p->grad->nd_cap >= nd) return AWE_OK;
    plan_gradient_free(p);
    GradState *st = new GradState();
    p->grad = st;
    const awe_desc &d = p->d;
    const size_t cells = (size_t)p->g.cells();
    st->T = T;
    st->fmt = fmt;
    st->nseg = (d.nt + T - 1) / T;
    const size_t es = fmt == AWE_CKPT_FP32 ? 4 : 2;
    st->tma = p->use_tma && d.precision == AWE_FAST;
    AWE_TRY(dev_alloc(p, (void **)&st->slots, (size_t)(st->tma ? T : T + 1) * cells * sizeof(float)));
    AWE_TRY(dev_alloc(p, &st->ckpt, (size_t)2 * st->nseg * cells * es));
    st->nblk = fmt == AWE_CKPT_BFP16 ? ((long long)cells + kBfpBlock - 1) / kBfpBlock : 1;
    AWE_TRY(dev_alloc(p, (void **)&st->scales, (size_t)2 * st->nseg * st->nblk * sizeof(float)));
    AWE_TRY(dev_alloc(p, (void **)&st->amax, sizeof(unsigned int)));
    AWE_TRY(dev_alloc(p, (void **)&st->X, cells * sizeof(float)));
    AWE_TRY(dev_alloc(p, (void **)&st->Y, cells * sizeof(float)));
    if (d.ndim == 3 && d.dabc && d.scheme == AWE_SCHEME_CPU) AWE_TRY(dev_alloc(p, (void **)&st->kap, cells * sizeof(float)));
    AWE_TRY(dev_alloc(p, (void **)&st->G, cells * sizeof(float2)));
    st->nd_cap = nd;
    AWE_TRY(dev_alloc(p, (void **)&st->dat, nd * sizeof(float)));
    AWE_TRY(dev_alloc(p, (void **)&st->r, nd * sizeof(float)));
    AWE_TRY(dev_alloc(p, (void **)&st->row_sum, (size_t)p->nsmp * sizeof(double)));
    if (st->tma) {
        AWE_TRY(dev_alloc(p, (void **)&st->vr, 3 * cells * sizeof(float)));
        AWE_TRY(dev_alloc(p, (void **)&st->gbuf, cells * sizeof(float)));
        int h1, h2, t1, t2;
        stepB3_tma_boxes(&h1, &h2, &t1, &t2);
        const Grid &g = p->g;
        bool ok = true;
        for (int j = 0; j < 3; j++) {
            const float *b = st->vr + (size_t)j * cells;
            ok = ok && make_tmap_3d(&st->vr_halo[j], b, g.n1, g.n2, g.n3, h1, h2) &&
                 make_tmap_3d(&st->vr_tile[j], b, g.n1, g.n2, g.n3, t1, t2);
        }
        ok = ok && make_tmap_3d(&st->g_halo, st->gbuf, g.n1, g.n2, g.n3, h1, h2) &&
             make_tmap_3d(&st->x_tile, st->X, g.n1, g.n2, g.n3, t1, t2) &&
             make_tmap_3d(&st->y_tile, st->Y, g.n1, g.n2, g.n3, t1, t2);
        if (!ok) {
            set_error("awe_gradient: tensor map encoding failed");
            return AWE_ERR_CUDA;
        }
    }
    if (p->sph_tma) {
        st->sph = sphA_tma_level_maps(&st->sl_halo, &st->sl_tile, st->slots, p->g, T + 1) &&
                  sphA_tma_level_maps(&st->xy_halo[0], &st->xy_tile[0], st->X, p->g, 1) &&
                  sphA_tma_level_maps(&st->xy_halo[1], &st->xy_tile[1], st->Y, p->g, 1) &&
                  sphA_tma_level_maps(&st->v_halo, nullptr, p->vel, p->g, 1) &&
                  sphA_tma_pair_map(&st->g_tile, st->G, p->g);
        if (!st->sph) {
            set_error("awe_gradient: tensor map encoding failed");
            return AWE_ERR_CUDA;
        }
    }
    return AWE_OK;
}

static int float_bits(float f) {
    int i;
    std::memcpy(&i, &f, sizeof i);
    return i;
}

// corners of `pts` grouped by padded cell (counting sort, each cell's
// entries in (point, corner) order) into start[cells + 1] and ent
static awe_status build_cell_lists(awe_plan *p, const std::vector<GeoPoint> &pts, int nc, int **start, int2 **ent,
                                   size_t *cap, cudaStream_t s) {
    const long long cells = p->g.cells();
    std::vector<int> cnt((size_t)cells + 1, 0);
    for (const GeoPoint &pt : pts)
        for (int c = 0; c < nc; c++) {
            const long long n = pt.base + p->h_corner_off[c];
            if (n >= 0 && n < cells) cnt[(size_t)n + 1]++;
        }
    for (long long i = 0; i < cells; i++) cnt[(size_t)i + 1] += cnt[(size_t)i];
    std::vector<int2> e(std::max<size_t>((size_t)cnt[(size_t)cells], 1));
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (size_t k = 0; k < pts.size(); k++)
        for (int c = 0; c < nc; c++) {
            const long long n = pts[k].base + p->h_corner_off[c];
            if (n >= 0 && n < cells) e[(size_t)fill[(size_t)n]++] = make_int2((int)k, float_bits(pts[k].w[c]));
        }
    if (!*start) AWE_TRY(dev_alloc(p, (void **)start, ((size_t)cells + 1) * sizeof(int)));
    if (*cap < e.size()) {
        if (*ent) dev_free(p, *ent);
        *ent = nullptr;
        AWE_TRY(dev_alloc(p, (void **)ent, e.size() * sizeof(int2)));
        *cap = e.size();
    }
    CUDA_TRY(cudaMemcpyAsync(*start, cnt.data(), cnt.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(*ent, e.data(), e.size() * sizeof(int2), cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaStreamSynchronize(s));  // the host vectors go out of scope
    return AWE_OK;
}

static int grid_for(long long n) {
    long long b = (n + 255) / 256;
    return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

static awe_status ckpt_store(awe_plan *p, int idx, const float *u, cudaStream_t s) {
    GradState *st = p->grad;
    const long long cells = p->g.cells();
    if (st->fmt == AWE_CKPT_BFP16) {
        short *q = (short *)st->ckpt + (size_t)idx * cells;
        launch_ckpt_store_bfp(u, cells, q, st->scales + (size_t)idx * st->nblk, grid_for(cells), s);
    } else if (st->fmt != AWE_CKPT_FP32) {
        void *q = (char *)st->ckpt + (size_t)idx * cells * 2;
        launch_ckpt_store16(st->fmt == AWE_CKPT_FP16, u, cells, st->amax, q, st->scales + idx, grid_for(cells), s);
    } else {
        float *q = (float *)st->ckpt + (size_t)idx * cells;
        CUDA_TRY(cudaMemcpyAsync(q, u, (size_t)cells * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    return AWE_OK;
}

static awe_status ckpt_load(awe_plan *p, int idx, float *u, cudaStream_t s) {
    GradState *st = p->grad;
    const long long cells = p->g.cells();
    if (st->fmt == AWE_CKPT_BFP16) {
        const short *q = (const short *)st->ckpt + (size_t)idx * cells;
        launch_ckpt_load_bfp(q, st->scales + (size_t)idx * st->nblk, cells, u, grid_for(cells), s);
    } else if (st->fmt != AWE_CKPT_FP32) {
        const void *q = (const char *)st->ckpt + (size_t)idx * cells * 2;
        launch_ckpt_load16(st->fmt == AWE_CKPT_FP16, q, cells, st->scales + idx, u, grid_for(cells), s);
    } else {
        const float *q = (const float *)st->ckpt + (size_t)idx * cells;
        CUDA_TRY(cudaMemcpyAsync(u, q, (size_t)cells * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    return AWE_OK;
}

// Spherical GPU-program scheme (sfAWEFDspher3Dgpu's step, AWE_FAST).  Forward
// with the two levels stored at the start of every segment's first iteration
// (the previous level, sponge pending, and the current one before its
// injection); per segment, last first, the levels after injection A_k are
// recomputed out of place into slots 1..T (slot 0: A_{k0-1}); the adjoint
// sweep j = nt .. 0 keeps z_{j+1} and z_{j+2} in two buffers:
//   z_j = W M (L^T(I c z_{j+1}) + 2 z_{j+1} - W z_{j+2}) + W M R^T r_{j-1},
//   dJ/dc += z_{j+1} L(A_j),  c = dt^2 v^2, folded to dJ/dm = dJ/dc (-c^2/dt^2).
// image >= 0: awe_rtm's conditions (the data themselves back-propagated;
// AWE_IMAGE_XCORR sums z A on the model window, AWE_IMAGE_BORN the gradient formula)
// one TMA spherical step of the recompute: the current level at plane offset
// cur_f0 of `halo`, the previous at prv_f0 of `tile`, the new level into nxt
static awe_status sph_tma_step(awe_plan *p, const CUtensorMap &halo, const CUtensorMap &tile, float *nxt, int cur_f0,
                               int prv_f0, cudaStream_t s) {
    prof_begin(p, s);
    const cudaError_t e = launch_stepA_sph_tma(halo, tile, p->sph_maps[4], nxt, p->pa, p->sph_shape, p->sched_counter,
                                               p->sched_base, p->d_err, p->spin_limit, s, cur_f0, prv_f0);
    prof_end(p, s);
    p->sched_base += (unsigned long long)p->sph_shape.items + p->sph_shape.grid;
    if (e != cudaSuccess) {
        set_error("spherical TMA step launch failed: %s", cudaGetErrorString(e));
        return AWE_ERR_CUDA;
    }
    return AWE_OK;
}

static awe_status gradient_spher_one(awe_plan *p, const float *d_wav, int ncs, const float *d_dobs, int T, int fmt,
                                     double *d_grad, double *misfit, float *d_dsyn, cudaStream_t s, int image) {
    const awe_desc &d = p->d;
    const StepAParams &pa = p->pa;
    AWE_TRY(grad_alloc(p, T, fmt));
    GradState *st = p->grad;
    const Grid &g = p->g;
    const long long cells = g.cells();
    const size_t bytes = (size_t)cells * sizeof(float);
    float *dat = d_dsyn ? d_dsyn : st->dat;
    long long launches = 0;

    StepHook hook = [&](int it, const float *prev, const float *cur, cudaStream_t ss) -> awe_status {
        if (it % T != 0) return AWE_OK;
        const int seg = it / T;
        AWE_TRY(ckpt_store(p, 2 * seg, prev, ss));
        AWE_TRY(ckpt_store(p, 2 * seg + 1, cur, ss));
        return AWE_OK;
    };
    AWE_TRY(planA_run(p, d_wav, ncs, dat, nullptr, s, &hook));
    launches += p->launches;
    const bool xcorr = image == AWE_IMAGE_XCORR;
    std::vector<double> rows;
    if (image < 0) {
        launch_residual(dat, d_dobs, st->r, p->nsmp, p->nr, st->row_sum, s);
        rows.resize(p->nsmp);
        CUDA_TRY(cudaMemcpyAsync(rows.data(), st->row_sum, rows.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    } else if (p->nr > 0) {
        CUDA_TRY(cudaMemcpyAsync(st->r, d_dobs, (size_t)p->nsmp * p->nr * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }

    CUDA_TRY(cudaMemsetAsync(st->X, 0, bytes, s));
    CUDA_TRY(cudaMemsetAsync(st->Y, 0, bytes, s));
    CUDA_TRY(cudaMemsetAsync(st->G, 0, (size_t)cells * sizeof(float2), s));
    float *X = st->X, *Y = st->Y;
    // j = nt: z_nt = W M R^T r_{nt-1}
    launch_rec_adjA(Y, p->rec, p->nr, st->r + (size_t)(d.nt - 1) * p->nr, pa, p->corner_off, s);
    std::swap(X, Y);
    launches++;
    for (int seg = st->nseg - 1; seg >= 0; seg--) {
        const int k0 = seg * T, k1 = std::min(k0 + T, d.nt);
        float *slot = st->slots;  // slot[k - k0 + 1] = A_k
        AWE_TRY(ckpt_load(p, 2 * seg, slot, s));
        AWE_TRY(ckpt_load(p, 2 * seg + 1, slot + cells, s));
        for (int k = k0; k < k1; k++) {
            float *cur = slot + (size_t)(k - k0 + 1) * cells;
            launch_injectA(false, 3, cur, p->src, nullptr, p->ns, d_wav, k, false, p->corner_off, s, 1, ncs);
            if (k + 1 < k1) {
                if (st->sph) {  // slot i = k - k0 + 1 from slots i and i - 1, into slot i + 1
                    const int i = k - k0 + 1;
                    AWE_TRY(sph_tma_step(p, st->sl_halo, st->sl_tile, cur + cells, i * g.n3, (i - 1) * g.n3, s));
                } else {
                    prof_begin(p, s);
                    launch_stepA_oop(pa.geom, false, cur, cur - cells, cur + cells, p->vel, pa, s);
                    prof_end(p, s);
                }
            }
            launches += (p->ns > 0) + (k + 1 < k1);
        }
        for (int j = k1 - 1; j >= k0; j--) {
            if (st->sph) {
                const int ix = X == st->X ? 0 : 1;  // Y is the other buffer
                prof_begin(p, s, AWE_PROF_ADJOINT);
                const cudaError_t e = launch_adjA_sph_tma(
                    st->xy_halo[ix], st->v_halo, st->sl_halo, (j - k0 + 1) * g.n3, st->xy_tile[1 - ix], st->g_tile, Y,
                    st->G, pa, p->sph_shape, p->sched_counter, p->sched_base, p->d_err, p->spin_limit, xcorr, s);
                prof_end(p, s);
                p->sched_base += (unsigned long long)p->sph_shape.items + p->sph_shape.grid;
                if (e != cudaSuccess) {
                    set_error("spherical TMA adjoint launch failed: %s", cudaGetErrorString(e));
                    return AWE_ERR_CUDA;
                }
            } else {
                prof_begin(p, s, AWE_PROF_ADJOINT);
                launch_adjA_sph(X, Y, slot + (size_t)(j - k0 + 1) * cells, p->vel, st->G, pa, s, xcorr);
                prof_end(p, s);
            }
            launches++;
            if (j >= 1) {
                launch_rec_adjA(Y, p->rec, p->nr, st->r + (size_t)(j - 1) * p->nr, pa, p->corner_off, s);
                launches++;
            }
            std::swap(X, Y);
        }
    }
    if (xcorr) launch_image_cut(st->G, g, p->nbd, d.n, d.ndim, d_grad, s);
    else launch_grad_fold(st->G, p->vel, d.dt, g, p->nbd, d.n, d.ndim, d_grad, s, true);
    launches++;
    CUDA_TRY(cudaStreamSynchronize(s));
    double J = 0;
    for (double v : rows) J += 0.5 * v;
    *misfit = J;
    p->launches = launches;
    return AWE_OK;
}

// Several shots (awe_set_shots: points of shot s address field s): one shot
// after the other on the single-shot machinery, with the shot's points
// (bases moved back to field 0) and its columns of the data; gradients and
// misfits summed.
static awe_status plan_gradient_spher(awe_plan *p, const float *d_wav, int ncs, const float *d_dobs, int T, int fmt,
                                      double *d_grad, double *misfit, float *d_dsyn, cudaStream_t s, int image) {
    const awe_desc &d = p->d;
    if (d.expl) {
        set_error("awe_gradient: the reflectivity-scaled injection (expl=y) depends on the model; use expl=n");
        return AWE_ERR_UNSUPPORTED;
    }
    if (p->move_mode >= 0) {
        set_error("awe_gradient: fixed sources and receivers only");
        return AWE_ERR_UNSUPPORTED;
    }
    const int nshot = p->pa.nshot > 1 ? p->pa.nshot : 1;
    if (nshot == 1) return gradient_spher_one(p, d_wav, ncs, d_dobs, T, fmt, d_grad, misfit, d_dsyn, s, image);
    if (ncs != 1) {
        set_error("awe_gradient: the shots of awe_set_shots share one wavelet (ncs = 1)");
        return AWE_ERR_UNSUPPORTED;
    }
    const long long cells = p->g.cells();
    const int NS = p->ns, NR = p->nr;
    int max_nr = 1;
    for (int v : p->shot_nr) max_nr = std::max(max_nr, v);
    std::vector<GeoPoint> pts(p->h_src);
    pts.insert(pts.end(), p->h_rec.begin(), p->h_rec.end());
    {
        int a = 0;
        for (int q = 0; q < nshot; q++)
            for (int i = 0; i < p->shot_ns[q]; i++) pts[a++].base -= q * cells;
        for (int q = 0; q < nshot; q++)
            for (int i = 0; i < p->shot_nr[q]; i++) pts[a++].base -= q * cells;
    }
    const size_t mcells = (size_t)d.n[0] * d.n[1] * d.n[2];
    GeoPoint *d_pts = nullptr;
    float *dobs_s = nullptr, *dsyn_s = nullptr;
    double *grad_s = nullptr;
    GeoPoint *src0 = p->src, *rec0 = p->rec;
    auto cleanup = [&]() {
        p->src = src0;
        p->rec = rec0;
        p->ns = NS;
        p->nr = NR;
        p->pa.nshot = nshot;
        dev_free(p, d_pts);
        dev_free(p, dobs_s);
        dev_free(p, dsyn_s);
        dev_free(p, grad_s);
    };
    awe_status st = dev_alloc(p, (void **)&d_pts, std::max<size_t>(pts.size(), 1) * sizeof(GeoPoint));
    if (st == AWE_OK) st = dev_alloc(p, (void **)&dobs_s, (size_t)p->nsmp * max_nr * sizeof(float));
    if (st == AWE_OK && d_dsyn) st = dev_alloc(p, (void **)&dsyn_s, (size_t)p->nsmp * max_nr * sizeof(float));
    if (st == AWE_OK) st = dev_alloc(p, (void **)&grad_s, mcells * sizeof(double));
    if (st == AWE_OK && !pts.empty() &&
        cudaMemcpyAsync(d_pts, pts.data(), pts.size() * sizeof(GeoPoint), cudaMemcpyHostToDevice, s) != cudaSuccess) {
        set_error("awe_gradient: point upload failed");
        st = AWE_ERR_CUDA;
    }
    if (st == AWE_OK && cudaMemsetAsync(d_grad, 0, mcells * sizeof(double), s) != cudaSuccess) {
        set_error("awe_gradient: clearing the gradient failed");
        st = AWE_ERR_CUDA;
    }
    p->pa.nshot = 1;
    p->nr = max_nr;  // sizes the gradient's trace buffers for every shot
    if (st == AWE_OK) st = grad_alloc(p, T, fmt);
    double J = 0;
    long long launches = 0;
    int s0 = 0, r0 = 0;
    for (int q = 0; q < nshot && st == AWE_OK; q++) {
        const int ns = p->shot_ns[q], nr = p->shot_nr[q];
        p->src = d_pts + s0;
        p->ns = ns;
        p->rec = d_pts + NS + r0;
        p->nr = nr;
        if (nr > 0 && cudaMemcpy2DAsync(dobs_s, (size_t)nr * sizeof(float), d_dobs + r0, (size_t)NR * sizeof(float),
                                        (size_t)nr * sizeof(float), p->nsmp, cudaMemcpyDeviceToDevice,
                                        s) != cudaSuccess) {
            set_error("awe_gradient: data gather failed");
            st = AWE_ERR_CUDA;
            break;
        }
        double Jq = 0;
        st = gradient_spher_one(p, d_wav, ncs, dobs_s, T, fmt, grad_s, &Jq, dsyn_s, s, image);
        if (st != AWE_OK) break;
        launch_add_f64(d_grad, grad_s, (long long)mcells, s);
        if (d_dsyn && nr > 0 &&
            cudaMemcpy2DAsync(d_dsyn + r0, (size_t)NR * sizeof(float), dsyn_s, (size_t)nr * sizeof(float),
                              (size_t)nr * sizeof(float), p->nsmp, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
            set_error("awe_gradient: data scatter failed");
            st = AWE_ERR_CUDA;
            break;
        }
        J += Jq;
        launches += p->launches + 1;
        s0 += ns;
        r0 += nr;
    }
    if (st == AWE_OK) {
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("awe_gradient: %s", cudaGetErrorString(e));
            st = AWE_ERR_CUDA;
        }
    }
    cleanup();
    *misfit = J;
    p->launches = launches;
    return st;
}

awe_status plan_gradient(awe_plan *p, const float *d_wav, int ncs, const float *d_dobs, const awe_grad_opts &o,
                         double *d_grad, double *misfit, float *d_dsyn, cudaStream_t s, int image) {
    const awe_desc &d = p->d;
    const bool spher = d.scheme == AWE_SCHEME_GPU && d.coords == AWE_SPHER && d.ndim == 3;
    if ((d.scheme != AWE_SCHEME_CPU || d.coords != AWE_CART) && !spher) {
        set_error("awe_gradient: the adjoint covers the cartesian CPU-program scheme and the spherical 3D "
                  "GPU-program scheme");
        return AWE_ERR_UNSUPPORTED;
    }
    if (spher) {
        if (d.precision != AWE_FAST) {
            set_error("awe_gradient: precision must be AWE_FAST");
            return AWE_ERR_UNSUPPORTED;
        }
        int T = o.ckpt_every > 0 ? o.ckpt_every : (int)std::ceil(std::sqrt((double)d.nt));
        T = std::max(1, std::min(T, d.nt));
        if (o.ckpt_format != AWE_CKPT_BF16 && o.ckpt_format != AWE_CKPT_FP32 && o.ckpt_format != AWE_CKPT_FP16 &&
            o.ckpt_format != AWE_CKPT_BFP16) {
            set_error("awe_gradient: unknown checkpoint format %d", o.ckpt_format);
            return AWE_ERR_INVALID;
        }
        return plan_gradient_spher(p, d_wav, ncs, d_dobs, T, o.ckpt_format, d_grad, misfit, d_dsyn, s, image);
    }
    if (p->den || d.hybrid) {
        set_error("awe_gradient: variable density and the hybrid ABC have no adjoint here");
        return AWE_ERR_UNSUPPORTED;
    }
    if (d.precision != AWE_FAST) {
        set_error("awe_gradient: precision must be AWE_FAST");
        return AWE_ERR_UNSUPPORTED;
    }
    const Grid &g = p->g;
    const int W = p->nop + 2;
    if (d.ndim == 3 && d.dabc && (g.n1 <= 2 * W || g.n2 <= 2 * W || g.n3 <= 2 * W)) {
        set_error("awe_gradient: padded grid too small for the one-way ABC transpose");
        return AWE_ERR_INVALID;
    }
    int T = o.ckpt_every > 0 ? o.ckpt_every : (int)std::ceil(std::sqrt((double)d.nt));
    if (T > d.nt) T = d.nt;
    if (T < 1) T = 1;
    if (o.ckpt_format != AWE_CKPT_BF16 && o.ckpt_format != AWE_CKPT_FP32 && o.ckpt_format != AWE_CKPT_FP16 &&
        o.ckpt_format != AWE_CKPT_BFP16) {
        set_error("awe_gradient: unknown checkpoint format %d", o.ckpt_format);
        return AWE_ERR_INVALID;
    }
    AWE_TRY(grad_alloc(p, T, o.ckpt_format));
    GradState *st = p->grad;
    const long long cells = g.cells();
    const size_t bytes = (size_t)cells * sizeof(float);
    float *dat = d_dsyn ? d_dsyn : st->dat;
    if (st->h_rows_n < (size_t)p->nsmp) {
        if (st->h_rows) cudaFreeHost(st->h_rows);
        st->h_rows = nullptr;
        st->h_rows_n = 0;
        CUDA_TRY(cudaMallocHost((void **)&st->h_rows, (size_t)p->nsmp * sizeof(double)));
        st->h_rows_n = (size_t)p->nsmp;
    }
    const bool xcorr = image == AWE_IMAGE_XCORR;
    const StepBParams sp = stepB_params(p);
    const bool sponge = d.dabc && !d.hybrid;
    AdjParams ap{};
    ap.g = g;
    ap.k = p->k;
    ap.nd = d.ndim;
    ap.nop = p->nop;
    ap.w1 = sponge ? p->w[0] : nullptr;
    ap.w2 = sponge ? p->w[1] : nullptr;
    ap.w3 = sponge ? p->w[2] : nullptr;
    ap.xcorr = xcorr;
    AbcB abc{p->abc[0], p->abc[1], p->abc[2], p->abc[3], p->abc[4], p->abc[5]};
    // receivers and sources in the adjoint step itself (one launch per step)
    // where the grid is small enough for per-cell lists and no ABC transpose
    // follows the step
    const bool fuse_pts = !st->tma && !st->kap && cells <= (1LL << 24);
    // 3D TMA path: one boundary launch per adjoint step (k_bnd3_adj) instead of
    // the kappa fold, three ABC-transpose launches and the g pass; AWE_BND3=0
    // keeps the separate launches (the tests compare both)
    const bool bnd_adj = st->tma && st->kap && stepB3_bnd(p);
    if (fuse_pts) {
        if (!st->lists_ok) {
            const int nc = d.ndim == 3 ? 8 : 4;
            AWE_TRY(build_cell_lists(p, p->h_rec, nc, &st->rc_start, &st->rc_ent, &st->rc_cap, s));
            AWE_TRY(build_cell_lists(p, p->h_src, nc, &st->sc_start, &st->sc_ent, &st->sc_cap, s));
            st->lists_ok = true;
        }
        ap.rc_start = st->rc_start;
        ap.rc_ent = st->rc_ent;
        ap.sc_start = st->sc_start;
        ap.sc_ent = st->sc_ent;
        ap.ncs = ncs;
        ap.one_wavelet = ncs == 1;
    }

    // the whole gradient as stream work on `s`
    auto seq = [&](cudaStream_t s, long long &launches) -> awe_status {

    // 1. forward with checkpoints of both levels at the start of every segment
    StepHook hook = [&](int it, const float *prev, const float *cur, cudaStream_t ss) -> awe_status {
        if (it % T != 0) return AWE_OK;
        const int seg = it / T;
        AWE_TRY(ckpt_store(p, 2 * seg, prev, ss));
        AWE_TRY(ckpt_store(p, 2 * seg + 1, cur, ss));
        return AWE_OK;
    };
    AWE_TRY(planB_run_hooked(p, d_wav, ncs, dat, nullptr, s, &hook));
    launches += p->launches;

    // 2. residual and misfit (FP64 per row, summed in row order on the host);
    // an image back-propagates the recorded data themselves
    if (image < 0) {
        launch_residual(dat, d_dobs, st->r, p->nsmp, p->nr, st->row_sum, s);
        CUDA_TRY(cudaMemcpyAsync(st->h_rows, st->row_sum, (size_t)p->nsmp * sizeof(double), cudaMemcpyDeviceToHost,
                                 s));
    } else {
        CUDA_TRY(cudaMemcpyAsync(st->r, d_dobs, (size_t)p->nsmp * p->nr * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }

    // 3. adjoint sweep
    CUDA_TRY(cudaMemsetAsync(st->X, 0, bytes, s));
    CUDA_TRY(cudaMemsetAsync(st->Y, 0, bytes, s));
    CUDA_TRY(cudaMemsetAsync(st->G, 0, (size_t)cells * sizeof(float2), s));
    if (st->kap) CUDA_TRY(cudaMemsetAsync(st->kap, 0, bytes, s));
    float *X = st->X, *Y = st->Y;
    const CUtensorMap *xmap = &st->x_tile, *ymap = &st->y_tile;
    for (int seg = st->nseg - 1; seg >= 0; seg--) {
        const int k0 = seg * T, k1 = std::min(k0 + T, d.nt);
        float *slot0 = st->slots;
        if (st->tma) {
            // recompute with three rolling levels; the step kernel stores L(V_k) in slot k - k0
            AWE_TRY(ckpt_load(p, 2 * seg, st->vr, s));
            AWE_TRY(ckpt_load(p, 2 * seg + 1, st->vr + cells, s));
            for (int k = k0; k < k1; k++) {
                const int j = k - k0;
                float *A = st->vr + (size_t)(j % 3) * cells, *B = st->vr + (size_t)((j + 1) % 3) * cells;
                float *N = st->vr + (size_t)((j + 2) % 3) * cells;
                // the slot gets L(V_k) for the gradient, V_k itself for the cross-correlation image
                AWE_TRY(stepB_full(p, sp, A, B, N, k, d_wav, ncs, &st->vr_halo[(j + 1) % 3], &st->vr_tile[j % 3], s,
                                   launches, xcorr ? nullptr : slot0 + (size_t)j * cells));
                if (xcorr) CUDA_TRY(cudaMemcpyAsync(slot0 + (size_t)j * cells, B, bytes, cudaMemcpyDeviceToDevice, s));
            }
        } else {
            AWE_TRY(ckpt_load(p, 2 * seg, slot0, s));
            AWE_TRY(ckpt_load(p, 2 * seg + 1, slot0 + cells, s));
            for (int k = k0; k <= k1 - 2; k++) {
                const int j = k - k0;
                float *A = slot0 + (size_t)j * cells, *B = A + cells, *N = B + cells;
                AWE_TRY(stepB_full(p, sp, A, B, N, k, d_wav, ncs, nullptr, nullptr, s, launches));
            }
        }
        for (int k = k1 - 1; k >= k0; k--) {
            if (bnd_adj) {
                // kappa of the previous adjoint step folded into this step's nu, the
                // transposed ABC and g = I vel2 nu in one launch
                Bnd3AdjParams bp{};
                bp.g = g;
                bp.mu = X;
                bp.kap = st->kap;
                bp.gout = st->gbuf;
                bp.vel2 = p->vel;
                bp.zl = abc.zl, bp.zh = abc.zh, bp.xl = abc.xl, bp.xh = abc.xh, bp.yl = abc.yl, bp.yh = abc.yh;
                bp.w1 = ap.w1, bp.w2 = ap.w2, bp.w3 = ap.w3;
                bp.top = !d.fsrf;
                launch_bnd3_adj(bp, s);
                launches++;
            } else if (d.ndim == 3 && d.dabc) {
                launch_abc_adjB(p->nop, d.fsrf, X, st->kap, abc, g, s);
                launches += 3;
            }
            if (st->tma) {
                if (!bnd_adj) launch_adj_g(X, p->vel, st->gbuf, g, p->nop, s);
                prof_begin(p, s, AWE_PROF_ADJOINT);
                cudaError_t e = launch_stepB3_adj(st->g_halo, *ymap, *xmap, Y, slot0 + (size_t)(k - k0) * cells,
                                                  st->G, sp, p->tma_shape, p->sched_counter, p->sched_base, p->d_err,
                                                  s);
                prof_end(p, s);
                p->sched_base += (unsigned long long)p->tma_shape.items + p->tma_shape.grid;
                if (e != cudaSuccess) {
                    set_error("TMA adjoint launch failed: %s", cudaGetErrorString(e));
                    return AWE_ERR_CUDA;
                }
                launches += bnd_adj ? 1 : 2;
            } else {
                const float *Vk = slot0 + (size_t)(k - k0 + 1) * cells;
                if (fuse_pts) {
                    ap.rrow = (k % d.jdata == 0 && p->nr > 0) ? st->r + (size_t)(k / d.jdata) * p->nr : nullptr;
                    ap.wav = (p->ns > 0 && !xcorr) ? d_wav : nullptr;
                    ap.it = k;
                }
                prof_begin(p, s, AWE_PROF_ADJOINT);
                launch_adjB(X, Y, Vk, p->vel, st->G, ap, s);
                prof_end(p, s);
                launches++;
            }
            if (d.ndim == 3 && d.dabc && !bnd_adj) {  // (bnd_adj: folded by the next step's launch)
                launch_kap_fold(Y, st->kap, ap, s);
                launches++;
            }
            if (k % d.jdata == 0 && p->nr > 0 && !fuse_pts) {
                launch_rec_adj(Y, p->rec, p->nr, st->r + (size_t)(k / d.jdata) * p->nr, ap, p->corner_off, s);
                launches++;
            }
            if (p->ns > 0 && !xcorr && !fuse_pts) {
                launch_src_grad(st->G, X, p->src, p->ns, d_wav, k, ncs, ncs == 1, d.ndim, p->corner_off, s);
                launches++;
            }
            std::swap(X, Y);
            std::swap(xmap, ymap);
        }
    }
    if (xcorr) launch_image_cut(st->G, g, p->nbd, d.n, d.ndim, d_grad, s);
    else launch_grad_fold(st->G, p->vel, d.dt, g, p->nbd, d.n, d.ndim, d_grad, s);
    launches++;
    return AWE_OK;
    };  // seq

    // Without the TMA path (whose work-counter bases are host state) and
    // without snapshot delivery or profiling, the sequence is captured once as
    // a CUDA graph and replayed while its buffers and settings stay the same
    // (what matters for launch-bound 2D grids).
    const bool graph = !st->tma && !p->snap_cb && !p->profile;
    long long launches = 0;
    const void *key[4] = {d_wav, d_dobs, d_grad, dat};
    bool same = st->g_ncs == ncs && st->g_image == image;
    for (int q = 0; q < 4; q++) same = same && st->g_key[q] == key[q];
    if (graph && !(same && (st->gexec || st->g_seen))) {  // new settings: run directly and remember them
        if (st->gexec) cudaGraphExecDestroy(st->gexec);
        st->gexec = nullptr;
        for (int q = 0; q < 4; q++) st->g_key[q] = key[q];
        st->g_ncs = ncs;
        st->g_image = image;
        st->g_seen = true;
        AWE_TRY(seq(s, launches));
    } else if (graph && (st->gexec || st->g_seen)) {  // repeated settings: capture once, then replay
        if (!st->gexec) {
            cudaStream_t cs;
            CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
            cudaGraph_t gr = nullptr;
            awe_status rs = AWE_OK;
            cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                rs = seq(cs, launches);
                e = cudaStreamEndCapture(cs, &gr);
            }
            if (rs == AWE_OK && e == cudaSuccess) e = cudaGraphInstantiate(&st->gexec, gr, 0);
            if (gr) cudaGraphDestroy(gr);
            cudaStreamDestroy(cs);
            if (rs != AWE_OK) return rs;
            if (e != cudaSuccess) {
                st->gexec = nullptr;
                set_error("CUDA graph capture of the gradient failed: %s", cudaGetErrorString(e));
                return AWE_ERR_CUDA;
            }
            st->g_launches = launches;
        }
        CUDA_TRY(cudaGraphLaunch(st->gexec, s));
        launches = st->g_launches;
    } else {
        AWE_TRY(seq(s, launches));
    }
    CUDA_TRY(cudaStreamSynchronize(s));
    double J = 0;
    for (int q = 0; image < 0 && q < p->nsmp; q++) J += 0.5 * st->h_rows[q];
    *misfit = J;
    p->launches = launches;
    return AWE_OK;
}

}  // namespace awe
