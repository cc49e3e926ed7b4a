// Host side of the CPU-program scheme (MAWEFDcart{2D,3D}cpu.c): padding,
// coefficient tables, model preparation and the per-step launch sequence.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
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
#define AWE_TRY(expr)                      \
    do {                                   \
        awe_status s_ = (expr);            \
        if (s_ != AWE_OK) return s_;       \
    } while (0)

// cut2d / cut3d_slice first index (fdutil.c:574-717): floor((o - opad)/d) in float
static int window_first(float o, float opad, float d) { return (int)(std::floor)((o - opad) / d); }

static awe_status upload(awe_plan *p, float **dst, const float *src, size_t n) {
    if (!*dst) AWE_TRY(dev_alloc(p, (void **)dst, n * sizeof(float)));
    CUDA_TRY(cudaMemcpy(*dst, src, n * sizeof(float), cudaMemcpyHostToDevice));
    return AWE_OK;
}

awe_status planB_init(awe_plan *p) {
    awe_desc &d = p->d;
    if (d.fdorder == 0) d.fdorder = 4;  // MAWEFDcart2Dcpu.c:126
    p->ndim = d.ndim;
    p->nop = d.fdorder / 2;
    int nb = d.nb;
    if (nb < p->nop) nb = p->nop;                              // :211
    if (d.dabc && d.hybrid && nb <= p->nop) nb = 2 * p->nop;  // :212
    p->nbd = nb;
    const int n3 = d.ndim == 3 ? d.n[2] : 1;
    p->g = Grid{d.n[0] + 2 * nb, d.n[1] + 2 * nb, d.ndim == 3 ? n3 + 2 * nb : 1};
    for (int a = 0; a < d.ndim; a++) p->opad[a] = d.o[a] - nb * d.d[a];  // fdutil_init
    float dd[3] = {d.d[0], d.d[1], d.ndim == 3 ? d.d[2] : 1.f};
    fd_coefficients(p->nop, d.ndim, dd, d.optfd, p->k);

    const size_t cells = (size_t)p->g.cells();
    AWE_TRY(dev_alloc(p, (void **)&p->u[0], cells * sizeof(float)));
    AWE_TRY(dev_alloc(p, (void **)&p->u[1], cells * sizeof(float)));
    AWE_TRY(dev_alloc(p, (void **)&p->vel, cells * sizeof(float)));
    AWE_TRY(dev_alloc(p, (void **)&p->corner_off, 8 * sizeof(long long)));

    if (d.dabc && !d.hybrid) {
        std::vector<float> w;
        sponge_weights(nb, w);
        const int len[3] = {p->g.n1, p->g.n2, p->g.n3};
        for (int a = 0; a < 3; a++) {
            std::vector<float> t(len[a], 1.f);
            if (a < d.ndim)
                for (int i = 0; i < nb && i < len[a]; i++) {
                    t[i] = w[nb - i - 1];
                    t[len[a] - 1 - i] = w[nb - i - 1];
                }
            undamped_range(t, p->wlo[a], p->whi[a]);
            AWE_TRY(upload(p, &p->w[a], t.data(), t.size()));
        }
    }
    if (d.dabc && d.hybrid && nb - p->nop > 0) {
        std::vector<float> dm;
        hybrid_damp(nb - p->nop, dm);
        AWE_TRY(upload(p, &p->damp, dm.data(), dm.size()));
    }

    // TMA-staged step kernel for the 3D 8th-order case; AWE_STEP_KERNEL=simple
    // forces the one-thread-per-cell kernel (used by the tests to compare both)
    const char *kern = std::getenv("AWE_STEP_KERNEL");
    const bool force_simple = kern && std::strcmp(kern, "simple") == 0;
    if (!force_simple && stepB3_tma_eligible(d.ndim, p->nop, false, p->g)) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
        const char *lenv = std::getenv("AWE_TMA_CHUNK");
        p->tma_shape = stepB3_tma_shape(p->g, sms > 0 ? sms : 1, lenv ? std::atoi(lenv) : 0);
        AWE_TRY(dev_alloc(p, (void **)&p->sched_counter, sizeof(unsigned long long)));
        AWE_TRY(dev_alloc(p, (void **)&p->d_err, sizeof(int)));
        CUDA_TRY(cudaMemset(p->sched_counter, 0, sizeof(unsigned long long)));
        CUDA_TRY(cudaMemset(p->d_err, 0, sizeof(int)));
        p->sched_base = 0;
        if (stepB3_tma_maps(p->tmaps, p->u, p->vel, p->g)) p->use_tma = true;
        const char *spin = std::getenv("AWE_PIPELINE_SPIN_LIMIT");
        if (spin && *spin) p->spin_limit = std::atoll(spin);
    }
    // line-end copies of the 3D boundary launch (made before any capture of
    // the time loop; AWE_BND_ENDS=0: the launch reads the level itself)
    const char *eenv = std::getenv("AWE_BND_ENDS");
    if (d.ndim == 3 && d.dabc && !d.hybrid && bnd3_eligible(p->nop, p->g) && !(eenv && std::strcmp(eenv, "0") == 0))
        for (int k = 0; k < 2; k++)
            AWE_TRY(dev_alloc(p, (void **)&p->ends[k], (size_t)p->g.n2 * p->g.n3 * 16 * sizeof(float)));

    p->nsmp = (d.nt - 1) / d.jdata + 1;
    p->nsnap = d.jsnap > 0 ? (d.nt - 1) / d.jsnap + 1 : 0;
    for (int a = 0; a < 3; a++) {
        const int npad = a == 0 ? p->g.n1 : a == 1 ? p->g.n2 : p->g.n3;
        if (a >= d.ndim) {
            p->snap_f[a] = 0;
            p->snap_m[a] = 1;
        } else if (d.bnds) {
            p->snap_f[a] = 0;
            p->snap_m[a] = npad;
        } else {
            p->snap_f[a] = window_first(d.o[a], p->opad[a], d.d[a]);
            p->snap_m[a] = d.n[a];
        }
    }
    p->snap_elems = (size_t)p->snap_m[0] * p->snap_m[1] * p->snap_m[2];
    return AWE_OK;
}

awe_status planB_model(awe_plan *p, const float *vel, const float *den) {
    // The model goes to the device as passed, into a level buffer (the levels
    // are cleared at the start of every run), and the padded tables are made
    // there (k_model.cu): the same float operations as the host restatement
    // of fdutil.c's expand / abcone*_make, without a host pass over the
    // padded grid.
    const awe_desc &d = p->d;
    const Grid &g = p->g;
    const size_t cells = (size_t)g.cells();
    const size_t raw = (size_t)d.n[0] * d.n[1] * (d.ndim == 3 ? d.n[2] : 1);
    cudaStream_t s = p->stream;
    ModelPrep m{};
    m.g = g;
    m.n1 = d.n[0];
    m.n2 = d.n[1];
    m.n3 = d.ndim == 3 ? d.n[2] : 1;
    m.nb = p->nbd;
    m.nd = d.ndim;
    m.dt = d.dt;
    m.dt2 = d.dt * d.dt;
    m.d1 = d.d[0];
    m.d2 = d.d[1];
    m.d3 = d.ndim == 3 ? d.d[2] : 1.f;
    m.zero1 = (d.fsrf && !d.hybrid) ? std::min(p->nbd + 1, g.n1) : 0;
    float *stage = p->u[1];
    // no earlier work of this plan (on any stream) may still read the level
    // buffers or the model tables
    CUDA_TRY(cudaDeviceSynchronize());
    CUDA_TRY(cudaMemcpyAsync(stage, vel, raw * sizeof(float), cudaMemcpyHostToDevice, s));
    if (d.dabc) {
        const size_t sz[6] = {(size_t)g.n2 * g.n3, (size_t)g.n2 * g.n3, (size_t)g.n1 * g.n3, (size_t)g.n1 * g.n3,
                              (size_t)g.n1 * g.n2, (size_t)g.n1 * g.n2};
        for (int k = 0; k < (d.ndim == 3 ? 6 : 4); k++)
            if (!p->abc[k]) AWE_TRY(dev_alloc(p, (void **)&p->abc[k], sz[k] * sizeof(float)));
        float *const tabs[6] = {p->abc[0], p->abc[1], p->abc[2], p->abc[3], p->abc[4], p->abc[5]};
        launch_model_abc(stage, m, tabs, s);
    }
    if (!p->vel) AWE_TRY(dev_alloc(p, (void **)&p->vel, cells * sizeof(float)));
    launch_model_pad(stage, p->vel, m, true, s);
    if (den) {
        CUDA_TRY(cudaMemcpyAsync(stage, den, raw * sizeof(float), cudaMemcpyHostToDevice, s));
        if (!p->den) AWE_TRY(dev_alloc(p, (void **)&p->den, cells * sizeof(float)));
        launch_model_pad(stage, p->den, m, false, s);
    }
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(s));
    return AWE_OK;
}

awe_status set_geometry_common(awe_plan *p, int ns, const float *sou, int nr, const float *rec) {
    const awe_desc &d = p->d;
    const Grid &g = p->g;
    const int nd = d.ndim;
    const long long s2 = g.n1, s3 = (long long)g.n1 * g.n2;
    const bool spher = d.coords == AWE_SPHER;
    // reference fdm axes: cartesian z=axis1, x=axis2, y=axis3; spherical
    // programs map z=theta (axis 2), x=r (axis 1), y=phi (axis 3)
    // (MAWEFDspher3Dgpu.cu:167-173, MAWEFDspher2Dgpu.cu:151)
    FdmAxes f{};
    long long sz, sx, sy;
    if (!spher) {
        f = FdmAxes{p->opad[0], p->opad[1], p->opad[2], d.d[0], d.d[1], nd == 3 ? d.d[2] : 1.f, g.n1, g.n2, g.n3};
        sz = 1;
        sx = s2;
        sy = s3;
    } else {
        f = FdmAxes{p->opad[1], p->opad[0], p->opad[2], d.d[1], d.d[0], nd == 3 ? d.d[2] : 1.f, g.n2, g.n1, g.n3};
        sz = s2;
        sx = 1;
        sy = s3;
    }
    // corner order of lint*_make weights: (z, x[, y]) bits 001=z, 010=x, 100=y
    long long off[8];
    for (int c = 0; c < 8; c++) off[c] = ((c & 1) ? sz : 0) + ((c & 2) ? sx : 0) + ((c & 4) ? sy : 0);
    std::memcpy(p->h_corner_off, off, sizeof off);
    CUDA_TRY(cudaMemcpy(p->corner_off, off, sizeof off, cudaMemcpyHostToDevice));

    auto make = [&](const float *xyz, int n, std::vector<GeoPoint> &out, std::vector<Lint> *keep) {
        out.resize(n);
        if (keep) keep->resize(n);
        for (int i = 0; i < n; i++) {
            float x, y = 0.f, z;
            if (nd == 2) {
                x = xyz[2 * i];
                z = xyz[2 * i + 1];
            } else {
                x = xyz[3 * i];
                y = xyz[3 * i + 1];
                z = xyz[3 * i + 2];
            }
            Lint l = lint_make(nd, x, y, z, f);
            GeoPoint gp;
            gp.base = l.jz * sz + l.jx * sx + (nd == 3 ? l.jy * sy : 0);
            std::memcpy(gp.w, l.w, sizeof gp.w);
            out[i] = gp;
            if (keep) (*keep)[i] = l;
        }
    };
    make(sou, ns, p->h_src, &p->h_src_lint);
    make(rec, nr, p->h_rec, nullptr);
    // the point buffers are kept while large enough (a captured time loop
    // that read them stays valid)
    const int need_s = ns > 0 ? ns : 1, need_r = nr > 0 ? nr : 1;
    if (!p->src || p->src_cap < need_s) {
        if (p->src) dev_free(p, p->src);
        p->src = nullptr;
        p->src_cap = 0;
        AWE_TRY(dev_alloc(p, (void **)&p->src, need_s * sizeof(GeoPoint)));
        p->src_cap = need_s;
    }
    if (!p->rec || p->rec_cap < need_r) {
        if (p->rec) dev_free(p, p->rec);
        p->rec = nullptr;
        p->rec_cap = 0;
        AWE_TRY(dev_alloc(p, (void **)&p->rec, need_r * sizeof(GeoPoint)));
        p->rec_cap = need_r;
    }
    CUDA_TRY(cudaDeviceSynchronize());  // earlier runs may still read the old points
    if (ns) CUDA_TRY(cudaMemcpy(p->src, p->h_src.data(), ns * sizeof(GeoPoint), cudaMemcpyHostToDevice));
    if (nr) CUDA_TRY(cudaMemcpy(p->rec, p->h_rec.data(), nr * sizeof(GeoPoint), cudaMemcpyHostToDevice));
    p->ns = ns;
    p->nr = nr;

    // scheme CPU: a source node inside the sponge band but outside the
    // boundary shell would be sponged before its injection by the fused
    // step; such runs defer the whole sponge to after the injection
    p->sponge_deferred = false;
    p->src_in_shell = false;
    if (d.scheme == AWE_SCHEME_CPU && d.dabc && !d.hybrid) {
        const int shell = (nd == 3) ? p->nop + 2 : 0;
        const int nc = nd == 3 ? 8 : 4;
        for (const GeoPoint &gp : p->h_src)
            for (int c = 0; c < nc; c++) {
                if (gp.w[c] == 0.f) continue;
                const long long n = gp.base + off[c];
                const int i3 = (int)(n / s3), i2 = (int)((n % s3) / s2), i1 = (int)(n % s2);
                const int ii[3] = {i1, i2, i3}, nn[3] = {g.n1, g.n2, g.n3};
                bool band = false, inshell = false;
                for (int a = 0; a < nd; a++) {
                    const int dist = std::min(ii[a], nn[a] - 1 - ii[a]);
                    band = band || dist < p->nbd;
                    inshell = inshell || dist < shell;
                }
                if (band && !inshell) p->sponge_deferred = true;
                if (inshell) p->src_in_shell = true;
            }
    }
    return AWE_OK;
}

bool stepB3_bnd(const awe_plan *p) {
    const awe_desc &d = p->d;
    const char *env = std::getenv("AWE_BND3");
    return d.scheme == AWE_SCHEME_CPU && d.ndim == 3 && d.dabc && !d.hybrid && !p->sponge_deferred &&
           bnd3_eligible(p->nop, p->g) && !(env && std::strcmp(env, "0") == 0);
}

StepBParams stepB_params(const awe_plan *p) {
    const awe_desc &d = p->d;
    const Grid &g = p->g;
    const bool sponge = d.dabc && !d.hybrid;
    StepBParams sp{};
    sp.g = g;
    sp.k = p->k;
    sp.w1 = p->w[0];
    sp.w2 = p->w[1];
    sp.w3 = p->w[2];
    sp.damp_prev = sponge;
    sp.sponge_new = sponge && !p->sponge_deferred;
    sp.shell = (d.ndim == 3 && sponge) ? p->nop + 2 : 0;
    for (int a = 0; a < 3; a++) {
        sp.ilo[a] = sponge ? p->wlo[a] : 0;
        sp.ihi[a] = sponge ? p->whi[a] : (a == 0 ? g.n1 : a == 1 ? g.n2 : g.n3);
    }
    sp.prv = nullptr;
    sp.spin = p->spin_limit;
    return sp;
}

// One full time step it: the new level is written to `nxt`, which is the
// buffer holding the previous level (in place, prv_map == null or the TMA
// maps of that buffer) or a third buffer (out of place: `prv` names the
// previous level, and for the TMA kernel `cur_map`/`prv_map` are given).
awe_status stepB_full(awe_plan *p, const StepBParams &sp0, const float *prv, const float *cur, float *nxt, int it,
                      const float *d_wav, int ncs, const CUtensorMap *cur_map, const CUtensorMap *prv_map,
                      cudaStream_t s, long long &launches, float *lap_out, const GeoPoint *ext_pts, int ext_n,
                      int ext_stride, float *ext_row) {
    const awe_desc &d = p->d;
    const Grid &g = p->g;
    const bool exact = d.precision == AWE_EXACT;
    const bool sponge = d.dabc && !d.hybrid;
    const int shell = sp0.shell;
    StepBParams sp = sp0;
    sp.prv = (prv != nxt) ? prv : nullptr;
    // 2D: sources (few) and receivers ride in the step kernel's launch
    const bool fuse_src = d.ndim == 2 && p->ns > 0 && p->ns <= kFusedSources;
    if (fuse_src) {
        const PointsAt ps = points_at(p, p->src, p->ns, p->src_rows, it);
        sp.inj = ps.pts;
        sp.inj_n = p->ns;
        sp.inj_stride = ps.stride;
        sp.inj_wav = d_wav;
        sp.inj_it = it;
        sp.inj_ncs = ncs;
        sp.inj_one = ncs == 1;
    }
    if (d.ndim == 2 && ext_n > 0) {
        sp.ext = ext_pts;
        sp.ext_n = ext_n;
        sp.ext_stride = ext_stride;
        sp.ext_row = ext_row;
    }
    prof_begin(p, s);
    if (p->use_tma && cur_map && prv_map) {
        cudaError_t e = launch_stepB3_tma_with(exact, *cur_map, *prv_map, p->tmaps[4], nxt, sp, p->tma_shape,
                                               p->sched_counter, p->sched_base, p->d_err, s, lap_out);
        p->sched_base += (unsigned long long)p->tma_shape.items + p->tma_shape.grid;
        if (e != cudaSuccess) {
            set_error("TMA step launch failed: %s", cudaGetErrorString(e));
            return AWE_ERR_CUDA;
        }
    } else {
        launch_stepB(d.ndim, p->nop, exact, p->den != nullptr, cur, nxt, p->vel, p->den, sp, s);
    }
    prof_end(p, s);
    launches++;
    const bool bnd = stepB3_bnd(p);
    // the boundary launch injects too, unless a source touches the cells the ABC reads
    const bool inj_in_bnd = bnd && !p->src_in_shell;
    if (p->ns > 0 && !fuse_src && !inj_in_bnd) {
        const PointsAt ps = points_at(p, p->src, p->ns, p->src_rows, it);
        launch_injectB_off(d.ndim, exact, nxt, p->vel, ps.pts, p->ns, d_wav, it, ncs, ncs == 1, p->corner_off, s,
                           ps.stride);
        launches++;
    }
    if (bnd) {
        Bnd3Params bp{};
        bp.g = g;
        bp.uo = nxt;
        bp.um = cur;
        bp.vel = p->vel;
        bp.zl = p->abc[0];
        bp.zh = p->abc[1];
        bp.xl = p->abc[2];
        bp.xh = p->abc[3];
        bp.yl = p->abc[4];
        bp.yh = p->abc[5];
        bp.w1 = p->w[0];
        bp.w2 = p->w[1];
        bp.w3 = p->w[2];
        bp.top = !d.fsrf;
        if (p->ends_run) {
            bp.em = p->ends[p->ends_idx];
            bp.eo = p->ends[1 - p->ends_idx];
            p->ends_idx ^= 1;
        }
        bp.rec = ext_pts;
        bp.nr = ext_n;
        bp.rec_stride = ext_stride;
        bp.rec_row = ext_n > 0 ? ext_row : nullptr;
        if (inj_in_bnd && p->ns > 0) {
            const PointsAt ps = points_at(p, p->src, p->ns, p->src_rows, it);
            bp.src = ps.pts;
            bp.ns = p->ns;
            bp.src_stride = ps.stride;
            bp.wav = d_wav;
            bp.it = it;
            bp.ncs = ncs;
            bp.one_wavelet = ncs == 1;
        }
        launch_bnd3(exact, bp, s);
        launches++;
        return AWE_OK;
    }
    if (d.dabc) {
        AbcB abc{p->abc[0], p->abc[1], p->abc[2], p->abc[3], p->abc[4], p->abc[5]};
        if (d.hybrid) {
            launch_hybridB(d.ndim, p->nop, p->nbd, exact, d.fsrf, nxt, cur, abc, p->damp, g, s);
            launches += d.ndim;
        } else {
            // the axis-1 ABC pass also applies the shell sponge to the axis-1 ends of
            // lines the later passes leave alone (not when the sponge is deferred)
            const bool zf = sponge && !p->sponge_deferred && shell > 0 && d.ndim == 3 && abc_zfused(p->nop, g, shell);
            if (d.ndim == 3) {
                if (zf) launch_abconeB(3, p->nop, exact, d.fsrf, nxt, cur, abc, g, s, p->w[0], p->w[1], p->w[2], shell);
                else launch_abconeB(3, p->nop, exact, d.fsrf, nxt, cur, abc, g, s);
                launches += 3;
            }
            if (sponge && p->sponge_deferred) {
                launch_band_sponge(d.ndim, std::max(p->nbd, shell), exact, nxt, p->w[0], p->w[1], p->w[2], g, s);
                launches += d.ndim;  // one kernel per slab orientation
            } else if (shell > 0) {
                launch_band_sponge(d.ndim, shell, exact, nxt, p->w[0], p->w[1], p->w[2], g, s, zf ? 1 : 0);
                launches += d.ndim;
            }
        }
    }
    return AWE_OK;
}

awe_status planB_run(awe_plan *p, const float *d_wav, int ncs, float *d_dat, float *d_wfl, cudaStream_t s) {
    return planB_run_hooked(p, d_wav, ncs, d_dat, d_wfl, s, nullptr);
}

awe_status planB_run_hooked(awe_plan *p, const float *d_wav, int ncs, float *d_dat, float *d_wfl, cudaStream_t s,
                            const StepHook *hook) {
    const awe_desc &d = p->d;
    const Grid &g = p->g;
    const bool exact = d.precision == AWE_EXACT;
    const bool sponge = d.dabc && !d.hybrid;
    const size_t bytes = (size_t)g.cells() * sizeof(float);
    long long launches = 0;

    CUDA_TRY(cudaMemsetAsync(p->u[0], 0, bytes, s));
    CUDA_TRY(cudaMemsetAsync(p->u[1], 0, bytes, s));
    if (p->use_tma) {  // the TMA kernel's work counter restarts with every run (graph replays included)
        CUDA_TRY(cudaMemsetAsync(p->sched_counter, 0, sizeof(unsigned long long), s));
        p->sched_base = 0;
    }
    // the boundary launches pass the line ends from step to step; the first
    // step reads those of the zero level
    struct EndsOff {
        awe_plan *p;
        ~EndsOff() { p->ends_run = false; }
    } ends_off{p};
    p->ends_run = false;
    if (p->ends[0] && stepB3_bnd(p)) {
        CUDA_TRY(cudaMemsetAsync(p->ends[0], 0, (size_t)g.n2 * g.n3 * 16 * sizeof(float), s));
        p->ends_idx = 0;
        p->ends_run = true;
    }
    if (p->nsnap > 0 && !d_wfl && p->snap_cb && !p->d_snap_tmp)
        AWE_TRY(dev_alloc(p, (void **)&p->d_snap_tmp, p->snap_elems * sizeof(float)));
    p->snap_pending = -1;  // a frame left queued by a failed run is not delivered

    const StepBParams sp = stepB_params(p);
    const float *pw1 = sponge ? p->w[0] : nullptr;

    float *cur = p->u[1], *nxt = p->u[0];
    int icur = 1;
    int row = 0, isnap = 0;
    // 2D: the traces of step it (the level the step reads, pending sponge
    // applied, as the reference extracts after its swap) are gathered by the
    // step's own launch; 3D: by the step's boundary launch
    const bool fuse_rec = (d.ndim == 2 || stepB3_bnd(p)) && p->nr > 0;
    for (int it = 0; it < d.nt; it++) {
        if (hook) AWE_TRY((*hook)(it, nxt, cur, s));
        const bool ext = fuse_rec && it % d.jdata == 0;
        const PointsAt pe = points_at(p, p->rec, p->nr, p->rec_rows, it);
        AWE_TRY(stepB_full(p, sp, nxt, cur, nxt, it, d_wav, ncs, &p->tmaps[icur], &p->tmaps[2 + (1 - icur)], s,
                           launches, nullptr, pe.pts, ext ? p->nr : 0, pe.stride,
                           ext ? d_dat + (size_t)row * p->nr : nullptr));
        std::swap(cur, nxt);  // nxt now holds the time level `it` (sponge pending)
        icur ^= 1;
        if (p->nsnap > 0 && it % d.jsnap == 0) {
            float *frame = d_wfl ? d_wfl + (size_t)isnap * p->snap_elems : p->d_snap_tmp;
            if (frame) {
                launch_snapshot(d.ndim, nxt, frame, g, p->snap_f[0], p->snap_f[1], p->snap_f[2], p->snap_m[0],
                                p->snap_m[1], p->snap_m[2], pw1, p->w[1], p->w[2], s);
                launches++;
                AWE_TRY(deliver_snapshot(p, frame, isnap, it, s));
            }
            isnap++;
        }
        if (it % d.jdata == 0) {
            if (!fuse_rec) {
                const PointsAt pr = points_at(p, p->rec, p->nr, p->rec_rows, it);
                launch_extract_off(d.ndim, exact, nxt, pr.pts, p->nr, d_dat + (size_t)row * p->nr, pw1, p->w[1],
                                   p->w[2], g, p->corner_off, s, pr.stride);
                launches += p->nr > 0;
            }
            row++;
        }
    }
    p->launches = launches;
    return flush_snapshots(p);
}

}  // namespace awe
