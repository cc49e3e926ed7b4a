// Host side of the GPU-program scheme (MAWEFD{cart,spher}{2D,3D}gpu.cu):
// padding, sponge and metric tables, one-way coefficients, injection scales
// and the per-step launch sequence.  Host arithmetic follows the reference's
// float expressions (built with -ffp-contract=off); float arguments to the
// math functions use the float overloads, as the reference's CUDA C++ does.
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
#define AWE_TRY(expr)                \
    do {                             \
        awe_status s_ = (expr);      \
        if (s_ != AWE_OK) return s_; \
    } while (0)

constexpr int kNopA = 4;  // cart_kernels.cu:401, spher_kernels.cu:402

template <class T>
static awe_status upload_t(awe_plan *p, T **dst, const T *src, size_t n) {
    if (!*dst) AWE_TRY(dev_alloc(p, (void **)dst, n * sizeof(T)));
    CUDA_TRY(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return AWE_OK;
}

static int floor_first(float o, float opad, float d, float eps) { return (int)(std::floor)((o - opad) / d + eps); }

awe_status planA_init(awe_plan *p) {
    awe_desc &d = p->d;
    p->ndim = d.ndim;
    p->nop = 1;
    const bool spher = d.coords == AWE_SPHER;
    const int geom = spher ? (d.ndim == 2 ? 2 : 3) : (d.ndim == 2 ? 0 : 1);
    const int nb = d.nb < kNopA ? kNopA : d.nb;  // MAWEFDcart2Dgpu.cu:144
    p->nbd = nb;
    p->g = Grid{d.n[0] + 2 * nb, d.n[1] + 2 * nb, d.ndim == 3 ? d.n[2] + 2 * nb : 1};
    const Grid &g = p->g;
    if (g.n1 < 12 || g.n2 < 12 || (d.ndim == 3 && g.n3 < 12)) {
        set_error("the GPU-program scheme needs at least 12 padded samples per axis");
        return AWE_ERR_UNSUPPORTED;
    }
    if (geom == 1 && d.n[0] != d.n[1]) {
        // sfAWEFDcart3Dgpu indexes the velocity and its one-way tables as if
        // nx == nz (cart_kernels.cu:456, MAWEFDcart3Dgpu.cu:271-294)
        set_error("the cartesian 3D GPU program is defined only for nx == nz (got nz=%d nx=%d)", d.n[0], d.n[1]);
        return AWE_ERR_UNSUPPORTED;
    }
    for (int a = 0; a < d.ndim; a++) p->opad[a] = d.o[a] - nb * d.d[a];

    StepAParams &pa = p->pa;
    pa = StepAParams{};
    pa.g = g;
    pa.geom = geom;
    pa.nd = d.ndim;
    pa.nb = nb;
    pa.dt2 = d.dt * d.dt;
    const int round1 = 8 * ((g.n1 + 7) / 8), round2 = 8 * ((g.n2 + 7) / 8);
    switch (geom) {
        case 0:  // cart 2D: kernel axes (x, z) = memory (2, 1)
            pa.pri[0] = 1, pa.pri[1] = 0;
            pa.mask = 1;  // freeSurf_2D unconditional (MAWEFDcart2Dgpu.cu:424)
            pa.spill = round2 - g.n2;
            pa.shell = 6, pa.shell_axes = 1;
            pa.dd1 = d.d[0] * d.d[0];
            pa.dd2 = d.d[1] * d.d[1];
            break;
        case 1:  // cart 3D: kernel axes (x, y, z) = memory (2, 3, 1)
            pa.pri[0] = 1, pa.pri[1] = 2, pa.pri[2] = 0;
            pa.mask = 2;  // freeSurf_3D unconditional before the boundary (MAWEFDcart3Dgpu.cu:417)
            pa.shell = 6, pa.shell_axes = 7;
            pa.dd1 = d.d[0] * d.d[0];
            pa.dd2 = d.d[1] * d.d[1];
            pa.dd3 = d.d[2] * d.d[2];
            break;
        case 2:  // polar: kernel axes (r, theta) = memory (1, 2)
            pa.pri[0] = 0, pa.pri[1] = 1;
            pa.mask = d.fsrf ? 3 : 0;
            pa.spill = round1 - g.n1;
            pa.shell = 6, pa.shell_axes = 2;
            break;
        default:  // spherical: kernel axes (r, phi, theta) = memory (1, 3, 2)
            pa.pri[0] = 0, pa.pri[1] = 2, pa.pri[2] = 1;
            pa.mask = d.fsrf ? 3 : 0;
            pa.spill = round1 - g.n1;
            pa.shell = 0, pa.shell_axes = 0;
            break;
    }
    (void)round1;

    // sponge factor by index, spongeKernel_2D/3D: exp(-|(i-1)^2 log(alpha)| / nb^2),
    // log of the float alpha in float (the C++ overload), the rest in double
    std::vector<double> dtab(nb + 1, 1.0);
    std::vector<float> ftab(nb + 1, 1.f);
    const float alpha = 0.90;
    for (int i = 1; i <= nb; i++) {
        dtab[i] = std::exp(-1.0 * std::fabs((std::pow((i - 1.0), 2) * (double)std::log(alpha)) / (std::pow(nb, 2))));
        ftab[i] = (float)dtab[i];
    }
    double *d_dtab = nullptr;
    float *d_ftab = nullptr;
    AWE_TRY(upload_t(p, &d_dtab, dtab.data(), dtab.size()));
    AWE_TRY(upload_t(p, &d_ftab, ftab.data(), ftab.size()));
    pa.dtab = d_dtab;
    pa.ftab = d_ftab;

    // metric tables, evaluated as the kernels do per cell (spher_kernels.cu:404-526)
    if (geom == 2) {
        const float dra = d.d[0], dth = d.d[1], ora = p->opad[0];
        std::vector<float> am(g.n1), ap(g.n1), b(g.n1), b0(g.n1);
        for (int ira = 0; ira < g.n1; ira++) {
            const float ra = dra * ira + ora;
            am[ira] = (1 / (dra * dra)) + (1 / (2 * ra * dra));
            ap[ira] = (1 / (dra * dra)) - (1 / (2 * ra * dra));
            b[ira] = (1 / (ra * ra * dth * dth));
            b0[ira] = (-2 / (ra * ra * dth * dth));
        }
        pa.a0 = (-2 / (dra * dra));
        float *t0 = nullptr, *t1 = nullptr, *t2 = nullptr, *t3 = nullptr;
        AWE_TRY(upload_t(p, &t0, am.data(), am.size()));
        AWE_TRY(upload_t(p, &t1, ap.data(), ap.size()));
        AWE_TRY(upload_t(p, &t2, b.data(), b.size()));
        AWE_TRY(upload_t(p, &t3, b0.data(), b0.size()));
        pa.tr0 = t0, pa.tr1 = t1, pa.tr2 = t2, pa.tr3 = t3;
    } else if (geom == 3) {
        const float dra = d.d[0], dth = d.d[1], dph = d.d[2], ora = p->opad[0], oth = p->opad[1];
        pa.dd1 = 2 * dra;
        pa.dd2 = dra * dra;
        pa.dd3 = 2 * dth;
        pa.dd4 = dth * dth;
        pa.dd5 = dph * dph;
        std::vector<float> a2(g.n1), cr(g.n1), B((size_t)g.n1 * g.n2), D((size_t)g.n1 * g.n2);
        for (int ira = 0; ira < g.n1; ira++) {
            const float ra = dra * ira + ora;
            a2[ira] = (2 / ra);
            cr[ira] = (1 / (ra * ra));
            for (int ith = 0; ith < g.n2; ith++) {
                const float th = dth * ith + oth;
                B[(size_t)ith * g.n1 + ira] = (std::cos(th) / (ra * ra * std::sin(th)));
                D[(size_t)ith * g.n1 + ira] = (1 / (ra * ra * std::sin(th) * std::sin(th)));
            }
        }
        float *t0 = nullptr, *t1 = nullptr, *u0 = nullptr, *u1 = nullptr;
        AWE_TRY(upload_t(p, &t0, a2.data(), a2.size()));
        AWE_TRY(upload_t(p, &t1, cr.data(), cr.size()));
        AWE_TRY(upload_t(p, &u0, B.data(), B.size()));
        AWE_TRY(upload_t(p, &u1, D.data(), D.size()));
        pa.tr0 = t0, pa.tr1 = t1, pa.tt0 = u0, pa.tt1 = u1;
    }

    const size_t cells = (size_t)g.cells();
    AWE_TRY(dev_alloc(p, (void **)&p->u[0], cells * sizeof(float)));
    AWE_TRY(dev_alloc(p, (void **)&p->u[1], cells * sizeof(float)));
    AWE_TRY(dev_alloc(p, (void **)&p->vel, cells * sizeof(float)));
    AWE_TRY(dev_alloc(p, (void **)&p->corner_off, 8 * sizeof(long long)));
    if (pa.shell > 0) AWE_TRY(dev_alloc(p, (void **)&p->aux, cells * sizeof(float)));

    pa.nshot = 1;
    pa.shot_cells = g.cells();
    // TMA-staged spherical step for AWE_FAST; AWE_STEP_KERNEL=simple keeps the
    // register-march kernel (the tests compare both)
    const char *kern = std::getenv("AWE_STEP_KERNEL");
    const bool force_simple = kern && std::strcmp(kern, "simple") == 0;
    // (the TMA kernels' sponge index walks the axes in this grid's priority
    // order (r, phi, theta) = memory axes (1, 3, 2))
    const bool pri_rpt = pa.pri[0] == 0 && pa.pri[1] == 2 && pa.pri[2] == 1;
    if (geom == 3 && d.precision == AWE_FAST && !force_simple && pri_rpt && sphA_tma_eligible(g, nb) &&
        sphA_tma_maps(p->sph_maps, p->u, p->vel, g, 1)) {
        AWE_TRY(dev_alloc(p, (void **)&p->sched_counter, sizeof(unsigned long long)));
        AWE_TRY(dev_alloc(p, (void **)&p->d_err, sizeof(int)));
        CUDA_TRY(cudaMemset(p->sched_counter, 0, sizeof(unsigned long long)));
        CUDA_TRY(cudaMemset(p->d_err, 0, sizeof(int)));
        cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, p->device);
        if (p->num_sms < 1) p->num_sms = 1;
        const char *spin = std::getenv("AWE_PIPELINE_SPIN_LIMIT");
        if (spin && *spin) p->spin_limit = std::atoll(spin);
        p->sph_tma = true;
    }
    // reciprocals of the Laplacian divisors (AWE_FAST multiplies; AWE_EXACT divides as the reference)
    const float dvs[5] = {pa.dd1, pa.dd2, pa.dd3, pa.dd4, pa.dd5};
    for (int j = 0; j < 5; j++) pa.rd[j] = dvs[j] != 0.f ? 1.f / dvs[j] : 0.f;

    // outputs: rows and snapshot windows as each program writes them
    const int jdata = d.jdata > 0 ? d.jdata : 1;
    p->nsmp = geom == 3 ? d.nt : d.nt / jdata;
    if (p->nsmp < 1) p->nsmp = 1;
    p->nsnap = d.jsnap > 0 ? (d.nt - 1) / d.jsnap + 1 : 0;
    const int npads[3] = {g.n1, g.n2, g.n3};
    for (int a = 0; a < 3; a++) {
        if (a >= d.ndim) {
            p->snap_f[a] = 0;
            p->snap_m[a] = 1;
        } else if (d.bnds) {
            p->snap_f[a] = 0;
            p->snap_m[a] = npads[a];
        } else {
            p->snap_m[a] = d.n[a];
            if (geom == 3) p->snap_f[a] = nb;                                                 // cut3d_sph
            else if (geom == 1) p->snap_f[a] = floor_first(d.o[a], p->opad[a], d.d[a], 0.0001f);  // cut3d
            else p->snap_f[a] = floor_first(d.o[a], p->opad[a], d.d[a], 0.f);                 // cut2d
        }
    }
    p->snap_transpose = geom == 2;
    p->snap_elems = (size_t)p->snap_m[0] * p->snap_m[1] * p->snap_m[2];
    return AWE_OK;
}

awe_status planA_model(awe_plan *p, const float *vel, const float *rfl) {
    const awe_desc &d = p->d;
    const Grid &g = p->g;
    StepAParams &pa = p->pa;
    const size_t cells = (size_t)g.cells();
    const int nb = p->nbd;
    p->h_vel_raw.assign(cells, 0.f);
    expand_model(d.ndim, vel, p->h_vel_raw.data(), nb, d.n);
    AWE_TRY(upload_t(p, &p->vel, p->h_vel_raw.data(), cells));
    const std::vector<float> &v = p->h_vel_raw;
    const float dt = d.dt;
    auto coef = [](float q) { return (1 - q) / (1 + q); };
    if (pa.geom == 0) {
        // MAWEFDcart2Dgpu.cu:280-285: h_vel indexed x-fastest; only the last
        // x sample survives the boundary kernel's loop
        const int nxpad = g.n2, nzpad = g.n1;
        pa.b2lo = coef(v[(size_t)kNopA * nxpad + nxpad - 1] * (dt / d.d[0]));
        pa.b2hi = coef(v[(size_t)(nzpad - kNopA - 1) * nxpad + nxpad - 1] * (dt / d.d[0]));
        if (d.refl) {
            if (!rfl) {
                set_error("refl=y needs a reflectivity image");
                return AWE_ERR_INVALID;
            }
            p->h_rfl_pad.assign(cells, 0.f);
            expand_model(2, rfl, p->h_rfl_pad.data(), nb, d.n);
        }
    } else if (pa.geom == 2) {
        const int nrapad = g.n1, nthpad = g.n2;
        pa.b2lo = coef(v[(size_t)kNopA * nrapad + nrapad - 1] * (dt / d.d[1]));
        pa.b2hi = coef(v[(size_t)(nthpad - kNopA - 1) * nrapad + nrapad - 1] * (dt / d.d[1]));
    } else if (pa.geom == 1) {
        // MAWEFDcart3Dgpu.cu:271-294 with its flat indices (the y-high table
        // filled as the loop intends; the reference writes only its diagonal)
        const size_t nxpad = g.n2, nypad = g.n3, nzpad = g.n1, n2 = nxpad * nzpad;
        std::vector<float> bzl(nxpad * nypad), bzh(nxpad * nypad), bxl(nzpad * nypad), bxh(nzpad * nypad),
            byl(nxpad * nzpad), byh(nxpad * nzpad);
        for (size_t ix = 0; ix < nxpad; ix++)
            for (size_t iy = 0; iy < nypad; iy++) {
                bzl[iy * nxpad + ix] = coef(v[iy * n2 + kNopA * nxpad + ix] * (dt / d.d[0]));
                bzh[iy * nxpad + ix] = coef(v[iy * n2 + (nzpad - kNopA - 1) * nxpad + ix] * (dt / d.d[0]));
            }
        for (size_t iz = 0; iz < nzpad; iz++)
            for (size_t iy = 0; iy < nypad; iy++) {
                bxl[iy * nzpad + iz] = coef(v[iy * n2 + iz * nxpad + kNopA] * (dt / d.d[1]));
                bxh[iy * nzpad + iz] = coef(v[iy * n2 + iz * nxpad + nxpad - kNopA - 1] * (dt / d.d[1]));
            }
        for (size_t iz = 0; iz < nzpad; iz++)
            for (size_t ix = 0; ix < nxpad; ix++) {
                byl[iz * nxpad + ix] = coef(v[kNopA * n2 + iz * nxpad + ix] * (dt / d.d[2]));
                byh[iz * nxpad + ix] = coef(v[(nypad - kNopA - 1) * n2 + iz * nxpad + ix] * (dt / d.d[2]));
            }
        float *t[6] = {nullptr};
        AWE_TRY(upload_t(p, &t[0], bzl.data(), bzl.size()));
        AWE_TRY(upload_t(p, &t[1], bzh.data(), bzh.size()));
        AWE_TRY(upload_t(p, &t[2], bxl.data(), bxl.size()));
        AWE_TRY(upload_t(p, &t[3], bxh.data(), bxh.size()));
        AWE_TRY(upload_t(p, &t[4], byl.data(), byl.size()));
        AWE_TRY(upload_t(p, &t[5], byh.data(), byh.size()));
        for (int k = 0; k < 6; k++) pa.tb[k] = t[k];
    }
    return AWE_OK;
}

// reflectivity of inject_sources_{2D,3D}: first neighbour (kernel order, its
// own flat indexing) whose velocity differs; neighbours outside the array
// (where the reference reads out of bounds) count as equal
static float refl_scale(const std::vector<float> &v, long long s, long long rs, long long ps, int nd) {
    static const int o2[7][2] = {{1, 0}, {0, 1}, {1, 1}, {0, -1}, {-1, -1}, {1, -1}, {-1, 1}};
    static const int o3[26][3] = {{0, 1, 0},   {1, 0, 0},   {0, 0, 1},   {0, -1, 0},  {-1, 0, 0},  {0, 0, -1},
                                  {0, 1, 1},   {0, -1, -1}, {0, 1, -1},  {0, -1, 1},  {1, 1, 0},   {-1, -1, 0},
                                  {1, -1, 0},  {-1, 1, 0},  {1, 0, 1},   {-1, 0, -1}, {1, 0, -1},  {-1, 0, 1},
                                  {1, 0, -1},  {1, 1, 1},   {1, 1, -1},  {1, -1, 1},  {1, -1, -1}, {-1, 1, 1},
                                  {-1, 1, -1}, {-1, -1, 1}};
    const long long n = (long long)v.size();
    if (s < 0 || s >= n) return 0.f;
    const float v0 = v[s];
    const int cnt = nd == 2 ? 7 : 26;
    for (int k = 0; k < cnt; k++) {
        const long long t = nd == 2 ? s + o2[k][0] * rs + o2[k][1] : s + o3[k][0] * ps + o3[k][1] * rs + o3[k][2];
        if (t < 0 || t >= n) continue;
        if (v0 != v[t]) return std::fabs((v0 - v[t]) / (v0 + v[t]));
    }
    return 0.f;
}

static awe_status prepare_injection(awe_plan *p, bool &scaled) {
    const awe_desc &d = p->d;
    const Grid &g = p->g;
    const int geom = p->pa.geom, ns = p->ns;
    scaled = d.expl != 0;
    if (!scaled || ns == 0) return AWE_OK;
    std::vector<float> sc((size_t)ns * 8, 1.f);
    for (int s = 0; s < ns; s++) {
        const Lint &l = p->h_src_lint[s];
        if (geom == 0 && d.refl) {  // inject_sources_2D_refl: rfl with the x-fastest flat index
            const long long nx = g.n2;
            const long long f[4] = {(long long)l.jz * nx + l.jx, (long long)(l.jz + 1) * nx + l.jx,
                                    (long long)l.jz * nx + l.jx + 1, (long long)(l.jz + 1) * nx + l.jx + 1};
            for (int c = 0; c < 4; c++) sc[s * 8 + c] = p->h_rfl_pad[f[c]];
            continue;
        }
        float r = 0.f;
        if (geom == 0) r = refl_scale(p->h_vel_raw, (long long)l.jz * g.n2 + l.jx, g.n2, 0, 2);
        else if (geom == 1)
            r = refl_scale(p->h_vel_raw, (long long)l.jy * g.n2 * g.n1 + (long long)l.jz * g.n2 + l.jx, g.n2,
                           (long long)g.n2 * g.n1, 3);
        else if (geom == 2) r = refl_scale(p->h_vel_raw, (long long)l.jz * g.n1 + l.jx, g.n1, 0, 2);
        else
            r = refl_scale(p->h_vel_raw, (long long)l.jy * g.n1 * g.n2 + (long long)l.jz * g.n1 + l.jx, g.n1,
                           (long long)g.n1 * g.n2, 3);
        for (int c = 0; c < 8; c++) sc[s * 8 + c] = r;
    }
    if (p->inj_scale) dev_free(p, p->inj_scale);
    p->inj_scale = nullptr;
    AWE_TRY(upload_t(p, &p->inj_scale, sc.data(), sc.size()));
    return AWE_OK;
}

// hook (may be null): called at the start of every iteration, before the
// injection, with prev = the previous level (sponge pending) and cur = the
// current level
awe_status planA_run(awe_plan *p, const float *d_wav, int ncs, float *d_dat, float *d_wfl, cudaStream_t s,
                     const StepHook *hook) {
    const awe_desc &d = p->d;
    const Grid &g = p->g;
    const StepAParams &pa = p->pa;
    const bool exact = d.precision == AWE_EXACT;
    const size_t bytes = (size_t)g.cells() * sizeof(float) * (pa.nshot > 0 ? pa.nshot : 1);
    bool scaled = false;
    AWE_TRY(prepare_injection(p, scaled));
    CUDA_TRY(cudaMemsetAsync(p->u[0], 0, bytes, s));
    CUDA_TRY(cudaMemsetAsync(p->u[1], 0, bytes, s));
    CUDA_TRY(cudaMemsetAsync(d_dat, 0, (size_t)p->nsmp * p->nr * sizeof(float), s));
    if (p->nsnap > 0 && !d_wfl && p->snap_cb && !p->d_snap_tmp)
        AWE_TRY(dev_alloc(p, (void **)&p->d_snap_tmp, p->snap_elems * sizeof(float)));
    p->snap_pending = -1;  // a frame left queued by a failed run is not delivered

    if (p->sph_tma) {  // maps of this run's level fields; the work counter restarts with every run
        if (!sphA_tma_maps(p->sph_maps, p->u, p->vel, g, pa.nshot)) {
            set_error("tensor-map encoding of the spherical step failed");
            return AWE_ERR_CUDA;
        }
        const char *lenv = std::getenv("AWE_TMA_CHUNK");
        p->sph_shape = sphA_tma_shape(g, pa.nshot, p->num_sms, lenv ? std::atoi(lenv) : 0);
        CUDA_TRY(cudaMemsetAsync(p->sched_counter, 0, sizeof(unsigned long long), s));
        p->sched_base = 0;
    }
    const int jdata = d.jdata > 0 ? d.jdata : 1;
    long long launches = 0;
    float *cur = p->u[1], *nxt = p->u[0];
    int itr = 0, isnap = 0;
    for (int it = 0; it < d.nt; it++) {
        if (hook) AWE_TRY((*hook)(it, nxt, cur, s));
        if (p->ns > 0) {
            const PointsAt ps = points_at(p, p->src, p->ns, p->src_rows, it);
            launch_injectA(exact, d.ndim, cur, ps.pts, p->inj_scale, p->ns, d_wav, it, scaled, p->corner_off, s,
                           ps.stride, ncs);
            launches++;
        }
        prof_begin(p, s);
        if (p->sph_tma) {
            const int ic = cur == p->u[0] ? 0 : 1;  // nxt is the other level
            const cudaError_t e =
                launch_stepA_sph_tma(p->sph_maps[ic], p->sph_maps[2 + (1 - ic)], p->sph_maps[4], nxt, pa,
                                     p->sph_shape, p->sched_counter, p->sched_base, p->d_err, p->spin_limit, s);
            p->sched_base += (unsigned long long)p->sph_shape.items + p->sph_shape.grid;
            if (e != cudaSuccess) {
                set_error("spherical TMA step launch failed: %s", cudaGetErrorString(e));
                return AWE_ERR_CUDA;
            }
        } else {
            launch_stepA(pa.geom, exact, cur, nxt, p->vel, pa, s);
        }
        prof_end(p, s);
        launches++;
        if (pa.shell > 0) {
            launch_bcA(exact, cur, nxt, p->aux, pa, s);
            launches += 2;
        }
        std::swap(cur, nxt);  // cur: the new level (final); nxt: previous (sponge pending)
        int row = -1;
        if (pa.geom == 1) {  // MAWEFDcart3Dgpu.cu:432-442: pre-incremented row
            if (it % jdata == 0) {
                itr += 1;
                if (itr < p->nsmp) row = itr;
            }
        } else if (pa.geom == 3) {
            row = it;
        } else if (it < p->nsmp) {
            row = it;
        }
        if (row >= 0 && p->nr > 0) {
            const PointsAt pr = points_at(p, p->rec, p->nr, p->rec_rows, it);
            launch_extract_off(d.ndim, exact, cur, pr.pts, p->nr, d_dat + (size_t)row * p->nr, nullptr, nullptr,
                               nullptr, g, p->corner_off, s, pr.stride);
            launches++;
        }
        if (p->nsnap > 0 && it % d.jsnap == 0) {
            float *frame = d_wfl ? d_wfl + (size_t)isnap * p->snap_elems : p->d_snap_tmp;
            if (frame) {
                if (p->snap_transpose)
                    launch_snapshot_transpose2(cur, frame, g, p->snap_f[0], p->snap_f[1], p->snap_m[0], p->snap_m[1],
                                               s);
                else
                    launch_snapshot(d.ndim, cur, frame, g, p->snap_f[0], p->snap_f[1], p->snap_f[2], p->snap_m[0],
                                    p->snap_m[1], p->snap_m[2], nullptr, nullptr, nullptr, s);
                launches++;
                AWE_TRY(deliver_snapshot(p, frame, isnap, it, s));
            }
            isnap++;
        }
    }
    p->launches = launches;
    return flush_snapshots(p);
}

}  // namespace awe
