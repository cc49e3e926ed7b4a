/* FP64 adjoint oracle for the misfit gradient of the CPU-program scheme.
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE: only tests/ load it, as the checker
 * of the engine's adjoint (awe_gradient).
 *
 * The reference has no adjoint; this file states the discrete adjoint of
 * the forward map that MAWEFDcart{2D,3D}cpu.c define (the map restated in
 * awe_oracle.c, from which the coefficient, sponge, one-way ABC and
 * interpolation helpers are reused), in double precision, with every forward
 * state kept in memory (small grids only).
 *
 * Forward map, per step k (V_k = field after its own sponge, V_0 = V_-1 = 0):
 *   P   = W V_{k-1}                          (second sponge of the old level)
 *   N   = I (2 V_k + vel2 L V_k - P) + (1 - I) P + S_k
 *   N'  = ABC(N; um = V_k)                   (3D, abcone3d_apply)
 *   V_{k+1} = W N'
 *   d_k = R (W V_k)        for k % jdata == 0 (row k / jdata)
 * with W the per-cell sponge factor (product of the axis factors), I the
 * mask of cells at least nop from every face, L the 2N-order Laplacian,
 * vel2 = v^2 dt^2 (zero on the free-surface rows), S_k the injection
 * (wav * w_corner) * vel2 at each source corner, R the receiver gather.
 * Misfit J = 0.5 sum_k ||d_k - dobs_k||^2.
 *
 * Adjoint, k = nt-1 .. 0, with mu_{k+1} = W lambda_{k+1} (mu_nt = 0):
 *   (nu_k, kappa_k) = ABC^T(mu_{k+1})       (nu: adjoint of N, kappa: of um)
 *   lambda_k = 2 I nu_k + L(I vel2 nu_k) + kappa_k + W (1 - 2 I) nu_{k+1}
 *              + W R^T r_k                   (r = d - dobs, rows that exist)
 *   dJ/dvel2 += I nu_k L(V_k) + sum_sources nu_k[node] wav w_corner
 * The gradient with respect to m = 1/v^2 is dJ/dvel2 * (-vel2 v^2) on the
 * padded grid, folded onto the model by the adjoint of the edge-replicating
 * padding.  Boundary coefficients (one-way ABC, sponge) are held fixed. */
#define AWE_REAL_DOUBLE
#include "awe_oracle.c"

typedef struct {
    int nd, nop, nbd, n1, n2, n3; /* padded sizes; n3 = 1 in 2D */
    size_t sx, sy, np;
    double c0, cz[11], cx[11], cy[11];
} g_t;

static double lap_at(const g_t *g, const double *u, size_t i) {
    double lap = u[i] * g->c0;
    for (int k = 1; k <= g->nop; k++) {
        lap += (u[i - k] + u[i + k]) * g->cz[k] + (u[i - k * g->sx] + u[i + k * g->sx]) * g->cx[k];
        if (g->nd == 3) lap += (u[i - k * g->sy] + u[i + k * g->sy]) * g->cy[k];
    }
    return lap;
}

/* L^T applied to a field that is zero outside the interior, at any cell */
static double lapT_at(const g_t *g, const double *f, int iz, int ix, int iy) {
    const size_t i = (size_t)iy * g->sy + (size_t)ix * g->sx + iz;
    double s = f[i] * g->c0;
    for (int k = 1; k <= g->nop; k++) {
        if (iz - k >= 0) s += f[i - k] * g->cz[k];
        if (iz + k < g->n1) s += f[i + k] * g->cz[k];
        if (ix - k >= 0) s += f[i - k * g->sx] * g->cx[k];
        if (ix + k < g->n2) s += f[i + k * g->sx] * g->cx[k];
        if (g->nd == 3) {
            if (iy - k >= 0) s += f[i - k * g->sy] * g->cy[k];
            if (iy + k < g->n3) s += f[i + k * g->sy] * g->cy[k];
        }
    }
    return s;
}

/* one update uo[i] = um[a] + (um[i] - uo[b]) * c and its transpose */
static void abc_fwd1(double *uo, const double *um, size_t i, size_t a, size_t b, double c) {
    uo[i] = um[a] + (um[i] - uo[b]) * c;
}
static void abc_adj1(double *mu, double *kap, size_t i, size_t a, size_t b, double c) {
    const double t = mu[i];
    mu[i] = 0;
    mu[b] -= c * t;
    kap[a] += t;
    kap[i] += c * t;
}

/* abcone3d_apply (fdutil.c:2085-2177) in FP64, forward (adj = 0) or its
 * transpose (adj = 1: updates visited in reverse order) */
static void abc3_run(const g_t *g, const abc3 *a, int fsrf, double *uo, const double *um, double *mu, double *kap,
                     int adj) {
    const int nop = g->nop, nz = g->n1, nx = g->n2, ny = g->n3;
    const size_t sx = g->sx, sy = g->sy;
    for (int pass = 0; pass < 3; pass++) {
        const int ps = adj ? 2 - pass : pass;
        for (int l1 = 0; l1 < (ps == 2 ? nx : ny); l1++)
            for (int l2 = 0; l2 < (ps == 0 ? nx : nz); l2++)
                for (int jj = 0; jj < nop; jj++) {
                    const int iop = adj ? nop - 1 - jj : jj;
                    size_t base, st;
                    int n;
                    double bl, bh;
                    if (ps == 0) { /* axis-1 faces: line (iy = l1, ix = l2) */
                        base = (size_t)l1 * sy + (size_t)l2 * sx;
                        st = 1;
                        n = nz;
                        bl = a->zl[(size_t)l1 * nx + l2];
                        bh = a->zh[(size_t)l1 * nx + l2];
                    } else if (ps == 1) { /* axis-2 faces: line (iy = l1, iz = l2) */
                        base = (size_t)l1 * sy + l2;
                        st = sx;
                        n = nx;
                        bl = a->xl[(size_t)l1 * nz + l2];
                        bh = a->xh[(size_t)l1 * nz + l2];
                    } else { /* axis-3 faces: line (ix = l1, iz = l2) */
                        base = (size_t)l1 * sx + l2;
                        st = sy;
                        n = ny;
                        bl = a->yl[(size_t)l1 * nz + l2];
                        bh = a->yh[(size_t)l1 * nz + l2];
                    }
                    const int top = !(ps == 0 && fsrf);
                    const size_t il = base + (size_t)(nop - iop) * st, ih = base + (size_t)(n - nop + iop - 1) * st;
                    if (!adj) {
                        if (top) abc_fwd1(uo, um, il, il + st, il + st, bl);
                        abc_fwd1(uo, um, ih, ih - st, ih - st, bh);
                    } else {
                        abc_adj1(mu, kap, ih, ih - st, ih - st, bh);
                        if (top) abc_adj1(mu, kap, il, il + st, il + st, bl);
                    }
                }
    }
}

typedef struct {
    const g_t *g;
    const double *W, *vel2;
    const unsigned char *I;
    const lint *cs;
    int ns, nc, expl, dabc, fsrf;
    const size_t *off;
    const float *wav;
    const abc3 *a;
} fctx;

/* one forward step: Vn = W ABC(N; B), N = I (2B + vel2 L B - W A) + (1-I) W A + S_k */
static void fstep(const fctx *c, const double *A, const double *B, double *Vn, double *N, int k) {
    const g_t *g = c->g;
    const size_t sx = g->sx, sy = g->sy;
    for (int iy = 0; iy < g->n3; iy++)
        for (int ix = 0; ix < g->n2; ix++)
            for (int iz = 0; iz < g->n1; iz++) {
                const size_t i = iy * sy + ix * sx + iz;
                const double P = c->W[i] * A[i];
                N[i] = c->I[i] ? 2 * B[i] + c->vel2[i] * lap_at(g, B, i) - P : P;
            }
    for (int s = 0; s < c->ns; s++) {
        const lint *q = &c->cs[s];
        const size_t base = (size_t)q->jy * sy + (size_t)q->jx * sx + (size_t)q->jz;
        const double dd = c->expl ? c->wav[(size_t)k] : c->wav[(size_t)k * c->ns + s];
        for (int j = 0; j < c->nc; j++) N[base + c->off[j]] += dd * q->w[j] * c->vel2[base + c->off[j]];
    }
    if (c->dabc && g->nd == 3) abc3_run(g, c->a, c->fsrf, N, B, NULL, NULL, 0);
    for (size_t i = 0; i < g->np; i++) Vn[i] = c->W[i] * N[i];
}

/* round x / scale to `bits` significant bits (round half to even), times
 * scale.  bits == 11 follows IEEE half precision below its normal range
 * (|x / scale| < 2^-14: a fixed spacing of 2^-24, gradual underflow) */
double orc_quantize(double x, double scale, int bits) {
    if (x == 0 || scale == 0) return x;
    const double y = x / scale;
    if (bits == 11 && fabs(y) < ldexp(1.0, -14)) return ldexp(nearbyint(ldexp(y, 24)), -24) * scale;
    int e;
    const double m = frexp(y, &e); /* |m| in [0.5, 1) */
    const double t = ldexp(m, bits);
    return ldexp(nearbyint(t), e - bits) * scale;
}

/* Block floating point as the engine's AWE_CKPT_BFP16 checkpoints store a
 * level (k_bfp_store): the level rounded to float, then per block of 64
 * consecutive cells s = max|v| / 32767, q = round(v * (1/s)) (half to even,
 * clamped to +-32767), v' = q * s, all in float; blocks with max|v| <= 1e-30
 * are stored as zeros. */
void orc_quantize_bfp16(double *u, size_t n) {
    for (size_t b = 0; b < n; b += 64) {
        const size_t e = b + 64 < n ? b + 64 : n;
        float m = 0.f;
        for (size_t i = b; i < e; i++) m = fabsf((float)u[i]) > m ? fabsf((float)u[i]) : m;
        const float sc = m > 1e-30f ? m / 32767.f : 0.f;
        const float inv = m > 1e-30f ? 1.f / sc : 0.f;
        for (size_t i = b; i < e; i++) {
            const float t = (float)u[i] * inv;
            float q = nearbyintf(t);
            q = q > 32767.f ? 32767.f : (q < -32767.f ? -32767.f : q);
            u[i] = (double)(q * sc);
        }
    }
}

/* The model is either velocity in float (vel_in: vel2 = v * (v * dt^2) in
 * float, as the engine) or slowness squared in double (m_in: vel2 = dt^2 / m
 * in double, so that finite differences of J are free of float rounding). */
static int grad_impl(const orc_par *p, int ndim, int jdata, const float *vel_in, const double *m_in, const float *wav,
                     int ns, const float *sou, int nr, const float *rec, const float *dobs, double *grad,
                     double *misfit, double *dsyn, int ckpt_every, int ckpt_bits, int image) {
    if (p->hybrid || jdata < 1) return 1;
    g_t g;
    g.nd = ndim;
    g.nop = p->fdorder / 2;
    if (g.nop < 1 || g.nop > 10) return 1;
    orc_par q = *p;
    if (ndim == 2) q.n3 = 1;
    orc_cart_padded(&q, &g.nbd, &g.n1, &g.n2, &g.n3);
    if (ndim == 2) g.n3 = 1;
    const int nbd = g.nbd, nop = g.nop, nz = g.n1, nx = g.n2, ny = g.n3;
    g.sx = nz;
    g.sy = (size_t)nz * nx;
    g.np = g.sy * ny;
    const size_t np = g.np, sx = g.sx, sy = g.sy;
    float d2[64], d1[64], dd[3] = {p->d1, p->d2, p->d3};
    fdcoef(nop, ndim, dd, p->optfd, d2, d1);
    g.c0 = d2[0];
    for (int k = 1; k <= nop; k++) {
        g.cz[k] = d2[k];
        g.cx[k] = d2[nop + k];
        g.cy[k] = ndim == 3 ? d2[2 * nop + k] : 0;
    }
    const float dt = p->dt;
    const int nt = p->nt, nsmp = (nt - 1) / jdata + 1;

    const size_t nmod = (size_t)p->n1 * p->n2 * (ndim == 3 ? p->n3 : 1);
    float *vin = malloc(nmod * sizeof(float));
    double *min = malloc(nmod * sizeof(double)), *mpad = malloc(np * sizeof(double));
    for (size_t i = 0; i < nmod; i++) {
        vin[i] = m_in ? (float)(1.0 / sqrt(m_in[i])) : vel_in[i];
        min[i] = m_in ? m_in[i] : 0.0;
    }
    float *vpad = malloc(np * sizeof(float));
    double *vel2 = malloc(np * sizeof(double));
    if (ndim == 2) expand2(vin, vpad, nbd, p->n1, p->n2);
    else expand3(vin, vpad, nbd, p->n1, p->n2, p->n3);
    if (m_in) { /* the same edge replication of m, in double */
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++)
                for (int iz = 0; iz < nz; iz++) {
                    int jz = iz - nbd, jx = ix - nbd, jy = ndim == 3 ? iy - nbd : 0;
                    const int m1 = p->n1, m2 = p->n2, m3 = ndim == 3 ? p->n3 : 1;
                    jz = jz < 0 ? 0 : (jz >= m1 ? m1 - 1 : jz);
                    jx = jx < 0 ? 0 : (jx >= m2 ? m2 - 1 : jx);
                    jy = jy < 0 ? 0 : (jy >= m3 ? m3 - 1 : jy);
                    mpad[iy * sy + ix * sx + iz] = min[((size_t)jy * m2 + jx) * m1 + jz];
                }
    }
    abc3 a = {0};
    double *W = malloc(np * sizeof(double));
    for (size_t i = 0; i < np; i++) W[i] = 1;
    if (p->dabc) {
        float spo[4096];
        sponge_w(nbd, spo);
        const int len[3] = {nz, nx, ny};
        double *t[3];
        for (int ax = 0; ax < 3; ax++) {
            t[ax] = malloc(len[ax] * sizeof(double));
            for (int i = 0; i < len[ax]; i++) t[ax][i] = 1;
            if (ax < ndim)
                for (int i = 0; i < nbd && i < len[ax]; i++) t[ax][i] = t[ax][len[ax] - 1 - i] = spo[nbd - i - 1];
        }
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++)
                for (int iz = 0; iz < nz; iz++) W[iy * sy + ix * sx + iz] = t[0][iz] * t[1][ix] * t[2][iy];
        for (int ax = 0; ax < 3; ax++) free(t[ax]);
        if (ndim == 3) {
            a.zl = malloc((size_t)ny * nx * sizeof(float));
            a.zh = malloc((size_t)ny * nx * sizeof(float));
            a.xl = malloc((size_t)ny * nz * sizeof(float));
            a.xh = malloc((size_t)ny * nz * sizeof(float));
            a.yl = malloc((size_t)nx * nz * sizeof(float));
            a.yh = malloc((size_t)nx * nz * sizeof(float));
            for (int iy = 0; iy < ny; iy++)
                for (int ix = 0; ix < nx; ix++) {
                    float d = vpad[iy * sy + ix * sx + nbd] * dt / p->d1;
                    a.zl[(size_t)iy * nx + ix] = (1 - d) / (1 + d);
                    d = vpad[iy * sy + ix * sx + nz - nbd - 1] * dt / p->d1;
                    a.zh[(size_t)iy * nx + ix] = (1 - d) / (1 + d);
                }
            for (int iy = 0; iy < ny; iy++)
                for (int iz = 0; iz < nz; iz++) {
                    float d = vpad[iy * sy + nbd * sx + iz] * dt / p->d2;
                    a.xl[(size_t)iy * nz + iz] = (1 - d) / (1 + d);
                    d = vpad[iy * sy + (nx - nbd - 1) * sx + iz] * dt / p->d2;
                    a.xh[(size_t)iy * nz + iz] = (1 - d) / (1 + d);
                }
            for (int ix = 0; ix < nx; ix++)
                for (int iz = 0; iz < nz; iz++) {
                    float d = vpad[nbd * sy + ix * sx + iz] * dt / p->d3;
                    a.yl[(size_t)ix * nz + iz] = (1 - d) / (1 + d);
                    d = vpad[(ny - nbd - 1) * sy + ix * sx + iz] * dt / p->d3;
                    a.yh[(size_t)ix * nz + iz] = (1 - d) / (1 + d);
                }
        }
    }
    const float dt2 = dt * dt;
    for (size_t i = 0; i < np; i++)
        vel2[i] = m_in ? (double)dt * (double)dt / mpad[i] : (double)(vpad[i] * (vpad[i] * dt2));
    if (p->fsrf)
        for (size_t line = 0; line < (size_t)nx * ny; line++)
            for (int iz = 0; iz < nbd + 1 && iz < nz; iz++) vel2[line * nz + iz] = 0;
    unsigned char *I = malloc(np);
    for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nx; ix++)
            for (int iz = 0; iz < nz; iz++)
                I[iy * sy + ix * sx + iz] = iz >= nop && iz < nz - nop && ix >= nop && ix < nx - nop &&
                                            (ndim == 2 || (iy >= nop && iy < ny - nop));

    /* points: flat base index + corner offsets + weights (lint*_make) */
    const float ozp = p->o1 - nbd * p->d1, oxp = p->o2 - nbd * p->d2, oyp = p->o3 - nbd * p->d3;
    const int nc = ndim == 3 ? 8 : 4;
    size_t off[8] = {0, 1, sx, sx + 1, sy, sy + 1, sy + sx, sy + sx + 1};
    lint *cs = malloc((ns > 0 ? ns : 1) * sizeof(lint)), *cr = malloc((nr > 0 ? nr : 1) * sizeof(lint));
    for (int i = 0; i < ns; i++) {
        if (ndim == 2) lint2d(sou[2 * i], sou[2 * i + 1], ozp, oxp, p->d1, p->d2, nz, nx, &cs[i]);
        else lint3d(sou[3 * i], sou[3 * i + 1], sou[3 * i + 2], ozp, oxp, oyp, p->d1, p->d2, p->d3, nz, nx, ny, &cs[i]);
    }
    for (int i = 0; i < nr; i++) {
        if (ndim == 2) lint2d(rec[2 * i], rec[2 * i + 1], ozp, oxp, p->d1, p->d2, nz, nx, &cr[i]);
        else lint3d(rec[3 * i], rec[3 * i + 1], rec[3 * i + 2], ozp, oxp, oyp, p->d1, p->d2, p->d3, nz, nx, ny, &cr[i]);
    }
#define BASE(c) ((size_t)(c)->jy * sy + (size_t)(c)->jx * sx + (size_t)(c)->jz)
#define WAVE(k, s) ((double)(p->expl ? wav[(size_t)(k)] : wav[(size_t)(k) * ns + (s)]))

    /* forward, every state kept: V[k] for k = 0..nt (V[-1] = 0) */
    double *V = calloc((size_t)(nt + 1) * np, sizeof(double));
    double *N = malloc(np * sizeof(double)), *zero = calloc(np, sizeof(double));
    double *r = calloc((size_t)nsmp * (nr > 0 ? nr : 1), sizeof(double));
    const fctx fc = {&g, W, vel2, I, cs, ns, nc, p->expl, p->dabc, p->fsrf, off, wav, &a};
    for (int k = 0; k < nt; k++) {
        const double *B = V + (size_t)k * np, *A = k > 0 ? V + (size_t)(k - 1) * np : zero;
        fstep(&fc, A, B, V + (size_t)(k + 1) * np, N, k);
        if (k % jdata == 0)
            for (int ir = 0; ir < nr; ir++) {
                double v = 0;
                for (int c = 0; c < nc; c++) {
                    const size_t n = BASE(&cr[ir]) + off[c];
                    v += W[n] * B[n] * cr[ir].w[c];
                }
                const size_t row = (size_t)(k / jdata) * nr + ir;
                if (dsyn) dsyn[row] = v;
                r[row] = image < 0 ? v - dobs[row] : (double)dobs[row]; /* an image back-propagates the data */
            }
    }
    double J = 0;
    for (size_t i = 0; i < (size_t)nsmp * nr; i++) J += 0.5 * r[i] * r[i];
    *misfit = J;

    /* checkpointed recompute: every ckpt_every steps the two levels V[k0-1],
     * V[k0] are rounded to ckpt_bits significant bits (one scale, the level's
     * max |v|, per level; ckpt_bits < 0: block floating point) and the
     * segment's later levels recomputed from them */
    if (ckpt_bits != 0 && ckpt_every > 0)  /* last segment first: each restart reads levels of the exact forward */
        for (int k0 = ((nt - 1) / ckpt_every) * ckpt_every; k0 >= 0; k0 -= ckpt_every) {
            for (int lv = k0 - 1; lv <= k0; lv++) {
                if (lv < 0) continue;
                double *u = V + (size_t)lv * np, amax = 0;
                if (ckpt_bits < 0) {
                    orc_quantize_bfp16(u, np);
                    continue;
                }
                for (size_t i = 0; i < np; i++) amax = fabs(u[i]) > amax ? fabs(u[i]) : amax;
                for (size_t i = 0; i < np; i++) u[i] = orc_quantize(u[i], amax, ckpt_bits);
            }
            for (int k = k0; k < k0 + ckpt_every - 1 && k < nt - 1; k++) {
                const double *B = V + (size_t)k * np, *A = k > 0 ? V + (size_t)(k - 1) * np : zero;
                fstep(&fc, A, B, V + (size_t)(k + 1) * np, N, k);
            }
        }

    /* adjoint */
    double *mu = calloc(np, sizeof(double)), *nu = malloc(np * sizeof(double));
    double *nun = calloc(np, sizeof(double)), *kap = calloc(np, sizeof(double));
    double *gv = calloc(np, sizeof(double)), *f = malloc(np * sizeof(double)), *lam = malloc(np * sizeof(double));
    for (int k = nt - 1; k >= 0; k--) {
        const double *Vk = V + (size_t)k * np;
        memcpy(nu, mu, np * sizeof(double));
        memset(kap, 0, np * sizeof(double));
        if (p->dabc && ndim == 3) abc3_run(&g, &a, p->fsrf, NULL, NULL, nu, kap, 1);
        for (size_t i = 0; i < np; i++) f[i] = I[i] ? (double)vel2[i] * nu[i] : 0;
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++)
                for (int iz = 0; iz < nz; iz++) {
                    const size_t i = iy * sy + ix * sx + iz;
                    lam[i] = (I[i] ? 2 * nu[i] : 0) + lapT_at(&g, f, iz, ix, iy) + kap[i] +
                             W[i] * (I[i] ? -1.0 : 1.0) * nun[i];
                    if (I[i]) gv[i] += nu[i] * (image == 0 ? Vk[i] : lap_at(&g, Vk, i));
                }
        if (k % jdata == 0)
            for (int ir = 0; ir < nr; ir++)
                for (int c = 0; c < nc; c++) {
                    const size_t n = BASE(&cr[ir]) + off[c];
                    lam[n] += W[n] * cr[ir].w[c] * r[(size_t)(k / jdata) * nr + ir];
                }
        for (int s = 0; s < ns && image != 0; s++)
            for (int c = 0; c < nc; c++) {
                const size_t n = BASE(&cs[s]) + off[c];
                gv[n] += nu[n] * WAVE(k, s) * cs[s].w[c];
            }
        for (size_t i = 0; i < np; i++) mu[i] = W[i] * lam[i];
        memcpy(nun, nu, np * sizeof(double));
    }
#undef BASE
#undef WAVE

    /* d vel2 / d m = -vel2 v^2, then the adjoint of the edge-replicating padding */
    const int m1 = p->n1, m2 = p->n2, m3 = ndim == 3 ? p->n3 : 1;
    memset(grad, 0, (size_t)m1 * m2 * m3 * sizeof(double));
    for (int iy = 0; iy < ny && image == 0; iy++) /* cross-correlation image: the model window */
        for (int ix = 0; ix < nx; ix++)
            for (int iz = 0; iz < nz; iz++) {
                const int jz = iz - nbd, jx = ix - nbd, jy = ndim == 3 ? iy - nbd : 0;
                if (jz >= 0 && jz < m1 && jx >= 0 && jx < m2 && jy >= 0 && jy < m3)
                    grad[((size_t)jy * m2 + jx) * m1 + jz] = gv[iy * sy + ix * sx + iz];
            }
    for (int iy = 0; iy < ny && image != 0; iy++)
        for (int ix = 0; ix < nx; ix++)
            for (int iz = 0; iz < nz; iz++) {
                const size_t i = iy * sy + ix * sx + iz;
                /* d vel2 / d m = -vel2^2 / dt^2 */
                const double gm = gv[i] * (-vel2[i] * vel2[i] / ((double)dt * (double)dt));
                int jz = iz - nbd, jx = ix - nbd, jy = ndim == 3 ? iy - nbd : 0;
                jz = jz < 0 ? 0 : (jz >= m1 ? m1 - 1 : jz);
                jx = jx < 0 ? 0 : (jx >= m2 ? m2 - 1 : jx);
                jy = jy < 0 ? 0 : (jy >= m3 ? m3 - 1 : jy);
                grad[((size_t)jy * m2 + jx) * m1 + jz] += gm;
            }
    free(vin);
    free(min);
    free(mpad);
    free(vpad);
    free(vel2);
    free(W);
    free(I);
    free(cs);
    free(cr);
    free(V);
    free(N);
    free(zero);
    free(r);
    free(mu);
    free(nu);
    free(nun);
    free(kap);
    free(gv);
    free(f);
    free(lam);
    free(a.zl);
    free(a.zh);
    free(a.xl);
    free(a.xh);
    free(a.yl);
    free(a.yh);
    return 0;
}

int orc_grad(const orc_par *p, int ndim, int jdata, const float *vel_in, const float *wav, int ns, const float *sou,
             int nr, const float *rec, const float *dobs, double *grad, double *misfit, double *dsyn) {
    return grad_impl(p, ndim, jdata, vel_in, NULL, wav, ns, sou, nr, rec, dobs, grad, misfit, dsyn, 0, 0, -1);
}

int orc_grad_m(const orc_par *p, int ndim, int jdata, const double *m, const float *wav, int ns, const float *sou,
               int nr, const float *rec, const float *dobs, double *grad, double *misfit, double *dsyn) {
    return grad_impl(p, ndim, jdata, NULL, m, wav, ns, sou, nr, rec, dobs, grad, misfit, dsyn, 0, 0, -1);
}

/* As orc_grad, with the adjoint sweep reading levels recomputed from
 * checkpoints rounded to `bits` significant bits every `every` steps (8: the
 * engine's BF16 checkpoints, 11: FP16 with its subnormal range, 24: FP32,
 * -1: the block floating point of AWE_CKPT_BFP16). */
int orc_grad_ckpt(const orc_par *p, int ndim, int jdata, const float *vel_in, const float *wav, int ns,
                  const float *sou, int nr, const float *rec, const float *dobs, int every, int bits, double *grad,
                  double *misfit, double *dsyn) {
    return grad_impl(p, ndim, jdata, vel_in, NULL, wav, ns, sou, nr, rec, dobs, grad, misfit, dsyn, every, bits, -1);
}

/* Reverse-time migration images on the same FP64 adjoint (the engine's
 * awe_rtm): the residual is the data themselves; condition 0 = zero-lag
 * cross-correlation sum_k I nu_k V_k on the model window, 1 = the Born
 * adjoint (the gradient formula with the data as residual). */
int orc_image(const orc_par *p, int ndim, int jdata, const float *vel_in, const float *wav, int ns, const float *sou,
              int nr, const float *rec, const float *data, int condition, double *image) {
    double unused = 0;
    if (condition != 0 && condition != 1) return 1;
    return grad_impl(p, ndim, jdata, vel_in, NULL, wav, ns, sou, nr, rec, data, image, &unused, NULL, 0, 0,
                     condition);
}
