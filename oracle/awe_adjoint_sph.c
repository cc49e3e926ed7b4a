/* CPU oracle, part 4: FP64 misfit gradient of the spherical GPU-program
 * scheme (the forward of MAWEFDspher3Dgpu.cu:449-566 as restated in
 * awe_oracle_gpu.c, gpu_spher3d).  TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 * The reference has no adjoint; this is the discrete adjoint of that forward
 * map, derived here, pinned by finite differences of its own misfit.
 *
 * Forward (U_0 = 0, A_{-1} = 0), it = 0 .. nt-1:
 *   A_it = U_it + S_it                         (injection into the current level)
 *   U_{it+1} = W M (c L A_it + 2 A_it - W A_{it-1})
 *   d_it = R U_{it+1}
 * c = dt^2 v^2 per cell, L the metric Laplacian on the interior (zero in the
 * 4-cell ring), W the sponge factor, M the free-surface mask (0 or 1), R the
 * trilinear receiver gather.  The levels are FP64, the sponge table and the
 * geometry as in gpu_spher3d; the metric terms in double.
 *
 * Adjoint of J = 0.5 sum |d - dobs|^2 (z_{nt+1} = z_{nt+2} = 0), j = nt .. 1:
 *   z_j = W M (L^T (c z_{j+1}) + 2 z_{j+1} - W z_{j+2} + R^T r_{j-1})
 *   dJ/dc = sum_{j = 0}^{nt-1} z_{j+1} L A_j
 * and dJ/dm = dJ/dc (-c^2 / dt^2) for m = 1/v^2, summed onto the model cells
 * by the transpose of the edge-replicating padding.  With expl = 1 the
 * injection's reflectivity scale (piecewise constant in v) is held fixed.
 *
 * Images (the engine's awe_rtm): image = 0 sums z_{j+1} A_j (zero-lag
 * cross-correlation) and returns the model window of the padded sum; image =
 * 1 is the gradient formula with the data themselves as the residual (Born
 * adjoint); image < 0 is the misfit gradient.
 *
 * Checkpoint emulation: every `every` steps the two levels the engine stores
 * at the start of an iteration (A_{k0-1} and U_{k0}) are rounded as the
 * engine's checkpoint format does (bits 8 / 11 / 24 with one scale per level,
 * -1 block floating point) and the segment's A_k recomputed from them. */
#include "awe_oracle_gpu.c"

double orc_quantize(double x, double scale, int bits);
void orc_quantize_bfp16(double *u, size_t n);

static void ckpt_round(double *u, size_t n, int bits) {
    if (bits < 0) {
        orc_quantize_bfp16(u, n);
        return;
    }
    double amax = 0;
    for (size_t i = 0; i < n; i++) amax = fabs(u[i]) > amax ? fabs(u[i]) : amax;
    for (size_t i = 0; i < n; i++) u[i] = orc_quantize(u[i], amax, bits);
}

typedef struct {
    int n1, n2, n3; /* padded r, theta, phi */
    size_t st, sp, np;
    double *A2, *Cr, *B, *D; /* 2/r, 1/r^2 per radius; cos/(r^2 sin), 1/(r^2 sin^2) per (theta, r) */
    double rdr, rdr2, rdth, rdth2, rdph2;
} sgrid;

static int s_interior(const sgrid *g, int ir, int ith, int iph) {
    return ir >= NOPA && ir < g->n1 - NOPA && ith >= NOPA && ith < g->n2 - NOPA && iph >= NOPA && iph < g->n3 - NOPA;
}

/* L u at an interior cell */
static double s_lap(const sgrid *g, const double *u, int ir, int ith, size_t c) {
    const size_t st = g->st, sp = g->sp;
    const size_t t = (size_t)ith * g->n1 + ir;
    const double pra = (u[c + 1] - u[c - 1]) * g->rdr;
    const double ppra = (u[c + 1] - 2 * u[c] + u[c - 1]) * g->rdr2;
    const double pth = (u[c + st] - u[c - st]) * g->rdth;
    const double ppth = (u[c + st] - 2 * u[c] + u[c - st]) * g->rdth2;
    const double ppph = (u[c + sp] - 2 * u[c] + u[c - sp]) * g->rdph2;
    return g->A2[ir] * pra + ppra + g->B[t] * pth + g->Cr[ir] * ppth + g->D[t] * ppph;
}

/* out += L^T y, by scattering each interior cell's stencil row */
static void s_lapT_add(const sgrid *g, const double *y, double *out) {
    const size_t st = g->st, sp = g->sp;
    for (int iph = NOPA; iph < g->n3 - NOPA; iph++)
        for (int ith = NOPA; ith < g->n2 - NOPA; ith++)
            for (int ir = NOPA; ir < g->n1 - NOPA; ir++) {
                const size_t c = (size_t)iph * sp + (size_t)ith * st + ir, t = (size_t)ith * g->n1 + ir;
                const double v = y[c];
                if (v == 0) continue;
                const double a = g->A2[ir] * g->rdr, b = g->B[t] * g->rdth, cr = g->Cr[ir] * g->rdth2,
                             d = g->D[t] * g->rdph2;
                out[c + 1] += v * (a + g->rdr2);
                out[c - 1] += v * (-a + g->rdr2);
                out[c] += v * (-2 * g->rdr2 - 2 * cr - 2 * d);
                out[c + st] += v * (b + cr);
                out[c - st] += v * (-b + cr);
                out[c + sp] += v * d;
                out[c - sp] += v * d;
            }
}

static int spher_impl(const orc_gpar *P, const float *vel_in, const double *m_in, const float *wav, int ns,
                      const float *sou, int nr, const float *rec, const float *dobs, int every, int bits,
                      double *grad, double *misfit, double *dsyn, int image) {
    const int nra = P->n1, nth = P->n2, nph = P->n3, nt = P->nt;
    const int nb = P->nb < NOPA ? NOPA : P->nb;
    sgrid g;
    g.n1 = nra + 2 * nb;
    g.n2 = nth + 2 * nb;
    g.n3 = nph + 2 * nb;
    g.st = g.n1;
    g.sp = (size_t)g.n1 * g.n2;
    g.np = g.sp * g.n3;
    const size_t np = g.np, st = g.st, sp = g.sp;
    const float orpad = P->o1 - nb * P->d1, othpad = P->o2 - nb * P->d2, ophpad = P->o3 - nb * P->d3;
    const double dra = P->d1, dth = P->d2, dph = P->d3, dt = P->dt;
    g.rdr = 1 / (2 * dra);
    g.rdr2 = 1 / (dra * dra);
    g.rdth = 1 / (2 * dth);
    g.rdth2 = 1 / (dth * dth);
    g.rdph2 = 1 / (dph * dph);
    g.A2 = malloc(g.n1 * sizeof(double));
    g.Cr = malloc(g.n1 * sizeof(double));
    g.B = malloc((size_t)g.n1 * g.n2 * sizeof(double));
    g.D = malloc((size_t)g.n1 * g.n2 * sizeof(double));
    for (int ir = 0; ir < g.n1; ir++) {
        const double ra = dra * ir + orpad;
        g.A2[ir] = 2 / ra;
        g.Cr[ir] = 1 / (ra * ra);
        for (int ith = 0; ith < g.n2; ith++) {
            const double th = dth * ith + othpad;
            g.B[(size_t)ith * g.n1 + ir] = cos(th) / (ra * ra * sin(th));
            g.D[(size_t)ith * g.n1 + ir] = 1 / (ra * ra * sin(th) * sin(th));
        }
    }
    /* model: c = dt^2 v^2 (float velocity, or m = 1/v^2 in double) */
    float *v = malloc(np * 4);
    double *c = malloc(np * sizeof(double));
    const int mn = nra * nth * nph;
    if (m_in) {
        float *vm = malloc((size_t)mn * 4);
        for (int i = 0; i < mn; i++) vm[i] = (float)(1 / sqrt(m_in[i]));
        pad_clamp(vm, v, nb, nra, nth, nph); /* for the reflectivity scale only */
        free(vm);
        for (int i3 = 0; i3 < g.n3; i3++)
            for (int i2 = 0; i2 < g.n2; i2++)
                for (int i1 = 0; i1 < g.n1; i1++) {
                    int j1 = i1 - nb, j2 = i2 - nb, j3 = i3 - nb;
                    j1 = j1 < 0 ? 0 : (j1 >= nra ? nra - 1 : j1);
                    j2 = j2 < 0 ? 0 : (j2 >= nth ? nth - 1 : j2);
                    j3 = j3 < 0 ? 0 : (j3 >= nph ? nph - 1 : j3);
                    c[(size_t)i3 * sp + (size_t)i2 * st + i1] = dt * dt / m_in[((size_t)j3 * nth + j2) * nra + j1];
                }
    } else {
        pad_clamp(vel_in, v, nb, nra, nth, nph);
        for (size_t i = 0; i < np; i++) c[i] = dt * dt * ((double)v[i] * v[i]);
    }
    /* sponge factor and free-surface mask per cell */
    double tab[4096];
    tab[0] = 1;
    for (int i = 1; i <= nb; i++) tab[i] = sponge_damp(i, nb);
    double *W = malloc(np * sizeof(double));
    unsigned char *M = malloc(np);
    const int spill = 8 * ((g.n1 + 7) / 8) - g.n1;
    for (int iph = 0; iph < g.n3; iph++)
        for (int ith = 0; ith < g.n2; ith++)
            for (int ir = 0; ir < g.n1; ir++) {
                const size_t i = (size_t)iph * sp + (size_t)ith * st + ir;
                W[i] = tab[sponge_i(ir, g.n1, iph, g.n3, ith, g.n2, nb)];
                const int line = iph * g.n2 + ith;
                M[i] = !(P->fsrf && (ir > g.n1 - nb || (ir < spill && line >= 1)));
            }
    glint *cs = malloc((ns ? ns : 1) * sizeof(glint)), *cr = malloc((nr ? nr : 1) * sizeof(glint));
    for (int i = 0; i < ns; i++)
        glint_make(3, sou[3 * i], sou[3 * i + 1], sou[3 * i + 2], othpad, orpad, ophpad, P->d2, P->d1, P->d3, g.n2,
                   g.n1, g.n3, &cs[i]);
    for (int i = 0; i < nr; i++)
        glint_make(3, rec[3 * i], rec[3 * i + 1], rec[3 * i + 2], othpad, orpad, ophpad, P->d2, P->d1, P->d3, g.n2,
                   g.n1, g.n3, &cr[i]);
    size_t off[8];
    for (int k = 0; k < 8; k++) off[k] = ((k & 1) ? st : 0) + ((k & 2) ? 1 : 0) + ((k & 4) ? sp : 0);
    double *sc = malloc((ns ? ns : 1) * sizeof(double));
    for (int s = 0; s < ns; s++) {
        const size_t b = (size_t)cs[s].jy * sp + (size_t)cs[s].jz * st + cs[s].jx;
        sc[s] = P->expl ? refl3(v, np, (long long)b, st, sp) : 1.0;
    }
#define RB(q) ((size_t)(q)->jy * sp + (size_t)(q)->jz * st + (q)->jx)

    /* forward: A[k] kept for k = 0..nt-1; U_{k0} kept at segment starts */
    const int T = every > 0 && bits != 0 ? every : nt;
    const int nseg = (nt + T - 1) / T;
    double *A = calloc((size_t)nt * np, sizeof(double)), *U = calloc(np, sizeof(double));
    double *Useg = calloc((size_t)nseg * np, sizeof(double)), *zero = calloc(np, sizeof(double));
    double *r = calloc((size_t)nt * (nr ? nr : 1), sizeof(double));
    /* one forward step from (Aprev, U) at iteration k: A_k -> Ak, U_{k+1} -> U */
    #define FSTEP(k, Aprev, Ak)                                                                          \
        do {                                                                                             \
            memcpy(Ak, U, np * sizeof(double));                                                          \
            for (int s = 0; s < ns; s++)                                                                 \
                for (int q = 0; q < 8; q++) Ak[RB(&cs[s]) + off[q]] += (double)wav[k] * cs[s].w[q] * sc[s]; \
            for (int iph = 0; iph < g.n3; iph++)                                                         \
                for (int ith = 0; ith < g.n2; ith++)                                                     \
                    for (int ir = 0; ir < g.n1; ir++) {                                                  \
                        const size_t i = (size_t)iph * sp + (size_t)ith * st + ir;                      \
                        const double lap = s_interior(&g, ir, ith, iph) ? s_lap(&g, Ak, ir, ith, i) : 0; \
                        U[i] = M[i] ? W[i] * (c[i] * lap + 2 * Ak[i] - W[i] * (Aprev)[i]) : 0;            \
                    }                                                                                    \
        } while (0)
    for (int k = 0; k < nt; k++) {
        if (k % T == 0) memcpy(Useg + (size_t)(k / T) * np, U, np * sizeof(double));
        double *Ak = A + (size_t)k * np;
        FSTEP(k, k > 0 ? A + (size_t)(k - 1) * np : zero, Ak);
        for (int ir = 0; ir < nr; ir++) {
            double acc = 0;
            for (int q = 0; q < 8; q++) acc += U[RB(&cr[ir]) + off[q]] * cr[ir].w[q];
            const size_t row = (size_t)k * nr + ir;
            if (dsyn) dsyn[row] = acc;
            r[row] = image < 0 ? acc - dobs[row] : (double)dobs[row]; /* an image back-propagates the data */
        }
    }
    double J = 0;
    for (size_t i = 0; i < (size_t)nt * nr; i++) J += 0.5 * r[i] * r[i];
    *misfit = J;
    /* checkpointed recompute, last segment first (each restart reads exact levels) */
    if (every > 0 && bits != 0) {
        double *prev = malloc(np * sizeof(double));
        for (int seg = nseg - 1; seg >= 0; seg--) {
            const int k0 = seg * T, k1 = k0 + T < nt ? k0 + T : nt;
            if (k0 > 0) memcpy(prev, A + (size_t)(k0 - 1) * np, np * sizeof(double));
            else memset(prev, 0, np * sizeof(double));
            memcpy(U, Useg + (size_t)seg * np, np * sizeof(double));
            ckpt_round(prev, np, bits);
            ckpt_round(U, np, bits);
            for (int k = k0; k < k1; k++) {
                double *Ak = A + (size_t)k * np;
                FSTEP(k, k > k0 ? A + (size_t)(k - 1) * np : prev, Ak);
            }
        }
        free(prev);
    }
#undef FSTEP

    /* adjoint */
    double *zx = calloc(np, sizeof(double)), *zy = calloc(np, sizeof(double)), *zn = malloc(np * sizeof(double));
    double *y = malloc(np * sizeof(double)), *G = calloc(np, sizeof(double));
    for (int j = nt; j >= 0; j--) {
        /* zx = z_{j+1}, zy = z_{j+2} */
        if (j < nt) {
            const double *Aj = A + (size_t)j * np;
            for (int iph = NOPA; iph < g.n3 - NOPA; iph++)
                for (int ith = NOPA; ith < g.n2 - NOPA; ith++)
                    for (int ir = NOPA; ir < g.n1 - NOPA; ir++) {
                        const size_t i = (size_t)iph * sp + (size_t)ith * st + ir;
                        G[i] += zx[i] * (image == 0 ? Aj[i] : s_lap(&g, Aj, ir, ith, i));
                    }
        }
        if (j == 0) break;
        for (size_t i = 0; i < np; i++) y[i] = c[i] * zx[i];
        for (size_t i = 0; i < np; i++) zn[i] = 2 * zx[i] - W[i] * zy[i];
        s_lapT_add(&g, y, zn);
        for (int ir = 0; ir < nr; ir++)
            for (int q = 0; q < 8; q++) zn[RB(&cr[ir]) + off[q]] += cr[ir].w[q] * r[(size_t)(j - 1) * nr + ir];
        for (size_t i = 0; i < np; i++) zn[i] = M[i] ? W[i] * zn[i] : 0;
        double *t = zy;
        zy = zx;
        zx = zn;
        zn = t;
    }
#undef RB
    memset(grad, 0, (size_t)mn * sizeof(double));
    for (int iph = 0; iph < g.n3 && image == 0; iph++) /* cross-correlation image: the model window */
        for (int ith = 0; ith < g.n2; ith++)
            for (int ir = 0; ir < g.n1; ir++) {
                const int j1 = ir - nb, j2 = ith - nb, j3 = iph - nb;
                if (j1 >= 0 && j1 < nra && j2 >= 0 && j2 < nth && j3 >= 0 && j3 < nph)
                    grad[((size_t)j3 * nth + j2) * nra + j1] = G[(size_t)iph * sp + (size_t)ith * st + ir];
            }
    for (int iph = 0; iph < g.n3 && image != 0; iph++)
        for (int ith = 0; ith < g.n2; ith++)
            for (int ir = 0; ir < g.n1; ir++) {
                const size_t i = (size_t)iph * sp + (size_t)ith * st + ir;
                int j1 = ir - nb, j2 = ith - nb, j3 = iph - nb;
                j1 = j1 < 0 ? 0 : (j1 >= nra ? nra - 1 : j1);
                j2 = j2 < 0 ? 0 : (j2 >= nth ? nth - 1 : j2);
                j3 = j3 < 0 ? 0 : (j3 >= nph ? nph - 1 : j3);
                grad[((size_t)j3 * nth + j2) * nra + j1] += G[i] * (-c[i] * c[i] / (dt * dt));
            }
    free(g.A2);
    free(g.Cr);
    free(g.B);
    free(g.D);
    free(v);
    free(c);
    free(W);
    free(M);
    free(cs);
    free(cr);
    free(sc);
    free(A);
    free(U);
    free(Useg);
    free(zero);
    free(r);
    free(zx);
    free(zy);
    free(zn);
    free(y);
    free(G);
    return 0;
}

int orc_gpu_spher3d_grad(const orc_gpar *P, const float *vel_in, const double *m_in, const float *wav, int ns,
                         const float *sou, int nr, const float *rec, const float *dobs, int every, int bits,
                         double *grad, double *misfit, double *dsyn) {
    return spher_impl(P, vel_in, m_in, wav, ns, sou, nr, rec, dobs, every, bits, grad, misfit, dsyn, -1);
}

/* images of the recorded data `data` (condition 0 cross-correlation, 1 Born) */
int orc_gpu_spher3d_image(const orc_gpar *P, const float *vel_in, const float *wav, int ns, const float *sou, int nr,
                          const float *rec, const float *data, int condition, double *image) {
    double unused = 0;
    return spher_impl(P, vel_in, NULL, wav, ns, sou, nr, rec, data, 0, 0, image, &unused, NULL, condition);
}
