/* CPU oracle: restatement of the reference's CPU acoustic programs.
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE (see awe_oracle.h).
 *
 * File/line citations are to Nacnud04/wavefield_imaging, CODE/.  Arrays are
 * flat: 2D u[ix*n1pad + iz], 3D u[(iy*n2pad + ix)*n1pad + iz] (axis 1 = z
 * fastest), the same element order as the reference's float** / float***
 * (sf_floatalloc2(nzpad,nxpad), sf_floatalloc3(nzpad,nxpad,nypad)). */
#include "awe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef AWE_REAL_DOUBLE
typedef double real;
#else
typedef float real;
#endif

#define SPI 3.14159265358979323846264338328 /* SF_PI */

/* ------------------------------------------------------------------ */
/* finite-difference coefficients: MAWEFDcart2Dcpu.c:423-551,
 * MAWEFDcart3Dcpu.c:404-531 (identical but for ndim) */
static int fact(int n) {
    int r = 1;
    for (int i = 1; i <= n; ++i) r *= i;
    return r;
}

/* normal_fdcoef, MAWEFDcart2Dcpu.c:486-500 */
static void normal_cc(int nop, float *cc, float *bb) {
    int half = fact(nop);
    half *= half;
    cc[0] = 0.f;
    bb[0] = 0.f;
    for (int n = 1; n <= nop; n++) {
        cc[n] = -2.f / (n * n) * cos(n * SPI) * half / fact(nop + n) / fact(nop - n);
        bb[n] = cc[n] * n / 2.f;
    }
}

/* optimal_fdcoef tables, MAWEFDcart2Dcpu.c:502-551 (published LS-optimal
 * coefficients: Liu 2013 for d2, Zhang & Yao 2013 for d1) */
static const float OPT_C[11][11] = {
    {0},
    {0.f, 1.f},
    {0.f, 1.369074f, -0.09266816},
    {0.f, 1.573661f, -0.1820268f, 0.01728053f},
    {0.f, 1.700010f, -0.2554615f, 0.04445392f, -0.004946851f},
    {0.f, 1.782836f, -0.3124513f, 0.07379487f, -0.01532122f, 0.001954439f},
    {0.f, 1.837023f, -0.3538895f, 0.09978343f, -0.02815486f, 0.006556587f, -0.0009405699f},
    {0.f, 1.874503f, -0.3845794f, 0.1215162f, -0.04121749f, 0.01295522f, -0.003313813f, 0.0005310053f},
    {0.f, 1.901160f, -0.4074304f, 0.1390909f, -0.05318775f, 0.02004823f, -0.006828249f, 0.001895771f,
     -0.0003369052f},
    {0.f, 1.919909f, -0.4240446f, 0.1526043f, -0.06322328f, 0.02676005f, -0.01080739f, 0.003907747f,
     -0.001158024f, 0.0002240247f},
    {0.f, 1.918204f, -0.4225858f, 0.1514992f, -0.06249474f, 0.02637196f, -0.01066631f, 0.003915625f,
     -0.001219872f, 0.0002863976f, -0.00003744830f}};
static const float OPT_B[7][7] = {{0},
                                  {0.0f, 0.5f},
                                  {0.0f, 0.67880327, -0.08962729},
                                  {0.0f, 0.77793115, -0.17388691, 0.02338713},
                                  {0.0f, 0.84149635, -0.24532989, 0.06081891, -0.00839807},
                                  {0.0f, 0.88414717, -0.30233648, 0.10275057, -0.02681517, 0.00398089},
                                  {0.0f, 0.91067892, -0.34187892, 0.13833962, -0.04880710, 0.01302148,
                                   -0.00199047}};

/* compute_fdcoef: d2[0] = -2 * sum of all d2 terms; d2[idim*nop+ii] =
 * c[ii]/d^2; d1[idim*nop+ii] = b[ii]/d.  dd[] = spacing per axis (z, x, y). */
static void fdcoef(int nop, int ndim, const float *dd, int optfd, float *d2, float *d1) {
    float cc[16], bb[16];
    normal_cc(nop, cc, bb);
    const float *c2 = optfd ? OPT_C[nop] : cc;
    const float *c1 = (optfd && nop <= 6) ? OPT_B[nop] : bb;
    d2[0] = 0.f;
    for (int idim = 0; idim < ndim; idim++) {
        float dsq = dd[idim] * dd[idim];
        for (int ii = 1; ii <= nop; ii++) {
            d2[idim * nop + ii] = c2[ii] / dsq;
            d2[0] += d2[idim * nop + ii];
        }
    }
    d2[0] *= -2.0f;
    d1[0] = 0.0f;
    for (int idim = 0; idim < ndim; idim++)
        for (int ii = 1; ii <= nop; ii++) d1[idim * nop + ii] = c1[ii] / dd[idim];
}

/* sponge_make, fdutil.c:2181-2200 */
static void sponge_w(int nb, float *w) {
    float sb = 4.0 * nb;
    for (int ib = 0; ib < nb; ib++) {
        float fb = ib / (sqrt(2.0) * sb);
        w[ib] = exp(-fb * fb);
    }
}

/* damp_make, MAWEFDcart2Dcpu.c:407-421 */
static void damp_w(int ntransit, float *w) {
    float sb = 4.0 * ntransit;
    for (int ib = 0; ib < ntransit; ib++) {
        float fb = ib / (sqrt(2.0) * sb);
        w[ib] = exp(-fb * fb);
    }
}

/* ------------------------------------------------------------------ */
/* geometry: lint2d_make fdutil.c:1363-1404, lint3d_make fdutil.c:1474-1539 */
typedef struct {
    int jz, jx, jy;
    float w[8]; /* 2D: w00 w01 w10 w11; 3D: w000 w001 w010 w011 w100 w101 w110 w111 */
} lint;

static void lint2d(float x, float z, float oz, float ox, float dz, float dx, int nzpad, int nxpad, lint *c) {
    float f1, f2;
    if (z >= oz && z < oz + (nzpad - 1) * dz && x >= ox && x < ox + (nxpad - 1) * dx) {
        c->jz = (int)((z - oz) / dz);
        c->jx = (int)((x - ox) / dx);
        f1 = (z - oz) / dz - c->jz;
        f2 = (x - ox) / dx - c->jx;
    } else {
        c->jz = 0;
        c->jx = 0;
        f1 = 1;
        f2 = 0;
    }
    c->jy = 0;
    c->w[0] = (1 - f1) * (1 - f2);
    c->w[1] = (f1) * (1 - f2);
    c->w[2] = (1 - f1) * (f2);
    c->w[3] = (f1) * (f2);
}

static void lint3d(float x, float y, float z, float oz, float ox, float oy, float dz, float dx, float dy, int nzpad,
                   int nxpad, int nypad, lint *c) {
    float f1, f2, f3;
    if (z >= oz && z < oz + (nzpad - 1) * dz && x >= ox && x < ox + (nxpad - 1) * dx && y >= oy &&
        y < oy + (nypad - 1) * dy) {
        c->jz = (int)((z - oz) / dz);
        c->jx = (int)((x - ox) / dx);
        c->jy = (int)((y - oy) / dy);
        f1 = (z - oz) / dz - c->jz;
        f2 = (x - ox) / dx - c->jx;
        f3 = (y - oy) / dy - c->jy;
    } else {
        c->jz = 0;
        c->jx = 0;
        c->jy = 0;
        f1 = 1;
        f2 = 0;
        f3 = 0;
    }
    c->w[0] = (1 - f3) * (1 - f1) * (1 - f2);
    c->w[1] = (1 - f3) * (f1) * (1 - f2);
    c->w[2] = (1 - f3) * (1 - f1) * (f2);
    c->w[3] = (1 - f3) * (f1) * (f2);
    c->w[4] = (f3) * (1 - f1) * (1 - f2);
    c->w[5] = (f3) * (f1) * (1 - f2);
    c->w[6] = (f3) * (1 - f1) * (f2);
    c->w[7] = (f3) * (f1) * (f2);
}

/* ------------------------------------------------------------------ */
/* padding: expand2d fdutil.c:435-458, expand3d fdutil.c:528-571 */
static void expand2(const float *a, float *b, int nb, int n1, int n2) {
    int n1p = n1 + 2 * nb, n2p = n2 + 2 * nb;
    for (int ix = 0; ix < n2; ix++)
        for (int iz = 0; iz < n1; iz++) b[(size_t)(nb + ix) * n1p + nb + iz] = a[(size_t)ix * n1 + iz];
    for (int ix = 0; ix < n2p; ix++)
        for (int iz = 0; iz < nb; iz++) {
            b[(size_t)ix * n1p + iz] = b[(size_t)ix * n1p + nb];
            b[(size_t)ix * n1p + n1p - iz - 1] = b[(size_t)ix * n1p + n1p - nb - 1];
        }
    for (int ix = 0; ix < nb; ix++)
        for (int iz = 0; iz < n1p; iz++) {
            b[(size_t)ix * n1p + iz] = b[(size_t)nb * n1p + iz];
            b[(size_t)(n2p - ix - 1) * n1p + iz] = b[(size_t)(n2p - nb - 1) * n1p + iz];
        }
}

static void expand3(const float *a, float *b, int nb, int n1, int n2, int n3) {
    size_t n1p = n1 + 2 * nb, n2p = n2 + 2 * nb, n3p = n3 + 2 * nb;
#define B3(iy, ix, iz) b[((size_t)(iy) * n2p + (ix)) * n1p + (iz)]
    for (int iy = 0; iy < n3; iy++)
        for (int ix = 0; ix < n2; ix++)
            for (int iz = 0; iz < n1; iz++) B3(nb + iy, nb + ix, nb + iz) = a[((size_t)iy * n2 + ix) * n1 + iz];
    for (size_t iy = 0; iy < n3p; iy++)
        for (size_t ix = 0; ix < n2p; ix++)
            for (int iz = 0; iz < nb; iz++) {
                B3(iy, ix, iz) = B3(iy, ix, nb);
                B3(iy, ix, n1p - iz - 1) = B3(iy, ix, n1p - nb - 1);
            }
    for (size_t iy = 0; iy < n3p; iy++)
        for (int ix = 0; ix < nb; ix++)
            for (size_t iz = 0; iz < n1p; iz++) {
                B3(iy, ix, iz) = B3(iy, nb, iz);
                B3(iy, n2p - ix - 1, iz) = B3(iy, n2p - nb - 1, iz);
            }
    for (int iy = 0; iy < nb; iy++)
        for (size_t ix = 0; ix < n2p; ix++)
            for (size_t iz = 0; iz < n1p; iz++) {
                B3(iy, ix, iz) = B3(nb, ix, iz);
                B3(n3p - iy - 1, ix, iz) = B3(n3p - nb - 1, ix, iz);
            }
#undef B3
}

int orc_cart_padded(const orc_par *p, int *nbd, int *n1pad, int *n2pad, int *n3pad) {
    int nop = p->fdorder / 2;
    int nb = p->nb;
    if (nb < nop) nb = nop; /* MAWEFDcart2Dcpu.c:211 */
    if (p->dabc && p->hybrid && nb <= nop) nb = 2 * nop; /* :212 */
    *nbd = nb;
    *n1pad = p->n1 + 2 * nb;
    *n2pad = p->n2 + 2 * nb;
    *n3pad = (p->n3 > 1) ? p->n3 + 2 * nb : 1;
    return 0;
}

/* ------------------------------------------------------------------ */
/* 2D cartesian, CODE/MAWEFDcart2Dcpu.c:107-404 */

/* step_forward_2d scalar path, ts_kernel.c:49-161 (u0 <- new field) */
static void step2d(real *u0, const real *u1, const float *vel, const float *rho, const float *d2, const float *d1,
                   int nop, int nzpad, int nxpad) {
    const float c0 = d2[0];
    const float *cz = &d2[0], *cx = &d2[nop];
    const float *bz = &d1[0], *bx = &d1[nop];
#pragma omp parallel for schedule(static, 1)
    for (int ix = nop; ix < nxpad - nop; ix++) {
        for (int iz = nop; iz < nzpad - nop; iz++) {
            size_t i = (size_t)ix * nzpad + iz;
            real lap = u1[i] * c0;
            for (int iop = 1; iop <= nop; iop++) {
                lap += (u1[i - iop] + u1[i + iop]) * cz[iop] +
                       (u1[i - (size_t)iop * nzpad] + u1[i + (size_t)iop * nzpad]) * cx[iop];
            }
            if (rho) {
                real du_z = 0.f, du_x = 0.f, dr_z = 0.f, dr_x = 0.f;
                for (int iop = 1; iop <= nop; iop++) {
                    du_z += (u1[i + iop] - u1[i - iop]) * bz[iop];
                    du_x += (u1[i + (size_t)iop * nzpad] - u1[i - (size_t)iop * nzpad]) * bx[iop];
                    dr_z += (rho[i + iop] - rho[i - iop]) * bz[iop];
                    dr_x += (rho[i + (size_t)iop * nzpad] - rho[i - (size_t)iop * nzpad]) * bx[iop];
                }
                lap -= (du_z * dr_z + du_x * dr_x) / rho[i];
            }
            u0[i] = (real)(2. * (double)u1[i] - (double)u0[i] + (double)(vel[i] * lap));
        }
    }
}

/* sponge2d_apply, fdutil.c:2206-2245 */
static void sponge2(real *u, const float *w, int nb, int nzpad, int nxpad) {
    for (int ib = 0; ib < nb; ib++) {
        float wb = w[nb - ib - 1];
        int ibz = nzpad - ib - 1;
        for (int ix = 0; ix < nxpad; ix++) {
            u[(size_t)ix * nzpad + ib] *= wb;
            u[(size_t)ix * nzpad + ibz] *= wb;
        }
    }
    for (int ib = 0; ib < nb; ib++) {
        float wb = w[nb - ib - 1];
        int ibx = nxpad - ib - 1;
        for (int iz = 0; iz < nzpad; iz++) {
            u[(size_t)ib * nzpad + iz] *= wb;
            u[(size_t)ibx * nzpad + iz] *= wb;
        }
    }
}

/* hybrid one-way ABC, apply_abc MAWEFDcart2Dcpu.c:553-614 */
static void hybrid2(real *u2, const real *u1, int nzpad, int nxpad, int nbd, const float *bzl, const float *bzh,
                    const float *bxl, const float *bxh, int nop, const float *damp, int fsrf) {
#define U(a, ix, iz) a[(size_t)(ix) * nzpad + (iz)]
    for (int ix = 0; ix < nxpad; ix++) {
        for (int ib = nbd - nop; ib < nbd; ib++) {
            int iz = nbd - ib - 1;
            U(u2, ix, iz) = U(u1, ix, iz + 1) + (U(u1, ix, iz) - U(u2, ix, iz + 1)) * bzl[ix];
            iz = nzpad - nbd + ib;
            U(u2, ix, iz) = U(u1, ix, iz - 1) + (U(u1, ix, iz) - U(u2, ix, iz - 1)) * bzh[ix];
        }
        if (damp) {
            for (int ib = 0; ib < nbd - nop; ib++) {
                float dib = damp[ib];
                int iz = nbd - ib - 1;
                real bc = U(u1, ix, iz + 1) + (U(u1, ix, iz) - U(u2, ix, iz + 1)) * bzl[ix];
                U(u2, ix, iz) = bc * (1.f - dib) + U(u2, ix, iz) * dib;
                iz = nzpad - nbd + ib;
                bc = U(u1, ix, iz - 1) + (U(u1, ix, iz) - U(u2, ix, iz - 1)) * bzh[ix];
                U(u2, ix, iz) = bc * (1.f - dib) + U(u2, ix, iz) * dib;
            }
        }
        if (fsrf)
            for (int iz = 0; iz < nbd + 1; iz++) U(u2, ix, iz) = 0;
    }
    for (int iz = 0; iz < nzpad; iz++) {
        for (int ib = nbd - nop; ib < nbd; ib++) {
            int ix = nbd - ib - 1;
            U(u2, ix, iz) = U(u1, ix + 1, iz) + (U(u1, ix, iz) - U(u2, ix + 1, iz)) * bxl[iz];
            ix = nxpad - nbd + ib;
            U(u2, ix, iz) = U(u1, ix - 1, iz) + (U(u1, ix, iz) - U(u2, ix - 1, iz)) * bxh[iz];
        }
        if (damp) {
            for (int ib = 0; ib < nbd - nop; ib++) {
                float dib = damp[ib];
                int ix = nbd - ib - 1;
                real bc = U(u1, ix + 1, iz) + (U(u1, ix, iz) - U(u2, ix + 1, iz)) * bxl[iz];
                U(u2, ix, iz) = bc * (1.f - dib) + U(u2, ix, iz) * dib;
                ix = nxpad - nbd + ib;
                bc = U(u1, ix - 1, iz) + (U(u1, ix, iz) - U(u2, ix - 1, iz)) * bxh[iz];
                U(u2, ix, iz) = bc * (1.f - dib) + U(u2, ix, iz) * dib;
            }
        }
    }
#undef U
}

/* cut2d, fdutil.c:574-604, for the default window (the unpadded model) */
static int cut_first(float o, float opad, float d) { return (int)(floor)((o - opad) / d); }

int orc_cart2d_cpu(const orc_par *p, const float *vel_in, const float *den_in, const float *wav, int ns,
                   const float *sou, int nr, const float *rec, float *dat, float *snaps) {
#ifdef _OPENMP
    if (p->nthreads > 0) omp_set_num_threads(p->nthreads);
#endif
    int nop = p->fdorder / 2, nbd, nzpad, nxpad, n3pad;
    if (nop < 1 || nop > 10) return 1;
    orc_cart_padded(p, &nbd, &nzpad, &nxpad, &n3pad);
    const int nz = p->n1, nx = p->n2;
    const float dz = p->d1, dx = p->d2, dt = p->dt;
    /* fdutil_init, fdutil.c:264-297 */
    const float ozpad = p->o1 - nbd * dz, oxpad = p->o2 - nbd * dx;
    float d2[64], d1[64], dd[2] = {dz, dx};
    fdcoef(nop, 2, dd, p->optfd, d2, d1);

    size_t npad = (size_t)nzpad * nxpad;
    float *vel = malloc(npad * sizeof(float));
    float *rho = den_in ? malloc(npad * sizeof(float)) : NULL;
    real *u0 = calloc(npad, sizeof(real)), *u1 = calloc(npad, sizeof(real));
    expand2(vel_in, vel, nbd, nz, nx);
    if (rho) expand2(den_in, rho, nbd, nz, nx);

    lint *cs = malloc((ns > 0 ? ns : 1) * sizeof(lint)), *cr = malloc((nr > 0 ? nr : 1) * sizeof(lint));
    for (int i = 0; i < ns; i++) lint2d(sou[2 * i], sou[2 * i + 1], ozpad, oxpad, dz, dx, nzpad, nxpad, &cs[i]);
    for (int i = 0; i < nr; i++) lint2d(rec[2 * i], rec[2 * i + 1], ozpad, oxpad, dz, dx, nzpad, nxpad, &cr[i]);

    /* abcone2d_make(nbd,...) fdutil.c:1919-1957 with raw velocity */
    float *bzl = malloc(nxpad * sizeof(float)), *bzh = malloc(nxpad * sizeof(float));
    float *bxl = malloc(nzpad * sizeof(float)), *bxh = malloc(nzpad * sizeof(float));
    float spo[4096], damp[4096];
    int have_damp = 0;
    if (p->dabc) {
        for (int ix = 0; ix < nxpad; ix++) {
            float d = vel[(size_t)ix * nzpad + nbd] * dt / dz;
            bzl[ix] = (1 - d) / (1 + d);
            d = vel[(size_t)ix * nzpad + nzpad - nbd - 1] * dt / dz;
            bzh[ix] = (1 - d) / (1 + d);
        }
        for (int iz = 0; iz < nzpad; iz++) {
            float d = vel[(size_t)nbd * nzpad + iz] * dt / dx;
            bxl[iz] = (1 - d) / (1 + d);
            d = vel[(size_t)(nxpad - nbd - 1) * nzpad + iz] * dt / dx;
            bxh[iz] = (1 - d) / (1 + d);
        }
        if (p->hybrid) {
            if (nbd - nop > 0) {
                damp_w(nbd - nop, damp);
                have_damp = 1;
            }
        } else
            sponge_w(nbd, spo);
    }
    /* v <- v^2 dt^2, free surface zeroes the top nb+1 samples (:290-295) */
    const float dt2 = dt * dt;
    for (size_t i = 0; i < npad; i++) vel[i] *= vel[i] * dt2;
    if (p->fsrf && !p->hybrid)
        for (int ix = 0; ix < nxpad; ix++)
            for (int iz = 0; iz < nbd + 1; iz++) vel[(size_t)ix * nzpad + iz] = 0;

    const int fz = cut_first(p->o1, ozpad, dz), fx = cut_first(p->o2, oxpad, dx);
    const int jz = (int)floor(dz / dz), jx = (int)floor(dx / dx);
    size_t snapsz = p->bnds ? npad : (size_t)nz * nx, isnap = 0;

    for (int it = 0; it < p->nt; it++) {
        step2d(u0, u1, vel, rho, d2, d1, nop, nzpad, nxpad);
        /* lint2d_inject1_with_vv / lint2d_inject_with_vv, fdutil.c:1688-1700, :1590-1600 */
        for (int s = 0; s < ns; s++) {
            float dd = p->expl ? wav[it] : wav[(size_t)it * ns + s];
            const lint *c = &cs[s];
            size_t i00 = (size_t)c->jx * nzpad + c->jz;
            u0[i00] += dd * c->w[0] * vel[i00];
            u0[i00 + 1] += dd * c->w[1] * vel[i00 + 1];
            u0[i00 + nzpad] += dd * c->w[2] * vel[i00 + nzpad];
            u0[i00 + nzpad + 1] += dd * c->w[3] * vel[i00 + nzpad + 1];
        }
        if (p->dabc) {
            if (p->hybrid)
                hybrid2(u0, u1, nzpad, nxpad, nbd, bzl, bzh, bxl, bxh, nop, have_damp ? damp : NULL, p->fsrf);
            else {
                sponge2(u0, spo, nbd, nzpad, nxpad);
                sponge2(u1, spo, nbd, nzpad, nxpad);
            }
        }
        real *t = u0;
        u0 = u1;
        u1 = t;
        if (snaps && p->jsnap > 0 && it % p->jsnap == 0) {
            float *dst = snaps + isnap * snapsz;
            if (p->bnds)
                for (size_t i = 0; i < npad; i++) dst[i] = (float)u0[i];
            else
                for (int ix = 0; ix < nx; ix++)
                    for (int iz = 0; iz < nz; iz++)
                        dst[(size_t)ix * nz + iz] = (float)u0[(size_t)(fx + ix * jx) * nzpad + fz + iz * jz];
            isnap++;
        }
        /* lint2d_extract, fdutil.c:1596-1610 */
        for (int r = 0; r < nr; r++) {
            const lint *c = &cr[r];
            size_t i00 = (size_t)c->jx * nzpad + c->jz;
            dat[(size_t)it * nr + r] = (float)(u0[i00] * c->w[0] + u0[i00 + 1] * c->w[1] +
                                               u0[i00 + nzpad] * c->w[2] + u0[i00 + nzpad + 1] * c->w[3]);
        }
    }
    free(vel);
    free(rho);
    free(u0);
    free(u1);
    free(cs);
    free(cr);
    free(bzl);
    free(bzh);
    free(bxl);
    free(bxh);
    return 0;
}

/* ------------------------------------------------------------------ */
/* 3D cartesian, CODE/MAWEFDcart3Dcpu.c:40-387 */

/* step_forward_3d scalar path, ts_kernel.c:163-314 */
static void step3d(real *u0, const real *u1, const float *vel, const float *rho, const float *d2, const float *d1,
                   int nop, int nzpad, int nxpad, int nypad) {
    const float c0 = d2[0];
    const float *cz = &d2[0], *cx = &d2[nop], *cy = &d2[2 * nop];
    const float *bz = &d1[0], *bx = &d1[nop], *by = &d1[2 * nop];
    const size_t sx = nzpad, sy = (size_t)nzpad * nxpad;
#pragma omp parallel for schedule(static, 1)
    for (int iy = nop; iy < nypad - nop; iy++) {
        for (int ix = nop; ix < nxpad - nop; ix++) {
            for (int iz = nop; iz < nzpad - nop; iz++) {
                size_t i = iy * sy + ix * sx + iz;
                real lap = u1[i] * c0;
                for (int iop = 1; iop <= nop; iop++) {
                    lap += (u1[i - iop] + u1[i + iop]) * cz[iop] + (u1[i - iop * sx] + u1[i + iop * sx]) * cx[iop] +
                           (u1[i - iop * sy] + u1[i + iop * sy]) * cy[iop];
                }
                if (rho) {
                    real du_z = 0.f, du_x = 0.f, du_y = 0.f, dr_z = 0.f, dr_x = 0.f, dr_y = 0.f;
                    for (int iop = 1; iop <= nop; iop++) {
                        du_z += (u1[i + iop] - u1[i - iop]) * bz[iop];
                        du_x += (u1[i + iop * sx] - u1[i - iop * sx]) * bx[iop];
                        du_y += (u1[i + iop * sy] - u1[i - iop * sy]) * by[iop];
                        dr_z += (rho[i + iop] - rho[i - iop]) * bz[iop];
                        dr_x += (rho[i + iop * sx] - rho[i - iop * sx]) * bx[iop];
                        dr_y += (rho[i + iop * sy] - rho[i - iop * sy]) * by[iop];
                    }
                    lap -= (du_z * dr_z + du_x * dr_x + du_y * dr_y) / rho[i];
                }
                u0[i] = (real)(2. * (double)u1[i] - (double)u0[i] + (double)(vel[i] * lap));
            }
        }
    }
}

/* sponge3d_apply, fdutil.c:2248-2310.  Each face pass is split over the
 * lines of another axis; every cell belongs to one line, which runs its ib
 * loop in the reference's order, so the products are those of the serial
 * loops. */
static void sponge3(real *u, const float *w, int nb, int nzpad, int nxpad, int nypad) {
    const size_t sx = nzpad, sy = (size_t)nzpad * nxpad;
#pragma omp parallel for
    for (int iy = 0; iy < nypad; iy++)
        for (int ib = 0; ib < nb; ib++) {
            float wb = w[nb - ib - 1];
            int ibz = nzpad - ib - 1;
            for (int ix = 0; ix < nxpad; ix++) {
                u[iy * sy + ix * sx + ib] *= wb;
                u[iy * sy + ix * sx + ibz] *= wb;
            }
        }
#pragma omp parallel for
    for (int iy = 0; iy < nypad; iy++)
        for (int ib = 0; ib < nb; ib++) {
            float wb = w[nb - ib - 1];
            int ibx = nxpad - ib - 1;
            for (int iz = 0; iz < nzpad; iz++) {
                u[iy * sy + ib * sx + iz] *= wb;
                u[iy * sy + ibx * sx + iz] *= wb;
            }
        }
#pragma omp parallel for
    for (int ix = 0; ix < nxpad; ix++)
        for (int ib = 0; ib < nb; ib++) {
            float wb = w[nb - ib - 1];
            int iby = nypad - ib - 1;
            for (int iz = 0; iz < nzpad; iz++) {
                u[ib * sy + ix * sx + iz] *= wb;
                u[iby * sy + ix * sx + iz] *= wb;
            }
        }
}

typedef struct {
    float *zl, *zh; /* [nypad][nxpad] */
    float *xl, *xh; /* [nypad][nzpad] */
    float *yl, *yh; /* [nxpad][nzpad] */
} abc3;

/* abcone3d_apply, fdutil.c:2085-2177 (uo = new field, um = current).  Each
 * pass is split over lines that its recurrences never cross (the z pass over
 * y, the x pass over y, the y pass over x), so the result is the serial one. */
static void abcone3(real *uo, const real *um, int nop, const abc3 *a, int fsrf, int nzpad, int nxpad, int nypad) {
    const size_t sx = nzpad, sy = (size_t)nzpad * nxpad;
#pragma omp parallel for
    for (int iy = 0; iy < nypad; iy++)
        for (int ix = 0; ix < nxpad; ix++)
            for (int iop = 0; iop < nop; iop++) {
                size_t c = iy * sy + ix * sx;
                float bl = a->zl[(size_t)iy * nxpad + ix], bh = a->zh[(size_t)iy * nxpad + ix];
                if (!fsrf) {
                    int iz = nop - iop;
                    uo[c + iz] = um[c + iz + 1] + (um[c + iz] - uo[c + iz + 1]) * bl;
                }
                int iz = nzpad - nop + iop - 1;
                uo[c + iz] = um[c + iz - 1] + (um[c + iz] - uo[c + iz - 1]) * bh;
            }
#pragma omp parallel for
    for (int iy = 0; iy < nypad; iy++)
        for (int iz = 0; iz < nzpad; iz++)
            for (int iop = 0; iop < nop; iop++) {
                float bl = a->xl[(size_t)iy * nzpad + iz], bh = a->xh[(size_t)iy * nzpad + iz];
                int ix = nop - iop;
                size_t c = iy * sy + ix * sx + iz;
                uo[c] = um[c + sx] + (um[c] - uo[c + sx]) * bl;
                ix = nxpad - nop + iop - 1;
                c = iy * sy + ix * sx + iz;
                uo[c] = um[c - sx] + (um[c] - uo[c - sx]) * bh;
            }
#pragma omp parallel for
    for (int ix = 0; ix < nxpad; ix++)
        for (int iz = 0; iz < nzpad; iz++)
            for (int iop = 0; iop < nop; iop++) {
                float bl = a->yl[(size_t)ix * nzpad + iz], bh = a->yh[(size_t)ix * nzpad + iz];
                int iy = nop - iop;
                size_t c = iy * sy + ix * sx + iz;
                uo[c] = um[c + sy] + (um[c] - uo[c + sy]) * bl;
                iy = nypad - nop + iop - 1;
                c = iy * sy + ix * sx + iz;
                uo[c] = um[c - sy] + (um[c] - uo[c - sy]) * bh;
            }
}

/* hybrid ABC, apply_abc MAWEFDcart3Dcpu.c:533-625 */
static void hybrid3(real *u2, const real *u1, int nzpad, int nxpad, int nypad, int nbd, const abc3 *a, int nop,
                    const float *damp, int fsrf) {
    const size_t sx = nzpad, sy = (size_t)nzpad * nxpad;
#define U(arr, iy, ix, iz) arr[(size_t)(iy) * sy + (size_t)(ix) * sx + (iz)]
    for (int iy = 0; iy < nypad; iy++)
        for (int ix = 0; ix < nxpad; ix++) {
            float bl = a->zl[(size_t)iy * nxpad + ix], bh = a->zh[(size_t)iy * nxpad + ix];
            for (int ib = nbd - nop; ib < nbd; ib++) {
                int iz = nbd - ib - 1;
                U(u2, iy, ix, iz) = U(u1, iy, ix, iz + 1) + (U(u1, iy, ix, iz) - U(u2, iy, ix, iz + 1)) * bl;
                iz = nzpad - nbd + ib;
                U(u2, iy, ix, iz) = U(u1, iy, ix, iz - 1) + (U(u1, iy, ix, iz) - U(u2, iy, ix, iz - 1)) * bh;
            }
            if (damp)
                for (int ib = 0; ib < nbd - nop; ib++) {
                    float dib = damp[ib];
                    int iz = nbd - ib - 1;
                    real bc = U(u1, iy, ix, iz + 1) + (U(u1, iy, ix, iz) - U(u2, iy, ix, iz + 1)) * bl;
                    U(u2, iy, ix, iz) = bc * (1.f - dib) + U(u2, iy, ix, iz) * dib;
                    iz = nzpad - nbd + ib;
                    bc = U(u1, iy, ix, iz - 1) + (U(u1, iy, ix, iz) - U(u2, iy, ix, iz - 1)) * bh;
                    U(u2, iy, ix, iz) = bc * (1.f - dib) + U(u2, iy, ix, iz) * dib;
                }
            if (fsrf)
                for (int iz = 0; iz < nbd + 1; iz++) U(u2, iy, ix, iz) = 0;
        }
    for (int iy = 0; iy < nypad; iy++)
        for (int iz = 0; iz < nzpad; iz++) {
            float bl = a->xl[(size_t)iy * nzpad + iz], bh = a->xh[(size_t)iy * nzpad + iz];
            for (int ib = nbd - nop; ib < nbd; ib++) {
                int ix = nbd - ib - 1;
                U(u2, iy, ix, iz) = U(u1, iy, ix + 1, iz) + (U(u1, iy, ix, iz) - U(u2, iy, ix + 1, iz)) * bl;
                ix = nxpad - nbd + ib;
                U(u2, iy, ix, iz) = U(u1, iy, ix - 1, iz) + (U(u1, iy, ix, iz) - U(u2, iy, ix - 1, iz)) * bh;
            }
            if (damp)
                for (int ib = 0; ib < nbd - nop; ib++) {
                    float dib = damp[ib];
                    int ix = nbd - ib - 1;
                    real bc = U(u1, iy, ix + 1, iz) + (U(u1, iy, ix, iz) - U(u2, iy, ix + 1, iz)) * bl;
                    U(u2, iy, ix, iz) = bc * (1.f - dib) + U(u2, iy, ix, iz) * dib;
                    ix = nxpad - nbd + ib;
                    bc = U(u1, iy, ix - 1, iz) + (U(u1, iy, ix, iz) - U(u2, iy, ix - 1, iz)) * bh;
                    U(u2, iy, ix, iz) = bc * (1.f - dib) + U(u2, iy, ix, iz) * dib;
                }
        }
    for (int ix = 0; ix < nxpad; ix++)
        for (int iz = 0; iz < nzpad; iz++) {
            float bl = a->yl[(size_t)ix * nzpad + iz], bh = a->yh[(size_t)ix * nzpad + iz];
            for (int ib = nbd - nop; ib < nbd; ib++) {
                int iy = nbd - ib - 1;
                U(u2, iy, ix, iz) = U(u1, iy + 1, ix, iz) + (U(u1, iy, ix, iz) - U(u2, iy + 1, ix, iz)) * bl;
                iy = nypad - nbd + ib;
                U(u2, iy, ix, iz) = U(u1, iy - 1, ix, iz) + (U(u1, iy, ix, iz) - U(u2, iy - 1, ix, iz)) * bh;
            }
            if (damp)
                for (int ib = 0; ib < nbd - nop; ib++) {
                    float dib = damp[ib];
                    int iy = nbd - ib - 1;
                    real bc = U(u1, iy + 1, ix, iz) + (U(u1, iy, ix, iz) - U(u2, iy + 1, ix, iz)) * bl;
                    U(u2, iy, ix, iz) = bc * (1.f - dib) + U(u2, iy, ix, iz) * dib;
                    iy = nypad - nbd + ib;
                    bc = U(u1, iy - 1, ix, iz) + (U(u1, iy, ix, iz) - U(u2, iy - 1, ix, iz)) * bh;
                    U(u2, iy, ix, iz) = bc * (1.f - dib) + U(u2, iy, ix, iz) * dib;
                }
        }
#undef U
}

int orc_cart3d_cpu(const orc_par *p, const float *vel_in, const float *den_in, const float *wav, int ns,
                   const float *sou, int nr, const float *rec, float *dat, float *snaps) {
#ifdef _OPENMP
    if (p->nthreads > 0) omp_set_num_threads(p->nthreads);
#endif
    int nop = p->fdorder / 2, nbd, nzpad, nxpad, nypad;
    if (nop < 1 || nop > 10) return 1;
    orc_cart_padded(p, &nbd, &nzpad, &nxpad, &nypad);
    const int nz = p->n1, nx = p->n2, ny = p->n3;
    const float dz = p->d1, dx = p->d2, dy = p->d3, dt = p->dt;
    const float ozpad = p->o1 - nbd * dz, oxpad = p->o2 - nbd * dx, oypad = p->o3 - nbd * dy;
    float d2[64], d1[64], dd[3] = {dz, dx, dy};
    fdcoef(nop, 3, dd, p->optfd, d2, d1);
    const size_t sx = nzpad, sy = (size_t)nzpad * nxpad, npad = sy * nypad;

    float *vel = malloc(npad * sizeof(float));
    float *rho = den_in ? malloc(npad * sizeof(float)) : NULL;
    real *u0 = calloc(npad, sizeof(real)), *u1 = calloc(npad, sizeof(real));
    expand3(vel_in, vel, nbd, nz, nx, ny);
    if (rho) expand3(den_in, rho, nbd, nz, nx, ny);

    lint *cs = malloc((ns > 0 ? ns : 1) * sizeof(lint)), *cr = malloc((nr > 0 ? nr : 1) * sizeof(lint));
    for (int i = 0; i < ns; i++)
        lint3d(sou[3 * i], sou[3 * i + 1], sou[3 * i + 2], ozpad, oxpad, oypad, dz, dx, dy, nzpad, nxpad, nypad,
               &cs[i]);
    for (int i = 0; i < nr; i++)
        lint3d(rec[3 * i], rec[3 * i + 1], rec[3 * i + 2], ozpad, oxpad, oypad, dz, dx, dy, nzpad, nxpad, nypad,
               &cr[i]);

    /* abcone3d_make(nbd, ...) fdutil.c:1960-2019 on raw velocity */
    abc3 a = {0};
    float spo[4096], damp[4096];
    int have_damp = 0;
    if (p->dabc) {
        a.zl = malloc((size_t)nypad * nxpad * sizeof(float));
        a.zh = malloc((size_t)nypad * nxpad * sizeof(float));
        a.xl = malloc((size_t)nypad * nzpad * sizeof(float));
        a.xh = malloc((size_t)nypad * nzpad * sizeof(float));
        a.yl = malloc((size_t)nxpad * nzpad * sizeof(float));
        a.yh = malloc((size_t)nxpad * nzpad * sizeof(float));
        for (int iy = 0; iy < nypad; iy++)
            for (int ix = 0; ix < nxpad; ix++) {
                float d = vel[iy * sy + ix * sx + nbd] * dt / dz;
                a.zl[(size_t)iy * nxpad + ix] = (1 - d) / (1 + d);
                d = vel[iy * sy + ix * sx + nzpad - nbd - 1] * dt / dz;
                a.zh[(size_t)iy * nxpad + ix] = (1 - d) / (1 + d);
            }
        for (int iy = 0; iy < nypad; iy++)
            for (int iz = 0; iz < nzpad; iz++) {
                float d = vel[iy * sy + nbd * sx + iz] * dt / dx;
                a.xl[(size_t)iy * nzpad + iz] = (1 - d) / (1 + d);
                d = vel[iy * sy + (nxpad - nbd - 1) * sx + iz] * dt / dx;
                a.xh[(size_t)iy * nzpad + iz] = (1 - d) / (1 + d);
            }
        for (int ix = 0; ix < nxpad; ix++)
            for (int iz = 0; iz < nzpad; iz++) {
                float d = vel[nbd * sy + ix * sx + iz] * dt / dy;
                a.yl[(size_t)ix * nzpad + iz] = (1 - d) / (1 + d);
                d = vel[(nypad - nbd - 1) * sy + ix * sx + iz] * dt / dy;
                a.yh[(size_t)ix * nzpad + iz] = (1 - d) / (1 + d);
            }
        if (p->hybrid) {
            if (nbd - nop > 0) {
                damp_w(nbd - nop, damp);
                have_damp = 1;
            }
        } else
            sponge_w(nbd, spo);
    }
    const float dt2 = dt * dt;
    for (size_t i = 0; i < npad; i++) vel[i] *= vel[i] * dt2; /* :287-288 */
    if (p->fsrf && !p->hybrid)                                 /* :289-293 */
        for (int iy = 0; iy < nypad; iy++)
            for (int ix = 0; ix < nxpad; ix++)
                for (int iz = 0; iz < nbd + 1; iz++) vel[iy * sy + ix * sx + iz] = 0;

    /* snapshot window (default: the unpadded model), :341-354 + cut3d_slice */
    const int fz = cut_first(p->o1, ozpad, dz), fx = cut_first(p->o2, oxpad, dx);
    const int fy = cut_first(p->o3, oypad, dy);
    size_t snapsz = p->bnds ? npad : (size_t)nz * nx * ny, isnap = 0;

    for (int it = 0; it < p->nt; it++) {
        step3d(u0, u1, vel, rho, d2, d1, nop, nzpad, nxpad, nypad);
        /* lint3d_inject1_with_vv fdutil.c:1723-1740 / lint3d_inject_with_vv */
        for (int s = 0; s < ns; s++) {
            float dd = p->expl ? wav[it] : wav[(size_t)it * ns + s];
            const lint *c = &cs[s];
            size_t i0 = c->jy * sy + c->jx * sx + c->jz;
            size_t off[8] = {0, 1, sx, sx + 1, sy, sy + 1, sy + sx, sy + sx + 1};
            for (int k = 0; k < 8; k++) u0[i0 + off[k]] += dd * c->w[k] * vel[i0 + off[k]];
        }
        if (p->dabc) {
            if (p->hybrid)
                hybrid3(u0, u1, nzpad, nxpad, nypad, nbd, &a, nop, have_damp ? damp : NULL, p->fsrf);
            else {
                abcone3(u0, u1, nop, &a, p->fsrf, nzpad, nxpad, nypad);
                sponge3(u0, spo, nbd, nzpad, nxpad, nypad);
                sponge3(u1, spo, nbd, nzpad, nxpad, nypad);
            }
        }
        real *t = u0;
        u0 = u1;
        u1 = t;
        if (snaps && p->jsnap > 0 && it % p->jsnap == 0) {
            float *dst = snaps + isnap * snapsz;
            if (p->bnds)
                for (size_t i = 0; i < npad; i++) dst[i] = (float)u0[i];
            else
                for (int iy = 0; iy < ny; iy++)
                    for (int ix = 0; ix < nx; ix++)
                        for (int iz = 0; iz < nz; iz++)
                            dst[((size_t)iy * nx + ix) * nz + iz] = (float)u0[(fy + iy) * sy + (fx + ix) * sx + fz + iz];
            isnap++;
        }
        /* lint3d_extract fdutil.c:1653-1670 */
        for (int r = 0; r < nr; r++) {
            const lint *c = &cr[r];
            size_t i0 = c->jy * sy + c->jx * sx + c->jz;
            dat[(size_t)it * nr + r] =
                (float)(u0[i0] * c->w[0] + u0[i0 + 1] * c->w[1] + u0[i0 + sx] * c->w[2] + u0[i0 + sx + 1] * c->w[3] +
                        u0[i0 + sy] * c->w[4] + u0[i0 + sy + 1] * c->w[5] + u0[i0 + sy + sx] * c->w[6] +
                        u0[i0 + sy + sx + 1] * c->w[7]);
        }
    }
    free(vel);
    free(rho);
    free(u0);
    free(u1);
    free(cs);
    free(cr);
    free(a.zl);
    free(a.zh);
    free(a.xl);
    free(a.xh);
    free(a.yl);
    free(a.yh);
    return 0;
}

double orc_cart3d_cpu_steps(int n1pad, int n2pad, int n3pad, int fdorder, int nsteps, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    int nop = fdorder / 2;
    size_t npad = (size_t)n1pad * n2pad * n3pad;
    float d2[64], d1[64], dd[3] = {5.f, 5.f, 5.f};
    fdcoef(nop, 3, dd, 0, d2, d1);
    float *vel = malloc(npad * sizeof(float));
    real *u0 = malloc(npad * sizeof(real)), *u1 = malloc(npad * sizeof(real));
#pragma omp parallel for
    for (size_t i = 0; i < npad; i++) {
        vel[i] = 0.0225f;
        u0[i] = (real)((i * 2654435761u) % 1000) * 1e-3f;
        u1[i] = (real)((i * 40503u) % 1000) * 1e-3f;
    }
#ifdef _OPENMP
    double t0 = omp_get_wtime();
#endif
    for (int s = 0; s < nsteps; s++) {
        step3d(u0, u1, vel, NULL, d2, d1, nop, n1pad, n2pad, n3pad);
        real *t = u0;
        u0 = u1;
        u1 = t;
    }
#ifdef _OPENMP
    double t1 = omp_get_wtime();
#else
    double t0 = 0, t1 = 0;
#endif
    free(vel);
    free(u0);
    free(u1);
    return t1 - t0;
}
