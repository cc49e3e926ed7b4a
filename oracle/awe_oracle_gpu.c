/* CPU oracle, part 2: restatement of the reference's GPU programs
 * (CODE/MAWEFD{cart,spher}{2D,3D}gpu.cu over CODE/cart_kernels.cu and
 * CODE/spher_kernels.cu).  TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * Fields use the RSF axis order, axis 1 fastest: cartesian [y][x][z],
 * spherical [phi][theta][r].  The reference keeps cartesian pressure
 * x-fastest; the stencil does not depend on the layout, and where the
 * reference indexes an array with its own flat formula (reflectivity
 * injection, one-way coefficients) the same flat formula is applied here to
 * a buffer with the same element order as the reference's, so the values
 * read are the same.
 *
 * One-way boundary kernels race on the GPU; this restatement uses snapshot
 * semantics (every read sees the field before the kernel), one of the GPU's
 * possible executions, which the host emulation of the reference kernels
 * (oracle/ref/gpu_emul.cpp) reproduces by its thread order.
 *
 * Float operations follow the reference's expression order (compiled with
 * -ffp-contract=off); the sponge factor is FP64 as in the kernels. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "awe_oracle.h"

#define NOPA 4 /* cart_kernels.cu:401, spher_kernels.cu:402 */

/* spongeKernel_2D/3D factor for index distance i (cart_kernels.cu:723-815).
 * The kernels are C++: log(alpha) with a float alpha is the float logarithm
 * (logf), promoted to double; the rest of the expression is double. */
static double sponge_damp(int i, int nb) {
    float alpha = 0.90;
    return exp(-1.0 * fabs((pow((i - 1.0), 2) * (double)logf(alpha)) / (pow(nb, 2))));
}

/* sponge index for a cell; priority order as the kernel's argument order:
 * a (fast kernel axis), then b, then c (c < 0: 2D).  Returns 0 if undamped. */
static int sponge_i(int a, int na, int b, int nbb, int c, int nc, int nb) {
    if (a < nb || b < nb || (c >= 0 && c < nb)) {
        if (a < nb) return nb - a;
        if (b < nb) return nb - b;
        return nb - c;
    }
    if (a > na - nb || b > nbb - nb || (c >= 0 && c > nc - nb)) {
        if (a > na - nb) return a - (na - nb);
        if (b > nbb - nb) return b - (nbb - nb);
        return c - (nc - nb);
    }
    return 0;
}

static float damp_apply(float v, int i, const double *tab) { return i ? (float)((double)v * tab[i]) : v; }

/* lint2d_make / lint3d_make in the fdm axes (z, x, y) */
typedef struct {
    int jz, jx, jy;
    float w[8];
} glint;

static void glint_make(int nd, float x, float y, float z, float oz, float ox, float oy, float dz, float dx, float dy,
                       int nz, int nx, int ny, glint *c) {
    float f1, f2, f3 = 0.f;
    int in = z >= oz && z < oz + (nz - 1) * dz && x >= ox && x < ox + (nx - 1) * dx;
    if (nd == 3) in = in && y >= oy && y < oy + (ny - 1) * dy;
    if (in) {
        c->jz = (int)((z - oz) / dz);
        c->jx = (int)((x - ox) / dx);
        f1 = (z - oz) / dz - c->jz;
        f2 = (x - ox) / dx - c->jx;
        c->jy = 0;
        if (nd == 3) {
            c->jy = (int)((y - oy) / dy);
            f3 = (y - oy) / dy - c->jy;
        }
    } else {
        c->jz = c->jx = c->jy = 0;
        f1 = 1;
        f2 = 0;
        f3 = 0;
    }
    if (nd == 2) {
        c->w[0] = (1 - f1) * (1 - f2);
        c->w[1] = (f1) * (1 - f2);
        c->w[2] = (1 - f1) * (f2);
        c->w[3] = (f1) * (f2);
    } else {
        c->w[0] = (1 - f3) * (1 - f1) * (1 - f2);
        c->w[1] = (1 - f3) * (f1) * (1 - f2);
        c->w[2] = (1 - f3) * (1 - f1) * (f2);
        c->w[3] = (1 - f3) * (f1) * (f2);
        c->w[4] = (f3) * (1 - f1) * (1 - f2);
        c->w[5] = (f3) * (f1) * (1 - f2);
        c->w[6] = (f3) * (1 - f1) * (f2);
        c->w[7] = (f3) * (f1) * (f2);
    }
}

static void pad_clamp(const float *a, float *b, int nb, int n1, int n2, int n3) {
    int p1 = n1 + 2 * nb, p2 = n2 + 2 * nb, p3 = n3 > 1 ? n3 + 2 * nb : 1, o3 = n3 > 1 ? nb : 0;
    for (int i3 = 0; i3 < p3; i3++) {
        int j3 = i3 - o3 < 0 ? 0 : (i3 - o3 >= n3 ? n3 - 1 : i3 - o3);
        for (int i2 = 0; i2 < p2; i2++) {
            int j2 = i2 - nb < 0 ? 0 : (i2 - nb >= n2 ? n2 - 1 : i2 - nb);
            for (int i1 = 0; i1 < p1; i1++) {
                int j1 = i1 - nb < 0 ? 0 : (i1 - nb >= n1 ? n1 - 1 : i1 - nb);
                b[((size_t)i3 * p2 + i2) * p1 + i1] = a[((size_t)j3 * n2 + j2) * n1 + j1];
            }
        }
    }
}

/* inject_sources_2D reflectivity (cart_kernels.cu:232-276, spher_kernels.cu:
 * same structure): the first neighbour in the fixed order whose value differs;
 * neighbour offsets in the kernel's own flat indexing (row stride `rs`).
 * A neighbour outside the array (the reference reads out of bounds there)
 * counts as equal. */
static float refl2(const float *v, size_t n, long long s, long long rs) {
    const long long off[7][2] = {{1, 0}, {0, 1}, {1, 1}, {0, -1}, {-1, -1}, {1, -1}, {-1, 1}}; /* (dz, dx) */
    const float v0 = v[s];
    for (int k = 0; k < 7; k++) {
        long long t = s + off[k][0] * rs + off[k][1];
        if (t < 0 || (size_t)t >= n) continue;
        if (v0 != v[t]) return fabsf((v0 - v[t]) / (v0 + v[t]));
    }
    return 0;
}

/* inject_sources_3D reflectivity (cart_kernels.cu:278-372): 26 neighbours in
 * the kernel's order, offsets (dy, dz, dx) in its flat indexing */
static float refl3(const float *v, size_t n, long long s, long long rs, long long ps) {
    static const int off[26][3] = {{0, 1, 0},   {1, 0, 0},   {0, 0, 1},   {0, -1, 0},  {-1, 0, 0},  {0, 0, -1},
                                   {0, 1, 1},   {0, -1, -1}, {0, 1, -1},  {0, -1, 1},  {1, 1, 0},   {-1, -1, 0},
                                   {1, -1, 0},  {-1, 1, 0},  {1, 0, 1},   {-1, 0, -1}, {1, 0, -1},  {-1, 0, 1},
                                   {1, 0, -1},  {1, 1, 1},   {1, 1, -1},  {1, -1, 1},  {1, -1, -1}, {-1, 1, 1},
                                   {-1, 1, -1}, {-1, -1, 1}};
    const float v0 = v[s];
    for (int k = 0; k < 26; k++) {
        long long t = s + off[k][0] * ps + off[k][1] * rs + off[k][2];
        if (t < 0 || (size_t)t >= n) continue;
        if (v0 != v[t]) return fabsf((v0 - v[t]) / (v0 + v[t]));
    }
    return 0;
}

int orc_gpu_snap_frames(int nt, int jsnap) { return jsnap > 0 ? (nt - 1) / jsnap + 1 : 0; }

/* ------------------------------------------------------------------ */
/* table entry of point k at step it for a moving geometry (move < 0: fixed
 * points, entry k).  move 0: one row of n positions per step, the last row
 * held; move 1: k*(it+1), the index of MDYNAWEFDcart2Dgpu's kernels
 * (dyn_cart_kernels.cu:133 inject_sources_2D_dyn, :326 extract_2D_dyn). */
static size_t move_entry(int move, int k, int it, int n, int rows) {
    if (move == 0) return (size_t)(it < rows ? it : rows - 1) * n + k;
    if (move == 1) return (size_t)k * (it + 1);
    return (size_t)k;
}

/* MAWEFDcart2Dgpu.cu:362-492.  vel/rfl [nx][nz]; sou/rec (x,z); dat [nt/jdata][nr].
 * With a moving geometry (move >= 0) sou holds ns*nst and rec nr*nrt
 * points; move 1 is MDYNAWEFDcart2Dgpu.cu:362-432, whose loop is this one
 * with unscaled injection and the free surface only with free=y
 * (MDYNAWEFDcart2Dgpu.cu:393-396). */
static int gpu_cart2d_move(const orc_gpar *P, const float *vel_in, const float *rfl_in, const float *wav, int ns,
                           int nst, const float *sou, int nr, int nrt, const float *rec, int move, float *dat,
                           float *snaps) {
    const int nz = P->n1, nx = P->n2, nt = P->nt;
    const float dz = P->d1, dx = P->d2, dt = P->dt;
    const int nb = P->nb < NOPA ? NOPA : P->nb;
    const int nzpad = nz + 2 * nb, nxpad = nx + 2 * nb;
    const float ozpad = P->o1 - nb * dz, oxpad = P->o2 - nb * dx;
    const size_t npad = (size_t)nzpad * nxpad;
    float *v = malloc(npad * 4), *rf = malloc(npad * 4), *po = calloc(npad, 4), *ppo = calloc(npad, 4),
          *fpo = calloc(npad, 4);
    pad_clamp(vel_in, v, nb, nz, nx, 1);
    if (P->refl) pad_clamp(rfl_in, rf, nb, nz, nx, 1);
    double tab[4096];
    for (int i = 1; i <= nb; i++) tab[i] = sponge_damp(i, nb);
    /* one-way coefficients at the last x column (the only ones the kernel's
     * loop keeps), read with the driver's x-fastest flat index of the
     * z-fastest velocity, MAWEFDcart2Dgpu.cu:280-285 */
    float dq = v[(size_t)NOPA * nxpad + nxpad - 1] * (dt / dz), bzl = (1 - dq) / (1 + dq);
    dq = v[(size_t)(nzpad - NOPA - 1) * nxpad + nxpad - 1] * (dt / dz);
    float bzh = (1 - dq) / (1 + dq);
    const size_t nsrc = (size_t)ns * (move >= 0 ? nst : 1), nrec = (size_t)nr * (move >= 0 ? nrt : 1);
    glint *cs = malloc((nsrc ? nsrc : 1) * sizeof(glint)), *cr = malloc((nrec ? nrec : 1) * sizeof(glint));
    for (size_t i = 0; i < nsrc; i++)
        glint_make(2, sou[2 * i], 0, sou[2 * i + 1], ozpad, oxpad, 0, dz, dx, 1, nzpad, nxpad, 1, &cs[i]);
    for (size_t i = 0; i < nrec; i++)
        glint_make(2, rec[2 * i], 0, rec[2 * i + 1], ozpad, oxpad, 0, dz, dx, 1, nzpad, nxpad, 1, &cr[i]);
    const int fsurf = move != 1 || P->fsrf;
    const int jdata = P->jdata > 0 ? P->jdata : 1, nsmp = nt / jdata;
    const int fz = (int)(floor)((P->o1 - ozpad) / dz), fx = (int)(floor)((P->o2 - oxpad) / dx);
    size_t isnap = 0;
#define C2(ix, iz) ((size_t)(ix) * nzpad + (iz))
    for (int it = 0; it < nt; it++) {
        const float wa = wav[it];
        for (int s = 0; s < ns; s++) { /* inject into po, kernel order of corners */
            const glint *c = &cs[move_entry(move, s, it, ns, nst)];
            float r = 1.f;
            int mode = P->expl ? (P->refl ? 2 : 1) : 0;
            size_t k00 = C2(c->jx, c->jz), k01 = C2(c->jx, c->jz + 1), k10 = C2(c->jx + 1, c->jz),
                   k11 = C2(c->jx + 1, c->jz + 1);
            if (mode == 1) {
                r = refl2(v, npad, (long long)c->jz * nxpad + c->jx, nxpad);
                po[k00] += wa * c->w[0] * r;
                po[k01] += wa * c->w[1] * r;
                po[k10] += wa * c->w[2] * r;
                po[k11] += wa * c->w[3] * r;
            } else if (mode == 2) { /* inject_sources_2D_refl: rfl read with the x-fastest flat index */
                po[k00] += wa * c->w[0] * rf[(size_t)c->jz * nxpad + c->jx];
                po[k01] += wa * c->w[1] * rf[(size_t)(c->jz + 1) * nxpad + c->jx];
                po[k10] += wa * c->w[2] * rf[(size_t)c->jz * nxpad + c->jx + 1];
                po[k11] += wa * c->w[3] * rf[(size_t)(c->jz + 1) * nxpad + c->jx + 1];
            } else {
                po[k00] += wa * c->w[0];
                po[k01] += wa * c->w[1];
                po[k10] += wa * c->w[2];
                po[k11] += wa * c->w[3];
            }
        }
        /* solve_2D, cart_kernels.cu:403-443 */
        for (int ix = 0; ix < nxpad; ix++)
            for (int iz = 0; iz < nzpad; iz++) {
                size_t c = C2(ix, iz);
                float lap;
                if (ix >= NOPA && ix < nxpad - NOPA && iz >= NOPA && iz < nzpad - NOPA) {
                    float pxx = po[C2(ix + 1, iz)] - 2 * po[c] + po[C2(ix - 1, iz)];
                    pxx = pxx / (dx * dx);
                    float pzz = po[c + 1] - 2 * po[c] + po[c - 1];
                    pzz = pzz / (dz * dz);
                    lap = pxx + pzz;
                } else
                    lap = 0.;
                fpo[c] = (dt * dt) * (v[c] * v[c] * lap) + 2 * po[c] - ppo[c];
            }
        /* shift_2D: ppo <- po, po <- fpo */
        float *t = ppo;
        ppo = po;
        po = fpo;
        fpo = t;
        /* onewayBC_2D with snapshot reads (cart_kernels.cu:622-667): rows
         * 1..4 / nzpad-5..nzpad-2 (and below nxpad), every x, from column nxpad-1 */
        {
            float top[NOPA + 1], bot[NOPA + 1];
            for (int k = 1; k <= NOPA; k++) {
                top[k] = po[C2(nxpad - 1, k + 1)];
                bot[k] = po[C2(nxpad - 1, nzpad - NOPA - 2 + k)];
            }
            for (int ix = 0; ix < nxpad; ix++) {
                for (int k = 1; k <= NOPA; k++) {
                    int iz = k; /* top: iz == NOP - iop */
                    if (iz < nxpad) po[C2(ix, iz)] = ppo[C2(nxpad - 1, iz + 1)] + (ppo[C2(ix, iz)] - top[k]) * bzl;
                }
                for (int k = 1; k <= NOPA; k++) {
                    int iz = nzpad - NOPA - 2 + k; /* bottom: iz == nzpad-NOP+iop-1 */
                    if (iz < nxpad) po[C2(ix, iz)] = ppo[C2(nxpad - 1, iz - 1)] + (ppo[C2(ix, iz)] - bot[k]) * bzh;
                }
            }
        }
        /* spongeKernel_2D on po and ppo (kernel x = cart x), freeSurf_2D on po */
        for (int ix = 0; ix < nxpad; ix++)
            for (int iz = 0; iz < nzpad; iz++) {
                int i = sponge_i(ix, nxpad, iz, nzpad, -1, 0, nb);
                po[C2(ix, iz)] = damp_apply(po[C2(ix, iz)], i, tab);
                ppo[C2(ix, iz)] = damp_apply(ppo[C2(ix, iz)], i, tab);
                if (fsurf && ix > nxpad - nb) po[C2(ix, iz)] = 0;
            }
        /* freeSurf_2D's threads past nxpad (grid rounded up to 8) zero the
         * first samples of the next row (row = z in the kernel's x-fastest view) */
        if (fsurf)
            for (int iz = 0; iz + 1 < nzpad; iz++)
                for (int k = 0; k < 8 * ((nxpad + 7) / 8) - nxpad; k++) po[C2(k, iz + 1)] = 0;
        if (snaps && P->jsnap > 0 && it % P->jsnap == 0) {
            if (P->bnds) {
                memcpy(snaps + isnap * npad, po, npad * 4);
            } else {
                float *dst = snaps + isnap * (size_t)nz * nx;
                for (int ix = 0; ix < nx; ix++)
                    for (int iz = 0; iz < nz; iz++) dst[(size_t)ix * nz + iz] = po[C2(fx + ix, fz + iz)];
            }
            isnap++;
        }
        if (it < nsmp)
            for (int r = 0; r < nr; r++) {
                const glint *c = &cr[move_entry(move, r, it, nr, nrt)];
                dat[(size_t)it * nr + r] = po[C2(c->jx, c->jz)] * c->w[0] + po[C2(c->jx, c->jz + 1)] * c->w[1] +
                                           po[C2(c->jx + 1, c->jz)] * c->w[2] +
                                           po[C2(c->jx + 1, c->jz + 1)] * c->w[3];
            }
    }
#undef C2
    free(v);
    free(rf);
    free(po);
    free(ppo);
    free(fpo);
    free(cs);
    free(cr);
    return 0;
}

/* ------------------------------------------------------------------ */
/* MAWEFDcart3Dgpu.cu:380-466 (nx == nz, as that program's velocity indexing
 * assumes).  vel [ny][nx][nz]; sou/rec (x,y,z); dat [nt/jdata][nr] with the
 * program's pre-incremented row (row 0 stays zero). */
static int gpu_cart3d(const orc_gpar *P, const float *vel_in, const float *wav, int ns, const float *sou, int nr,
                      const float *rec, float *dat, float *snaps) {
    const int nz = P->n1, nx = P->n2, ny = P->n3, nt = P->nt;
    if (nx != nz) return 2;
    const float dz = P->d1, dx = P->d2, dy = P->d3, dt = P->dt;
    const int nb = P->nb < NOPA ? NOPA : P->nb;
    const int nzpad = nz + 2 * nb, nxpad = nx + 2 * nb, nypad = ny + 2 * nb;
    const float ozpad = P->o1 - nb * dz, oxpad = P->o2 - nb * dx, oypad = P->o3 - nb * dy;
    const size_t sx = nzpad, sy = (size_t)nzpad * nxpad, npad = sy * nypad;
    float *v = malloc(npad * 4), *po = calloc(npad, 4), *ppo = calloc(npad, 4), *fpo = calloc(npad, 4),
          *ps = malloc(npad * 4);
    pad_clamp(vel_in, v, nb, nz, nx, ny);
    double tab[4096];
    for (int i = 1; i <= nb; i++) tab[i] = sponge_damp(i, nb);
    /* one-way coefficient tables with the driver's flat indices
     * (MAWEFDcart3Dgpu.cu:271-294; equal to these with nxpad == nzpad) */
    const size_t n2 = (size_t)nxpad * nzpad;
    float *bzl = malloc(nxpad * nypad * 4), *bzh = malloc(nxpad * nypad * 4), *bxl = malloc(nzpad * nypad * 4),
          *bxh = malloc(nzpad * nypad * 4), *byl = malloc(nxpad * nzpad * 4), *byh = malloc(nxpad * nzpad * 4);
    for (int ix = 0; ix < nxpad; ix++)
        for (int iy = 0; iy < nypad; iy++) {
            float d = v[iy * n2 + NOPA * nxpad + ix] * (dt / dz);
            bzl[iy * nxpad + ix] = (1 - d) / (1 + d);
            d = v[iy * n2 + (nzpad - NOPA - 1) * nxpad + ix] * (dt / dz);
            bzh[iy * nxpad + ix] = (1 - d) / (1 + d);
        }
    for (int iz = 0; iz < nzpad; iz++)
        for (int iy = 0; iy < nypad; iy++) {
            float d = v[iy * n2 + iz * nxpad + NOPA] * (dt / dx);
            bxl[iy * nzpad + iz] = (1 - d) / (1 + d);
            d = v[iy * n2 + iz * nxpad + nxpad - NOPA - 1] * (dt / dx);
            bxh[iy * nzpad + iz] = (1 - d) / (1 + d);
        }
    for (int iz = 0; iz < nzpad; iz++)
        for (int ix = 0; ix < nxpad; ix++) {
            float d = v[NOPA * n2 + iz * nxpad + ix] * (dt / dy);
            byl[iz * nxpad + ix] = (1 - d) / (1 + d);
            d = v[(nypad - NOPA - 1) * n2 + iz * nxpad + ix] * (dt / dy);
            byh[iz * nxpad + ix] = (1 - d) / (1 + d);
        }
    glint *cs = malloc((ns ? ns : 1) * sizeof(glint)), *cr = malloc((nr ? nr : 1) * sizeof(glint));
    for (int i = 0; i < ns; i++)
        glint_make(3, sou[3 * i], sou[3 * i + 1], sou[3 * i + 2], ozpad, oxpad, oypad, dz, dx, dy, nzpad, nxpad,
                   nypad, &cs[i]);
    for (int i = 0; i < nr; i++)
        glint_make(3, rec[3 * i], rec[3 * i + 1], rec[3 * i + 2], ozpad, oxpad, oypad, dz, dx, dy, nzpad, nxpad,
                   nypad, &cr[i]);
    const int jdata = P->jdata > 0 ? P->jdata : 1, nsmp = nt / jdata;
    memset(dat, 0, (size_t)nsmp * nr * 4);
    const int fz = (int)(floor)((P->o1 - ozpad) / dz + 0.0001f), fx = (int)(floor)((P->o2 - oxpad) / dx + 0.0001f),
              fy = (int)(floor)((P->o3 - oypad) / dy + 0.0001f);
    int itr = 0;
    size_t isnap = 0;
#define C3(iy, ix, iz) ((size_t)(iy) * sy + (size_t)(ix) * sx + (iz))
    const size_t off[8] = {0, 1, sx, sx + 1, sy, sy + 1, sy + sx, sy + sx + 1};
    for (int it = 0; it < nt; it++) {
        const float wa = wav[it];
        for (int s = 0; s < ns; s++) {
            const glint *c = &cs[s];
            size_t b = C3(c->jy, c->jx, c->jz);
            float r = 1.f;
            if (P->expl) r = refl3(v, npad, (long long)c->jy * n2 + (long long)c->jz * nxpad + c->jx, nxpad, n2);
            for (int k = 0; k < 8; k++) po[b + off[k]] += P->expl ? wa * c->w[k] * r : wa * c->w[k];
        }
        /* solve_3D, cart_kernels.cu:445-492 */
        for (int iy = 0; iy < nypad; iy++)
            for (int ix = 0; ix < nxpad; ix++)
                for (int iz = 0; iz < nzpad; iz++) {
                    size_t c = C3(iy, ix, iz);
                    float lap;
                    if (ix >= NOPA && ix < nxpad - NOPA && iy >= NOPA && iy < nypad - NOPA && iz >= NOPA &&
                        iz < nzpad - NOPA) {
                        float pxx = po[c + sx] - 2 * po[c] + po[c - sx];
                        pxx = pxx / (dx * dx);
                        float pyy = po[c + sy] - 2 * po[c] + po[c - sy];
                        pyy = pyy / (dy * dy);
                        float pzz = po[c + 1] - 2 * po[c] + po[c - 1];
                        pzz = pzz / (dz * dz);
                        lap = pxx + pyy + pzz;
                    } else
                        lap = 0.;
                    fpo[c] = (dt * dt) * (v[c] * v[c] * lap) + 2 * po[c] - ppo[c];
                }
        float *t = ppo;
        ppo = po;
        po = fpo;
        fpo = t;
        /* freeSurf_3D (unconditional, z < nb) */
        for (int iy = 0; iy < nypad; iy++)
            for (int ix = 0; ix < nxpad; ix++)
                for (int iz = 0; iz < nb && iz < nzpad; iz++) po[C3(iy, ix, iz)] = 0;
        /* onewayBC_3D with snapshot reads (cart_kernels.cu:670-720): the last
         * applicable face formula wins; the x-high face uses the z-high table */
        memcpy(ps, po, npad * 4);
        for (int iy = 0; iy < nypad; iy++)
            for (int ix = 0; ix < nxpad; ix++)
                for (int iz = 0; iz < nzpad; iz++) {
                    size_t c = C3(iy, ix, iz);
                    int any = 0;
                    float val = 0;
                    if (iz <= NOPA) {
                        val = ppo[c + 1] + (ppo[c] - ps[c + 1]) * bzl[iy * nxpad + ix];
                        any = 1;
                    }
                    if (iz >= nzpad - NOPA - 1) {
                        val = ppo[c - 1] + (ppo[c] - ps[c - 1]) * bzh[iy * nxpad + ix];
                        any = 1;
                    }
                    if (ix <= NOPA) {
                        val = ppo[c + sx] + (ppo[c] - ps[c + sx]) * bxl[iy * nzpad + iz];
                        any = 1;
                    }
                    if (ix >= nxpad - NOPA - 1) {
                        val = ppo[c - sx] + (ppo[c] - ps[c - sx]) * bzh[iy * nzpad + iz];
                        any = 1;
                    }
                    if (iy <= NOPA) {
                        val = ppo[c + sy] + (ppo[c] - ps[c + sy]) * byl[iz * nxpad + ix];
                        any = 1;
                    }
                    if (iy >= nypad - NOPA - 1) {
                        val = ppo[c - sy] + (ppo[c] - ps[c - sy]) * byh[iz * nxpad + ix];
                        any = 1;
                    }
                    if (any) po[c] = val;
                }
        /* spongeKernel_3D on po, ppo: priority x, y, z */
        for (int iy = 0; iy < nypad; iy++)
            for (int ix = 0; ix < nxpad; ix++)
                for (int iz = 0; iz < nzpad; iz++) {
                    int i = sponge_i(ix, nxpad, iy, nypad, iz, nzpad, nb);
                    size_t c = C3(iy, ix, iz);
                    po[c] = damp_apply(po[c], i, tab);
                    ppo[c] = damp_apply(ppo[c], i, tab);
                }
        if (it % jdata == 0) {
            itr += 1;
            if (itr < nsmp)
                for (int r = 0; r < nr; r++) {
                    const glint *c = &cr[r];
                    size_t b = C3(c->jy, c->jx, c->jz);
                    float acc = po[b] * c->w[0];
                    for (int k = 1; k < 8; k++) acc = acc + po[b + off[k]] * c->w[k];
                    dat[(size_t)itr * nr + r] = acc;
                }
        }
        if (snaps && P->jsnap > 0 && it % P->jsnap == 0) {
            if (P->bnds) {
                memcpy(snaps + isnap * npad, po, npad * 4);
            } else {
                float *dst = snaps + isnap * (size_t)nz * nx * ny;
                for (int iy = 0; iy < ny; iy++)
                    for (int ix = 0; ix < nx; ix++)
                        for (int iz = 0; iz < nz; iz++)
                            dst[((size_t)iy * nx + ix) * nz + iz] = po[C3(fy + iy, fx + ix, fz + iz)];
            }
            isnap++;
        }
    }
#undef C3
    free(v);
    free(po);
    free(ppo);
    free(fpo);
    free(ps);
    free(bzl);
    free(bzh);
    free(bxl);
    free(bxh);
    free(byl);
    free(byh);
    free(cs);
    free(cr);
    return 0;
}

/* ------------------------------------------------------------------ */
/* MAWEFDspher2Dgpu.cu:341-419.  vel [nth][nra]; sou/rec (r, theta);
 * snapshots theta-fastest ([r][theta]) as that program writes them. */
static int gpu_polar2d(const orc_gpar *P, const float *vel_in, const float *wav, int ns, const float *sou, int nr,
                       const float *rec, float *dat, float *snaps) {
    const int nra = P->n1, nth = P->n2, nt = P->nt;
    const float dra = P->d1, dth = P->d2, dt = P->dt;
    const int nb = P->nb < NOPA ? NOPA : P->nb;
    const int nrapad = nra + 2 * nb, nthpad = nth + 2 * nb;
    const float orpad = P->o1 - nb * dra, othpad = P->o2 - nb * dth; /* fdm: x = r, z = theta */
    const size_t npad = (size_t)nrapad * nthpad;
    float *v = malloc(npad * 4), *po = calloc(npad, 4), *ppo = calloc(npad, 4), *fpo = calloc(npad, 4);
    pad_clamp(vel_in, v, nb, nra, nth, 1);
    double tab[4096];
    for (int i = 1; i <= nb; i++) tab[i] = sponge_damp(i, nb);
    float dq = v[(size_t)NOPA * nrapad + nrapad - 1] * (dt / dth), bthl = (1 - dq) / (1 + dq);
    dq = v[(size_t)(nthpad - NOPA - 1) * nrapad + nrapad - 1] * (dt / dth);
    float bthh = (1 - dq) / (1 + dq);
    glint *cs = malloc((ns ? ns : 1) * sizeof(glint)), *cr = malloc((nr ? nr : 1) * sizeof(glint));
    for (int i = 0; i < ns; i++)
        glint_make(2, sou[2 * i], 0, sou[2 * i + 1], othpad, orpad, 0, dth, dra, 1, nthpad, nrapad, 1, &cs[i]);
    for (int i = 0; i < nr; i++)
        glint_make(2, rec[2 * i], 0, rec[2 * i + 1], othpad, orpad, 0, dth, dra, 1, nthpad, nrapad, 1, &cr[i]);
    const int jdata = P->jdata > 0 ? P->jdata : 1, nsmp = nt / jdata;
    const int fth = (int)(floor)((P->o2 - othpad) / dth), fr = (int)(floor)((P->o1 - orpad) / dra);
    size_t isnap = 0;
#define CP(ith, ira) ((size_t)(ith) * nrapad + (ira))
    for (int it = 0; it < nt; it++) {
        const float wa = wav[it];
        for (int s = 0; s < ns; s++) {
            const glint *c = &cs[s]; /* jz = theta, jx = r */
            float r = P->expl ? refl2(v, npad, (long long)c->jz * nrapad + c->jx, nrapad) : 1.f;
            size_t k00 = CP(c->jz, c->jx), k01 = CP(c->jz + 1, c->jx), k10 = CP(c->jz, c->jx + 1),
                   k11 = CP(c->jz + 1, c->jx + 1);
            if (P->expl) {
                po[k00] += wa * c->w[0] * r;
                po[k01] += wa * c->w[1] * r;
                po[k10] += wa * c->w[2] * r;
                po[k11] += wa * c->w[3] * r;
            } else {
                po[k00] += wa * c->w[0];
                po[k01] += wa * c->w[1];
                po[k10] += wa * c->w[2];
                po[k11] += wa * c->w[3];
            }
        }
        /* solve_2D, spher_kernels.cu:404-453 */
        for (int ith = 0; ith < nthpad; ith++)
            for (int ira = 0; ira < nrapad; ira++) {
                size_t c = CP(ith, ira);
                float ra = dra * ira + orpad, lap, vv = v[c];
                if (ira >= NOPA && ira < nrapad - NOPA && ith >= NOPA && ith < nthpad - NOPA) {
                    float compra = ((1 / (dra * dra)) + (1 / (2 * ra * dra))) * po[c - 1] + (-2 / (dra * dra)) * po[c] +
                                   ((1 / (dra * dra)) - (1 / (2 * ra * dra))) * po[c + 1];
                    float compth = ((1 / (ra * ra * dth * dth))) * po[c - nrapad] +
                                   (-2 / (ra * ra * dth * dth)) * po[c] +
                                   ((1 / (ra * ra * dth * dth))) * po[c + nrapad];
                    lap = compra + compth;
                } else
                    lap = 0.;
                fpo[c] = (dt * dt) * (vv * vv) * lap + 2 * po[c] - ppo[c];
            }
        float *t = ppo;
        ppo = po;
        po = fpo;
        fpo = t;
        /* onewayBC_2D (spher_kernels.cu:667-715) with snapshot reads: theta rows */
        {
            float top[NOPA + 1], bot[NOPA + 1];
            for (int k = 1; k <= NOPA; k++) {
                top[k] = po[CP(k + 1, nrapad - 1)];
                bot[k] = po[CP(nthpad - NOPA - 2 + k, nrapad - 1)];
            }
            for (int k = 1; k <= NOPA; k++)
                for (int ira = 0; ira < nrapad; ira++) {
                    int ith = k;
                    po[CP(ith, ira)] = ppo[CP(ith + 1, nrapad - 1)] + (ppo[CP(ith, ira)] - top[k]) * bthl;
                    ith = nthpad - NOPA - 2 + k;
                    po[CP(ith, ira)] = ppo[CP(ith - 1, nrapad - 1)] + (ppo[CP(ith, ira)] - bot[k]) * bthh;
                }
        }
        for (int ith = 0; ith < nthpad; ith++)
            for (int ira = 0; ira < nrapad; ira++) {
                int i = sponge_i(ira, nrapad, ith, nthpad, -1, 0, nb);
                size_t c = CP(ith, ira);
                po[c] = damp_apply(po[c], i, tab);
                ppo[c] = damp_apply(ppo[c], i, tab);
                if (P->fsrf && ira > nrapad - nb) po[c] = 0;
            }
        if (P->fsrf) /* freeSurf_2D past nrapad: first samples of the next theta row */
            for (int ith = 0; ith + 1 < nthpad; ith++)
                for (int k = 0; k < 8 * ((nrapad + 7) / 8) - nrapad; k++) po[CP(ith + 1, k)] = 0;
        if (snaps && P->jsnap > 0 && it % P->jsnap == 0) {
            if (P->bnds) {
                float *dst = snaps + isnap * npad;
                for (int ira = 0; ira < nrapad; ira++)
                    for (int ith = 0; ith < nthpad; ith++) dst[(size_t)ira * nthpad + ith] = po[CP(ith, ira)];
            } else {
                float *dst = snaps + isnap * (size_t)nra * nth;
                for (int ira = 0; ira < nra; ira++)
                    for (int ith = 0; ith < nth; ith++) dst[(size_t)ira * nth + ith] = po[CP(fth + ith, fr + ira)];
            }
            isnap++;
        }
        if (it < nsmp)
            for (int r = 0; r < nr; r++) {
                const glint *c = &cr[r];
                dat[(size_t)it * nr + r] = po[CP(c->jz, c->jx)] * c->w[0] + po[CP(c->jz + 1, c->jx)] * c->w[1] +
                                           po[CP(c->jz, c->jx + 1)] * c->w[2] +
                                           po[CP(c->jz + 1, c->jx + 1)] * c->w[3];
            }
    }
#undef CP
    free(v);
    free(po);
    free(ppo);
    free(fpo);
    free(cs);
    free(cr);
    return 0;
}

/* ------------------------------------------------------------------ */
/* MAWEFDspher3Dgpu.cu:449-566.  vel [nph][nth][nra]; sou/rec (r, phi, theta);
 * dat [nt][nr] (one row per step).
 * adj_kt > 0: the program's adj=y branch.  The "sources" are then the
 * receivers, the series injected at point s in step it is wav[(nt-1-it)*ns + s]
 * (inject_sources_3D_adj, spher_kernels.cu:367-398: unscaled, the data row
 * nt-1-it), nothing is extracted, frames are taken at it % jsnap == 0 and at
 * it == nt-adj_kt, and after step nt-adj_kt the model window of the wavefield
 * goes to image [nph][nth][nra] and the loop ends (:533-563).  Returns the
 * frames written. */
static int gpu_spher3d_impl(const orc_gpar *P, const float *vel_in, const float *wav, int ns, const float *sou, int nr,
                            const float *rec, float *dat, float *snaps, int adj_kt, float *image) {
    const int nra = P->n1, nth = P->n2, nph = P->n3, nt = P->nt;
    const float dra = P->d1, dth = P->d2, dph = P->d3, dt = P->dt;
    const int nb = P->nb < NOPA ? NOPA : P->nb;
    const int nrapad = nra + 2 * nb, nthpad = nth + 2 * nb, nphpad = nph + 2 * nb;
    const float orpad = P->o1 - nb * dra, othpad = P->o2 - nb * dth, ophpad = P->o3 - nb * dph;
    const size_t st = nrapad, sp = (size_t)nrapad * nthpad, npad = sp * nphpad;
    float *v = malloc(npad * 4), *po = calloc(npad, 4), *ppo = calloc(npad, 4), *fpo = calloc(npad, 4);
    pad_clamp(vel_in, v, nb, nra, nth, nph);
    double tab[4096];
    for (int i = 1; i <= nb; i++) tab[i] = sponge_damp(i, nb);
    glint *cs = malloc((ns ? ns : 1) * sizeof(glint)), *cr = malloc((nr ? nr : 1) * sizeof(glint));
    /* fdm: z = theta, x = r, y = phi; point (x, y, z) = (r, phi, theta) */
    for (int i = 0; i < ns; i++)
        glint_make(3, sou[3 * i], sou[3 * i + 1], sou[3 * i + 2], othpad, orpad, ophpad, dth, dra, dph, nthpad, nrapad,
                   nphpad, &cs[i]);
    for (int i = 0; i < nr; i++)
        glint_make(3, rec[3 * i], rec[3 * i + 1], rec[3 * i + 2], othpad, orpad, ophpad, dth, dra, dph, nthpad, nrapad,
                   nphpad, &cr[i]);
    /* corner offsets: bit 0 = theta (z), bit 1 = r (x), bit 2 = phi (y) */
    size_t off[8];
    for (int k = 0; k < 8; k++) off[k] = ((k & 1) ? st : 0) + ((k & 2) ? 1 : 0) + ((k & 4) ? sp : 0);
    size_t isnap = 0;
    float *mA = malloc(nrapad * 4), *mC = malloc(nrapad * 4);
    float *mB = malloc((size_t)nthpad * nrapad * 4), *mD = malloc((size_t)nthpad * nrapad * 4);
    for (int ith = 0; ith < nthpad; ith++)
        for (int ira = 0; ira < nrapad; ira++) {
            const float ra = dra * ira + orpad, th = dth * ith + othpad;
            const size_t m = (size_t)ith * nrapad + ira;
            mA[ira] = 2 / ra;
            mB[m] = cosf(th) / (ra * ra * sinf(th));
            mC[ira] = 1 / (ra * ra);
            mD[m] = 1 / (ra * ra * sinf(th) * sinf(th));
        }
#define CS(iph, ith, ira) ((size_t)(iph) * sp + (size_t)(ith) * st + (ira))
    for (int it = 0; it < nt; it++) {
        for (int s = 0; s < ns; s++) {
            const float wa = adj_kt > 0 ? wav[(size_t)(nt - 1 - it) * ns + s] : wav[it];
            const glint *c = &cs[s];
            size_t b = CS(c->jy, c->jz, c->jx);
            float r = 1.f;
            if (P->expl && adj_kt <= 0) r = refl3(v, npad, (long long)b, st, sp);
            for (int k = 0; k < 8; k++)
                po[b + off[k]] += (P->expl && adj_kt <= 0) ? wa * c->w[k] * r : wa * c->w[k];
        }
        /* solve_3D, spher_kernels.cu:455-526; the metric factors are the
         * kernel's own float expressions of (ra, th), evaluated once per
         * (theta, r) before the loop (mA, mB, mC, mD), so every cell's
         * operations are the reference's */
#pragma omp parallel for
        for (int iph = 0; iph < nphpad; iph++)
            for (int ith = 0; ith < nthpad; ith++)
                for (int ira = 0; ira < nrapad; ira++) {
                    size_t c = CS(iph, ith, ira);
                    float vv = v[c], lap;
                    if (ira >= NOPA && ira < nrapad - NOPA && iph >= NOPA && iph < nphpad - NOPA && ith >= NOPA &&
                        ith < nthpad - NOPA) {
                        const size_t m = (size_t)ith * nrapad + ira;
                        float pra = po[c + 1] - po[c - 1];
                        pra = pra / (2 * dra);
                        float ppra = po[c + 1] - 2 * po[c] + po[c - 1];
                        ppra = ppra / (dra * dra);
                        float pth = po[c + st] - po[c - st];
                        pth = pth / (2 * dth);
                        float ppth = po[c + st] - 2 * po[c] + po[c - st];
                        ppth = ppth / (dth * dth);
                        float ppph = po[c + sp] - 2 * po[c] + po[c - sp];
                        ppph = ppph / (dph * dph);
                        lap = mA[ira] * pra + ppra + mB[m] * pth + mC[ira] * ppth + mD[m] * ppph;
                    } else
                        lap = 0.;
                    fpo[c] = (dt * dt) * (vv * vv) * lap + 2 * po[c] - ppo[c];
                }
        float *t = ppo;
        ppo = po;
        po = fpo;
        fpo = t;
        /* spongeKernel_3D on po, ppo: kernel axes (x, y, z) = (r, phi, theta) */
#pragma omp parallel for
        for (int iph = 0; iph < nphpad; iph++)
            for (int ith = 0; ith < nthpad; ith++)
                for (int ira = 0; ira < nrapad; ira++) {
                    int i = sponge_i(ira, nrapad, iph, nphpad, ith, nthpad, nb);
                    size_t c = CS(iph, ith, ira);
                    po[c] = damp_apply(po[c], i, tab);
                    ppo[c] = damp_apply(ppo[c], i, tab);
                    if (P->fsrf && ira > nrapad - nb) po[c] = 0;
                }
        if (P->fsrf) /* freeSurf_3D past nrapad: first samples of the next r line */
#pragma omp parallel for
            for (size_t line = 0; line < (size_t)nthpad * nphpad - 1; line++)
                for (int k = 0; k < 8 * ((nrapad + 7) / 8) - nrapad; k++) po[(line + 1) * nrapad + k] = 0;
        for (int r = 0; r < nr && adj_kt <= 0; r++) {
            const glint *c = &cr[r];
            size_t b = CS(c->jy, c->jz, c->jx);
            float acc = po[b] * c->w[0];
            for (int k = 1; k < 8; k++) acc = acc + po[b + off[k]] * c->w[k];
            dat[(size_t)it * nr + r] = acc;
        }
        if (snaps && P->jsnap > 0 && (it % P->jsnap == 0 || (adj_kt > 0 && it == nt - adj_kt))) {
            if (P->bnds) {
                memcpy(snaps + isnap * npad, po, npad * 4);
            } else {
                float *dst = snaps + isnap * (size_t)nra * nth * nph;
                for (int iph = 0; iph < nph; iph++)
                    for (int ith = 0; ith < nth; ith++)
                        for (int ira = 0; ira < nra; ira++)
                            dst[((size_t)iph * nth + ith) * nra + ira] = po[CS(nb + iph, nb + ith, nb + ira)];
            }
            isnap++;
        }
        if (adj_kt > 0 && it == nt - adj_kt) {
            for (int iph = 0; iph < nph; iph++)
                for (int ith = 0; ith < nth; ith++)
                    for (int ira = 0; ira < nra; ira++)
                        image[((size_t)iph * nth + ith) * nra + ira] = po[CS(nb + iph, nb + ith, nb + ira)];
            break;
        }
    }
#undef CS
    free(mA);
    free(mB);
    free(mC);
    free(mD);
    free(v);
    free(po);
    free(ppo);
    free(fpo);
    free(cs);
    free(cr);
    return (int)isnap;
}

static int gpu_spher3d(const orc_gpar *P, const float *vel_in, const float *wav, int ns, const float *sou, int nr,
                       const float *rec, float *dat, float *snaps) {
    return gpu_spher3d_impl(P, vel_in, wav, ns, sou, nr, rec, dat, snaps, 0, NULL) < 0;
}

/* sfAWEFDspher3Dgpu adj=y: data [nt][nr] back-injected at the receivers;
 * image [nph][nth][nra]; snaps as the program writes them.  Returns the
 * frames written, or -1 for kt outside [1, nt]. */
int orc_gpu_spher3d_adj(const orc_gpar *P, const float *vel, const float *data, int nr, const float *rec, int kt,
                        float *image, float *snaps) {
    if (kt < 1 || kt > P->nt) return -1;
    return gpu_spher3d_impl(P, vel, data, nr, rec, 0, NULL, NULL, snaps, kt, image);
}

/* The spherical scheme above with FP64 wavefields and arithmetic (inputs,
 * geometry and sponge table as above; trig in double), to state the FP32
 * error of the spherical configuration.  No snapshots. */
int orc_gpu_spher3d_fp64(const orc_gpar *P, const float *vel_in, const float *wav, int ns, const float *sou, int nr,
                         const float *rec, double *dat) {
    const int nra = P->n1, nth = P->n2, nph = P->n3, nt = P->nt;
    const double dra = P->d1, dth = P->d2, dph = P->d3, dt = P->dt;
    const int nb = P->nb < NOPA ? NOPA : P->nb;
    const int nrapad = nra + 2 * nb, nthpad = nth + 2 * nb, nphpad = nph + 2 * nb;
    const float orpad = P->o1 - nb * P->d1, othpad = P->o2 - nb * P->d2, ophpad = P->o3 - nb * P->d3;
    const size_t st = nrapad, sp = (size_t)nrapad * nthpad, npad = sp * nphpad;
    float *v = malloc(npad * 4);
    double *po = calloc(npad, 8), *ppo = calloc(npad, 8), *fpo = calloc(npad, 8);
    pad_clamp(vel_in, v, nb, nra, nth, nph);
    double tab[4096];
    for (int i = 1; i <= nb; i++) tab[i] = sponge_damp(i, nb);
    glint *cs = malloc((ns ? ns : 1) * sizeof(glint)), *cr = malloc((nr ? nr : 1) * sizeof(glint));
    for (int i = 0; i < ns; i++)
        glint_make(3, sou[3 * i], sou[3 * i + 1], sou[3 * i + 2], othpad, orpad, ophpad, P->d2, P->d1, P->d3, nthpad,
                   nrapad, nphpad, &cs[i]);
    for (int i = 0; i < nr; i++)
        glint_make(3, rec[3 * i], rec[3 * i + 1], rec[3 * i + 2], othpad, orpad, ophpad, P->d2, P->d1, P->d3, nthpad,
                   nrapad, nphpad, &cr[i]);
    size_t off[8];
    for (int k = 0; k < 8; k++) off[k] = ((k & 1) ? st : 0) + ((k & 2) ? 1 : 0) + ((k & 4) ? sp : 0);
#define CS(iph, ith, ira) ((size_t)(iph) * sp + (size_t)(ith) * st + (ira))
    for (int it = 0; it < nt; it++) {
        const double wa = wav[it];
        for (int s = 0; s < ns; s++) {
            const glint *c = &cs[s];
            size_t b = CS(c->jy, c->jz, c->jx);
            double r = 1.0;
            if (P->expl) r = refl3(v, npad, (long long)b, st, sp);
            for (int k = 0; k < 8; k++) po[b + off[k]] += wa * c->w[k] * r;
        }
        for (int iph = 0; iph < nphpad; iph++)
            for (int ith = 0; ith < nthpad; ith++)
                for (int ira = 0; ira < nrapad; ira++) {
                    size_t c = CS(iph, ith, ira);
                    const double ra = dra * ira + orpad, th = dth * ith + othpad, vv = v[c];
                    double lap = 0.;
                    if (ira >= NOPA && ira < nrapad - NOPA && iph >= NOPA && iph < nphpad - NOPA && ith >= NOPA &&
                        ith < nthpad - NOPA) {
                        const double pra = (po[c + 1] - po[c - 1]) / (2 * dra);
                        const double ppra = (po[c + 1] - 2 * po[c] + po[c - 1]) / (dra * dra);
                        const double pth = (po[c + st] - po[c - st]) / (2 * dth);
                        const double ppth = (po[c + st] - 2 * po[c] + po[c - st]) / (dth * dth);
                        const double ppph = (po[c + sp] - 2 * po[c] + po[c - sp]) / (dph * dph);
                        lap = (2 / ra) * pra + ppra + (cos(th) / (ra * ra * sin(th))) * pth + (1 / (ra * ra)) * ppth +
                              (1 / (ra * ra * sin(th) * sin(th))) * ppph;
                    }
                    fpo[c] = (dt * dt) * (vv * vv) * lap + 2 * po[c] - ppo[c];
                }
        double *t = ppo;
        ppo = po;
        po = fpo;
        fpo = t;
        for (int iph = 0; iph < nphpad; iph++)
            for (int ith = 0; ith < nthpad; ith++)
                for (int ira = 0; ira < nrapad; ira++) {
                    int i = sponge_i(ira, nrapad, iph, nphpad, ith, nthpad, nb);
                    size_t c = CS(iph, ith, ira);
                    if (i) {
                        po[c] *= tab[i];
                        ppo[c] *= tab[i];
                    }
                    if (P->fsrf && ira > nrapad - nb) po[c] = 0;
                }
        if (P->fsrf)
            for (size_t line = 0; line + 1 < (size_t)nthpad * nphpad; line++)
                for (int k = 0; k < 8 * ((nrapad + 7) / 8) - nrapad; k++) po[(line + 1) * nrapad + k] = 0;
        for (int r = 0; r < nr; r++) {
            const glint *c = &cr[r];
            size_t b = CS(c->jy, c->jz, c->jx);
            double acc = 0;
            for (int k = 0; k < 8; k++) acc += po[b + off[k]] * c->w[k];
            dat[(size_t)it * nr + r] = acc;
        }
    }
#undef CS
    free(v);
    free(po);
    free(ppo);
    free(fpo);
    free(cs);
    free(cr);
    return 0;
}

int orc_gpu_forward(int kind, const orc_gpar *P, const float *vel, const float *rfl, const float *wav, int ns,
                    const float *sou, int nr, const float *rec, float *dat, float *snaps) {
    switch (kind) {
        case 0: return gpu_cart2d_move(P, vel, rfl, wav, ns, 1, sou, nr, 1, rec, -1, dat, snaps);
        case 1: return gpu_cart3d(P, vel, wav, ns, sou, nr, rec, dat, snaps);
        case 2: return gpu_polar2d(P, vel, wav, ns, sou, nr, rec, dat, snaps);
        case 3: return gpu_spher3d(P, vel, wav, ns, sou, nr, rec, dat, snaps);
    }
    return 1;
}

int orc_gpu_cart2d_moving(const orc_gpar *P, const float *vel, const float *wav, int ns, int nst, const float *sou,
                          int nr, int nrt, const float *rec, int move, float *dat, float *snaps) {
    if (move != 0 && move != 1) return 1;
    return gpu_cart2d_move(P, vel, NULL, wav, ns, nst, sou, nr, nrt, rec, move, dat, snaps);
}
