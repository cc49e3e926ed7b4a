// Host emulation of the reference's GPU programs - test infrastructure for
// the oracle's checker, not product code.
//
// The reference's kernel files (CODE/cart_kernels.cu, CODE/spher_kernels.cu)
// are compiled unchanged as C++ host code: __global__ functions become plain
// functions and every launch runs the grid's threads one after another.  The
// per-step sequences of the programs' main() (MAWEFDcart2Dgpu.cu:362-492,
// MAWEFDcart3Dgpu.cu:380-466, MAWEFDspher2Dgpu.cu:341-419,
// MAWEFDspher3Dgpu.cu:449-566, and MDYNAWEFDcart2Dgpu.cu:362-432 over
// CODE/dyn_cart_kernels.cu) are restated below around those kernels, with
// the reference's own fdutil.c (lint2d_make, lint3d_make, fdutil_init,
// cut2d, cut3d, cut3d_sph) for geometry and windows.
//
// The one-way boundary kernels race on the GPU (threads read neighbours that
// other threads rewrite).  The emulation runs their threads in an order in
// which every thread reads before the cell it reads is rewritten ("snapshot"
// semantics, one of the GPU's possible executions): by distance to the
// nearest face along the swept axis for onewayBC_2D, and by the sum of the
// per-axis face distances for onewayBC_3D.
//
// Two places where the reference's behaviour is undefined are given one
// definite meaning here, so that fixtures are reproducible: the cart 3D
// program leaves most of its y-high one-way coefficients uninitialised
// (MAWEFDcart3Dgpu.cu:292 writes only the diagonal); here they are filled as
// the loop evidently intends.  Extraction rows beyond the data buffer (cart 3D
// pre-incremented row index) are dropped instead of written past its end.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>
#include <vector>

extern "C" {
#include "fdutil.h"
}

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
static dim3 threadIdx, blockIdx, blockDim, gridDim;
#define __global__
#define __device__
static float atomicAdd(float *a, float v) {
    float o = *a;
    *a = o + v;
    return o;
}

namespace ref_cart {
#include "cart_kernels.cu"
}
#undef INDEX2D
#undef INDEX3D
#undef NOP
namespace ref_spher {
#include "spher_kernels.cu"
}
#undef INDEX2D
#undef INDEX3D
#undef NOP
namespace ref_dyn {
#include "dyn_cart_kernels.cu"
}
#undef INDEX2D
#undef INDEX3D
#undef NOP
#define NOP 4
#define MIN(x, y) (((x) < (y)) ? (x) : (y))

// ---------------------------------------------------------------------------
// launch emulation
template <class F>
static void launch(dim3 g, dim3 b, F f) {
    gridDim = g;
    blockDim = b;
    for (unsigned bz = 0; bz < g.z; bz++)
        for (unsigned by = 0; by < g.y; by++)
            for (unsigned bx = 0; bx < g.x; bx++)
                for (unsigned tz = 0; tz < b.z; tz++)
                    for (unsigned ty = 0; ty < b.y; ty++)
                        for (unsigned tx = 0; tx < b.x; tx++) {
                            blockIdx = dim3(bx, by, bz);
                            threadIdx = dim3(tx, ty, tz);
                            f();
                        }
}

// launch with threads ordered by a key of the global thread index (ascending, stable)
template <class F, class K>
static void launch_ordered(dim3 g, dim3 b, F f, K key) {
    struct T {
        unsigned gx, gy, gz;
        long long k;
    };
    std::vector<T> ts;
    for (unsigned z = 0; z < g.z * b.z; z++)
        for (unsigned y = 0; y < g.y * b.y; y++)
            for (unsigned x = 0; x < g.x * b.x; x++) ts.push_back({x, y, z, key(x, y, z)});
    std::stable_sort(ts.begin(), ts.end(), [](const T &a, const T &c) { return a.k < c.k; });
    gridDim = g;
    blockDim = b;
    for (const T &t : ts) {
        blockIdx = dim3(t.gx / b.x, t.gy / b.y, t.gz / b.z);
        threadIdx = dim3(t.gx % b.x, t.gy % b.y, t.gz % b.z);
        f();
    }
}

static long long facedist(long long c, long long n) { return std::min(c, n - 1 - c); }

// The free-surface kernels test only `ira > nrapad - nb` along the fast axis,
// so the threads that round the grid up to a multiple of 8 write past the
// end of each line: into the first samples of the next line, and past the
// end of the array for the last line.  The emulation keeps that slack
// behind every field so those writes stay in owned memory (and are dropped).
static const size_t kSlack = 4096;

extern "C" {

typedef struct {
    int n1, n2, n3;
    float d1, d2, d3;
    float o1, o2, o3;
    int nb, nt;
    float dt;
    int jdata, jsnap, bnds, fsrf, expl, refl;
} gpuref_par;

// ---------------------------------------------------------------------------
// sfAWEFDcart2Dgpu: vel [nx][nz] (axis 1 = z); sou/rec (x, z) pairs
int gpuref_cart2d(const gpuref_par *P, const float *vel, const float *rfl, const float *wav, int ns,
                  const float *sou, int nr, const float *rec, float *dat, float *snaps) {
    using namespace ref_cart;
    const int nz = P->n1, nx = P->n2, nt = P->nt;
    const float dz = P->d1, dx = P->d2, dt = P->dt;
    int nb = P->nb < NOP ? NOP : P->nb;
    sf_axis az = sf_maxa(nz, P->o1, dz), ax = sf_maxa(nx, P->o2, dx);
    fdm2d fdm = fdutil_init(false, P->fsrf, az, ax, nb, 1);
    const int nxpad = fdm->nxpad, nzpad = fdm->nzpad;
    std::vector<float> h_vel((size_t)nxpad * nzpad), h_rfl((size_t)nxpad * nzpad);
    std::vector<float> tt1(vel, vel + (size_t)nx * nz);
    expand_cpu_2d(tt1.data(), h_vel.data(), fdm->nb, nz, nzpad, nx, nxpad);
    if (P->refl) {
        std::vector<float> tr(rfl, rfl + (size_t)nx * nz);
        expand_cpu_2d(tr.data(), h_rfl.data(), fdm->nb, nz, nzpad, nx, nxpad);
    }
    std::vector<float> bzl(nxpad), bzh(nxpad), bxl(nzpad), bxh(nzpad);
    for (int ix = 0; ix < nxpad; ix++) {  // MAWEFDcart2Dgpu.cu:280-285 (x-fastest indexing of h_vel)
        float d = h_vel[NOP * nxpad + ix] * (dt / dz);
        bzl[ix] = (1 - d) / (1 + d);
        d = h_vel[(nzpad - NOP - 1) * nxpad + ix] * (dt / dz);
        bzh[ix] = (1 - d) / (1 + d);
    }
    for (int iz = 0; iz < nzpad; iz++) {
        float d = h_vel[iz * nxpad + NOP] * (dt / dx);
        bxl[iz] = (1 - d) / (1 + d);
        d = h_vel[iz * nxpad + nxpad - NOP - 1] * (dt / dx);
        bxh[iz] = (1 - d) / (1 + d);
    }
    pt2d *ss = (pt2d *)calloc(ns > 0 ? ns : 1, sizeof(pt2d)), *rr = (pt2d *)calloc(nr > 0 ? nr : 1, sizeof(pt2d));
    for (int i = 0; i < ns; i++) {
        ss[i].x = sou[2 * i];
        ss[i].z = sou[2 * i + 1];
    }
    for (int i = 0; i < nr; i++) {
        rr[i].x = rec[2 * i];
        rr[i].z = rec[2 * i + 1];
    }
    lint2d cs = lint2d_make(ns, ss, fdm), cr = lint2d_make(nr, rr, fdm);
    const size_t npad = (size_t)nxpad * nzpad;
    std::vector<float> ppo(npad + kSlack, 0.f), po(npad + kSlack, 0.f), fpo(npad + kSlack, 0.f);
    float **pz = sf_floatalloc2(nzpad, nxpad), **oslice = sf_floatalloc2(nz, nx);
    const int nsmp = nt / (P->jdata > 0 ? P->jdata : 1);
    std::vector<float> dd((size_t)nsmp * nr + nr, 0.f);
    const dim3 g2((unsigned)ceil(nxpad / 8.0f), (unsigned)ceil(nzpad / 8.0f)), b2(8, 8);
    size_t isnap = 0;
    for (int it = 0; it < nt; it++) {
        dim3 gS(MIN(ns, (int)ceil(ns / 1024.0f)), 1), bS(MIN(ns, 1024), 1);
        float *pww = const_cast<float *>(wav);
        if (ns > 0) {
            if (P->expl) {
                if (P->refl)
                    launch(gS, bS, [&] {
                        inject_sources_2D_refl(po.data(), pww, h_rfl.data(), cs->w00, cs->w01, cs->w10, cs->w11,
                                               cs->jx, cs->jz, it, ns, nxpad, nzpad);
                    });
                else
                    launch(gS, bS, [&] {
                        inject_sources_2D(po.data(), pww, h_vel.data(), cs->w00, cs->w01, cs->w10, cs->w11, cs->jx,
                                          cs->jz, it, ns, nxpad, nzpad);
                    });
            } else
                launch(gS, bS, [&] {
                    inject_sources_2D_const(po.data(), pww, cs->w00, cs->w01, cs->w10, cs->w11, cs->jx, cs->jz, it,
                                            ns, nxpad, nzpad);
                });
        }
        launch(g2, b2, [&] { solve_2D(fpo.data(), po.data(), ppo.data(), h_vel.data(), dx, dz, dt, nxpad, nzpad); });
        launch(g2, b2, [&] { shift_2D(fpo.data(), po.data(), ppo.data(), nxpad, nzpad); });
        launch_ordered(
            g2, b2,
            [&] {
                onewayBC_2D(po.data(), ppo.data(), bzl.data(), bzh.data(), bxl.data(), bxh.data(), nxpad, nzpad);
            },
            [&](long long, long long y, long long) { return facedist(y, nzpad); });
        launch(g2, b2, [&] { spongeKernel_2D(po.data(), nxpad, nzpad, nb); });
        launch(g2, b2, [&] { spongeKernel_2D(ppo.data(), nxpad, nzpad, nb); });
        launch(g2, b2, [&] { freeSurf_2D(po.data(), nxpad, nzpad, nb); });
        if (snaps && P->jsnap > 0 && it % P->jsnap == 0) {
            for (int x = 0; x < nxpad; x++)
                for (int z = 0; z < nzpad; z++) pz[x][z] = po[(size_t)z * nxpad + x];
            if (P->bnds) {
                memcpy(snaps + isnap * npad, pz[0], npad * sizeof(float));
            } else {
                cut2d(pz, oslice, fdm, az, ax);
                memcpy(snaps + isnap * (size_t)nz * nx, oslice[0], (size_t)nz * nx * sizeof(float));
            }
            isnap++;
        }
        if (it < nsmp) {
            dim3 gR(MIN(nr, (int)ceil(nr / 1024.0f)), 1), bR(MIN(nr, 1024), 1);
            if (nr > 0)
                launch(gR, bR, [&] {
                    extract_2D(dd.data(), it, nr, nxpad, nzpad, po.data(), cr->jx, cr->jz, cr->w00, cr->w01, cr->w10,
                               cr->w11);
                });
        }
    }
    memcpy(dat, dd.data(), (size_t)nsmp * nr * sizeof(float));
    return 0;
}

// ---------------------------------------------------------------------------
// sfAWEFDcart3Dgpu: vel [ny][nx][nz]; needs nx == nz (the program indexes the
// velocity as if they were equal, MAWEFDcart3Dgpu.cu solve_3D velAddr)
int gpuref_cart3d(const gpuref_par *P, const float *vel, const float *wav, int ns, const float *sou, int nr,
                  const float *rec, float *dat, float *snaps) {
    using namespace ref_cart;
    const int nz = P->n1, nx = P->n2, ny = P->n3, nt = P->nt;
    const float dz = P->d1, dx = P->d2, dy = P->d3, dt = P->dt;
    if (nx != nz) return 2;
    int nb = P->nb < NOP ? NOP : P->nb;
    sf_axis az = sf_maxa(nz, P->o1, dz), ax = sf_maxa(nx, P->o2, dx), ay = sf_maxa(ny, P->o3, dy);
    fdm3d fdm = fdutil3d_init(false, P->fsrf, az, ax, ay, nb, 1);
    const int nxpad = fdm->nxpad, nypad = fdm->nypad, nzpad = fdm->nzpad;
    const size_t npad = (size_t)nxpad * nypad * nzpad;
    std::vector<float> tt1(vel, vel + (size_t)nx * ny * nz), h_vel(npad);
    expand_cpu_3d(tt1.data(), h_vel.data(), fdm->nb, nx, nxpad, ny, nypad, nz, nzpad);
    std::vector<float> bzl((size_t)nxpad * nypad), bzh(bzl.size()), bxl((size_t)nzpad * nypad), bxh(bxl.size()),
        byl((size_t)nxpad * nzpad), byh(byl.size());
    for (int ix = 0; ix < nxpad; ix++)  // MAWEFDcart3Dgpu.cu:271-294
        for (int iy = 0; iy < nypad; iy++) {
            float d = h_vel[(size_t)iy * nxpad * nzpad + NOP * nxpad + ix] * (dt / dz);
            bzl[(size_t)iy * nxpad + ix] = (1 - d) / (1 + d);
            d = h_vel[(size_t)iy * nxpad * nzpad + (nzpad - NOP - 1) * nxpad + ix] * (dt / dz);
            bzh[(size_t)iy * nxpad + ix] = (1 - d) / (1 + d);
        }
    for (int iz = 0; iz < nzpad; iz++)
        for (int iy = 0; iy < nypad; iy++) {
            float d = h_vel[(size_t)iy * nxpad * nzpad + iz * nxpad + NOP] * (dt / dx);
            bxl[(size_t)iy * nzpad + iz] = (1 - d) / (1 + d);
            d = h_vel[(size_t)iy * nxpad * nzpad + iz * nxpad + nxpad - NOP - 1] * (dt / dx);
            bxh[(size_t)iy * nzpad + iz] = (1 - d) / (1 + d);
        }
    for (int iz = 0; iz < nzpad; iz++)
        for (int ix = 0; ix < nxpad; ix++) {
            float d = h_vel[(size_t)NOP * nxpad * nzpad + iz * nxpad + ix] * (dt / dy);
            byl[(size_t)iz * nxpad + ix] = (1 - d) / (1 + d);
            d = h_vel[(size_t)(nypad - NOP - 1) * nxpad * nzpad + iz * nxpad + ix] * (dt / dy);
            byh[(size_t)iz * nxpad + ix] = (1 - d) / (1 + d);  // the reference writes only [iz*nxpad+iz]
        }
    pt3d *ss = (pt3d *)calloc(ns > 0 ? ns : 1, sizeof(pt3d)), *rr = (pt3d *)calloc(nr > 0 ? nr : 1, sizeof(pt3d));
    for (int i = 0; i < ns; i++) {
        ss[i].x = sou[3 * i];
        ss[i].y = sou[3 * i + 1];
        ss[i].z = sou[3 * i + 2];
    }
    for (int i = 0; i < nr; i++) {
        rr[i].x = rec[3 * i];
        rr[i].y = rec[3 * i + 1];
        rr[i].z = rec[3 * i + 2];
    }
    lint3d cs = lint3d_make(ns, ss, fdm), cr = lint3d_make(nr, rr, fdm);
    std::vector<float> ppo(npad + kSlack, 0.f), po(npad + kSlack, 0.f), fpo(npad + kSlack, 0.f);
    float ***p3 = sf_floatalloc3(nzpad, nxpad, nypad), ***oslice = sf_floatalloc3(nz, nx, ny);
    const int jdata = P->jdata > 0 ? P->jdata : 1, nsmp = nt / jdata;
    std::vector<float> dd((size_t)(nsmp + 1) * nr, 0.f);
    const dim3 g3((unsigned)ceil(nxpad / 8.0f), (unsigned)ceil(nypad / 8.0f), (unsigned)ceil(nzpad / 8.0f)),
        b3(8, 8, 8);
    int itr = 0;
    size_t isnap = 0;
    float *pww = const_cast<float *>(wav);
    for (int it = 0; it < nt; it++) {
        dim3 gS(MIN(ns, (int)ceil(ns / 1024.0f)), 1, 1), bS(MIN(ns, 1024), 1, 1);
        if (ns > 0) {
            if (P->expl)
                launch(gS, bS, [&] {
                    inject_sources_3D(po.data(), pww, h_vel.data(), cs->w000, cs->w001, cs->w010, cs->w011, cs->w100,
                                      cs->w101, cs->w110, cs->w111, cs->jx, cs->jy, cs->jz, it, ns, nxpad, nypad, nzpad);
                });
            else
                launch(gS, bS, [&] {
                    inject_sources_3D_const(po.data(), pww, cs->w000, cs->w001, cs->w010, cs->w011, cs->w100,
                                            cs->w101, cs->w110, cs->w111, cs->jx, cs->jy, cs->jz, it, ns, nxpad, nypad,
                                            nzpad);
                });
        }
        launch(g3, b3,
               [&] { solve_3D(fpo.data(), po.data(), ppo.data(), h_vel.data(), dx, dy, dz, dt, nxpad, nypad, nzpad); });
        launch(g3, b3, [&] { shift_3D(fpo.data(), po.data(), ppo.data(), nxpad, nypad, nzpad); });
        launch(g3, b3, [&] { freeSurf_3D(po.data(), nxpad, nypad, nzpad, fdm->nb); });
        launch_ordered(
            g3, b3,
            [&] {
                onewayBC_3D(po.data(), ppo.data(), bzl.data(), bzh.data(), bxl.data(), bxh.data(), byl.data(),
                            byh.data(), nxpad, nypad, nzpad);
            },
            [&](long long x, long long y, long long z) {
                return facedist(x, nxpad) + facedist(y, nypad) + facedist(z, nzpad);
            });
        launch(g3, b3, [&] { spongeKernel_3D(po.data(), nxpad, nypad, nzpad, fdm->nb); });
        launch(g3, b3, [&] { spongeKernel_3D(ppo.data(), nxpad, nypad, nzpad, fdm->nb); });
        if (it % jdata == 0) {
            itr += 1;
            dim3 gR(MIN(nr, (int)ceil(nr / 1024.0f)), 1, 1), bR(MIN(nr, 1024), 1, 1);
            if (nr > 0 && itr < nsmp)
                launch(gR, bR, [&] {
                    extract_3D(dd.data(), itr, nr, nxpad, nypad, nzpad, po.data(), cr->jx, cr->jy, cr->jz, cr->w000,
                               cr->w001, cr->w010, cr->w011, cr->w100, cr->w101, cr->w110, cr->w111);
                });
        }
        if (snaps && P->jsnap > 0 && it % P->jsnap == 0) {
            for (int x = 0; x < nxpad; x++)
                for (int z = 0; z < nzpad; z++)
                    for (int y = 0; y < nypad; y++)
                        p3[y][x][z] = po[(size_t)y * nzpad * nxpad + (size_t)z * nxpad + x];
            if (P->bnds) {
                memcpy(snaps + isnap * npad, p3[0][0], npad * sizeof(float));
            } else {
                cut3d(p3, oslice, fdm, az, ax, ay);
                memcpy(snaps + isnap * (size_t)nz * nx * ny, oslice[0][0], (size_t)nz * nx * ny * sizeof(float));
            }
            isnap++;
        }
    }
    memcpy(dat, dd.data(), (size_t)nsmp * nr * sizeof(float));
    return 0;
}

// ---------------------------------------------------------------------------
// sfAWEFDspher2Dgpu (polar): vel [nth][nra] (axis 1 = r); sou/rec (r, theta)
int gpuref_polar2d(const gpuref_par *P, const float *vel, const float *wav, int ns, const float *sou, int nr,
                   const float *rec, float *dat, float *snaps) {
    using namespace ref_spher;
    const int nra = P->n1, nth = P->n2, nt = P->nt;
    const float dra = P->d1, dth = P->d2, dt = P->dt;
    int nb = P->nb < NOP ? NOP : P->nb;
    sf_axis ara = sf_maxa(nra, P->o1, dra), ath = sf_maxa(nth, P->o2, dth);
    fdm2d fdm = fdutil_init(false, P->fsrf, ath, ara, nb, 1);
    const float oth = fdm->ozpad, ora = fdm->oxpad;
    const int nrapad = fdm->nxpad, nthpad = fdm->nzpad;
    const size_t npad = (size_t)nrapad * nthpad;
    std::vector<float> tt1(vel, vel + (size_t)nra * nth), h_vel(npad);
    expand_cpu_2d(tt1.data(), h_vel.data(), fdm->nb, nra, nrapad, nth, nthpad);
    std::vector<float> bthl(nrapad), bthh(nrapad), bral(nthpad), brah(nthpad);
    for (int ira = 0; ira < nrapad; ira++) {  // MAWEFDspher2Dgpu.cu:257-262
        float d = h_vel[NOP * nrapad + ira] * (dt / dth);
        bthl[ira] = (1 - d) / (1 + d);
        d = h_vel[(nthpad - NOP - 1) * nrapad + ira] * (dt / dth);
        bthh[ira] = (1 - d) / (1 + d);
    }
    for (int ith = 0; ith < nthpad; ith++) {
        float d = h_vel[ith * nrapad + NOP] * (dt / dra);
        bral[ith] = (1 - d) / (1 + d);
        d = h_vel[ith * nrapad + nrapad - NOP - 1] * (dt / dra);
        brah[ith] = (1 - d) / (1 + d);
    }
    pt2d *ss = (pt2d *)calloc(ns > 0 ? ns : 1, sizeof(pt2d)), *rr = (pt2d *)calloc(nr > 0 ? nr : 1, sizeof(pt2d));
    for (int i = 0; i < ns; i++) {
        ss[i].x = sou[2 * i];
        ss[i].z = sou[2 * i + 1];
    }
    for (int i = 0; i < nr; i++) {
        rr[i].x = rec[2 * i];
        rr[i].z = rec[2 * i + 1];
    }
    lint2d cs = lint2d_make(ns, ss, fdm), cr = lint2d_make(nr, rr, fdm);
    std::vector<float> ppo(npad + kSlack, 0.f), po(npad + kSlack, 0.f), fpo(npad + kSlack, 0.f);
    float **pz = sf_floatalloc2(nthpad, nrapad), **oslice = sf_floatalloc2(nth, nra);
    const int nsmp = nt / (P->jdata > 0 ? P->jdata : 1);
    std::vector<float> dd((size_t)nsmp * nr + nr, 0.f);
    const dim3 g2((unsigned)ceil(nrapad / 8.0f), (unsigned)ceil(nthpad / 8.0f)), b2(8, 8);
    size_t isnap = 0;
    float *pww = const_cast<float *>(wav);
    for (int it = 0; it < nt; it++) {
        dim3 gS(MIN(ns, (int)ceil(ns / 1024.0f)), 1), bS(MIN(ns, 1024), 1);
        if (ns > 0) {
            if (P->expl)
                launch(gS, bS, [&] {
                    inject_sources_2D(po.data(), pww, h_vel.data(), cs->w00, cs->w01, cs->w10, cs->w11, cs->jx, cs->jz,
                                      it, ns, nrapad, nthpad);
                });
            else
                launch(gS, bS, [&] {
                    inject_sources_2D_const(po.data(), pww, cs->w00, cs->w01, cs->w10, cs->w11, cs->jx, cs->jz, it,
                                            ns, nrapad, nthpad);
                });
        }
        launch(g2, b2,
               [&] { solve_2D(fpo.data(), po.data(), ppo.data(), h_vel.data(), dra, dth, ora, oth, dt, nrapad, nthpad); });
        launch(g2, b2, [&] { shift_2D(fpo.data(), po.data(), ppo.data(), nrapad, nthpad); });
        launch_ordered(
            g2, b2,
            [&] {
                onewayBC_2D(po.data(), ppo.data(), bthl.data(), bthh.data(), bral.data(), brah.data(), nrapad,
                            nthpad);
            },
            [&](long long, long long y, long long) { return facedist(y, nthpad); });
        launch(g2, b2, [&] { spongeKernel_2D(po.data(), nrapad, nthpad, nb); });
        launch(g2, b2, [&] { spongeKernel_2D(ppo.data(), nrapad, nthpad, nb); });
        if (P->fsrf) launch(g2, b2, [&] { freeSurf_2D(po.data(), nrapad, nthpad, nb); });
        if (snaps && P->jsnap > 0 && it % P->jsnap == 0) {
            for (int ra = 0; ra < nrapad; ra++)
                for (int th = 0; th < nthpad; th++) pz[ra][th] = po[(size_t)th * nrapad + ra];
            if (P->bnds) {
                memcpy(snaps + isnap * npad, pz[0], npad * sizeof(float));
            } else {
                cut2d(pz, oslice, fdm, ath, ara);
                memcpy(snaps + isnap * (size_t)nth * nra, oslice[0], (size_t)nth * nra * sizeof(float));
            }
            isnap++;
        }
        if (it < nsmp && nr > 0) {
            dim3 gR(MIN(nr, (int)ceil(nr / 1024.0f)), 1), bR(MIN(nr, 1024), 1);
            launch(gR, bR, [&] {
                extract_2D(dd.data(), it, nr, nrapad, nthpad, po.data(), cr->jx, cr->jz, cr->w00, cr->w01, cr->w10,
                           cr->w11);
            });
        }
    }
    memcpy(dat, dd.data(), (size_t)nsmp * nr * sizeof(float));
    return 0;
}

// ---------------------------------------------------------------------------
// sfAWEFDspher3Dgpu: vel [nph][nth][nra]; sou/rec (r, phi, theta) triplets
int gpuref_spher3d(const gpuref_par *P, const float *vel, const float *wav, int ns, const float *sou, int nr,
                   const float *rec, float *dat, float *snaps) {
    using namespace ref_spher;
    const int nra = P->n1, nth = P->n2, nph = P->n3, nt = P->nt;
    const float dra = P->d1, dth = P->d2, dph = P->d3, dt = P->dt;
    int nb = P->nb < NOP ? NOP : P->nb;
    sf_axis ara = sf_maxa(nra, P->o1, dra), ath = sf_maxa(nth, P->o2, dth), aph = sf_maxa(nph, P->o3, dph);
    fdm3d fdm = fdutil3d_init(false, P->fsrf, ath, ara, aph, nb, 1);
    const float oth = fdm->ozpad, ora = fdm->oxpad, oph = fdm->oypad;
    const int nrapad = fdm->nxpad, nthpad = fdm->nzpad, nphpad = fdm->nypad;
    const size_t npad = (size_t)nrapad * nthpad * nphpad;
    std::vector<float> tt1(vel, vel + (size_t)nra * nth * nph), h_vel(npad);
    expand_cpu_3D(tt1.data(), h_vel.data(), fdm->nb, nra, nrapad, nph, nphpad, nth, nthpad);
    pt3d *ss = (pt3d *)calloc(ns > 0 ? ns : 1, sizeof(pt3d)), *rr = (pt3d *)calloc(nr > 0 ? nr : 1, sizeof(pt3d));
    for (int i = 0; i < ns; i++) {
        ss[i].x = sou[3 * i];
        ss[i].y = sou[3 * i + 1];
        ss[i].z = sou[3 * i + 2];
    }
    for (int i = 0; i < nr; i++) {
        rr[i].x = rec[3 * i];
        rr[i].y = rec[3 * i + 1];
        rr[i].z = rec[3 * i + 2];
    }
    lint3d cs = lint3d_make(ns, ss, fdm), cr = lint3d_make(nr, rr, fdm);
    std::vector<float> ppo(npad + kSlack, 0.f), po(npad + kSlack, 0.f), fpo(npad + kSlack, 0.f), row(nr > 0 ? nr : 1);
    float ***oslice = sf_floatalloc3(nra, nth, nph);
    const dim3 g3((unsigned)ceil(nrapad / 8.0f), (unsigned)ceil(nphpad / 8.0f), (unsigned)ceil(nthpad / 8.0f)),
        b3(8, 8, 8);
    size_t isnap = 0;
    float *pww = const_cast<float *>(wav);
    for (int it = 0; it < nt; it++) {
        dim3 gS(MIN(ns, (int)ceil(ns / 1024.0f)), 1, 1), bS(MIN(ns, 1024), 1, 1);
        if (ns > 0) {
            if (P->expl)
                launch(gS, bS, [&] {
                    inject_sources_3D(po.data(), pww, h_vel.data(), cs->w000, cs->w001, cs->w010, cs->w011, cs->w100,
                                      cs->w101, cs->w110, cs->w111, cs->jx, cs->jy, cs->jz, it, ns, nrapad, nphpad,
                                      nthpad);
                });
            else
                launch(gS, bS, [&] {
                    inject_sources_3D_const(po.data(), pww, cs->w000, cs->w001, cs->w010, cs->w011, cs->w100,
                                            cs->w101, cs->w110, cs->w111, cs->jx, cs->jy, cs->jz, it, ns, nrapad,
                                            nphpad, nthpad);
                });
        }
        launch(g3, b3, [&] {
            solve_3D(fpo.data(), po.data(), ppo.data(), h_vel.data(), dra, dph, dth, ora, oph, oth, dt, nrapad,
                     nphpad, nthpad);
        });
        launch(g3, b3, [&] { shift_3D(fpo.data(), po.data(), ppo.data(), nrapad, nphpad, nthpad); });
        launch(g3, b3, [&] { spongeKernel_3D(po.data(), nrapad, nphpad, nthpad, nb); });
        launch(g3, b3, [&] { spongeKernel_3D(ppo.data(), nrapad, nphpad, nthpad, nb); });
        if (P->fsrf) launch(g3, b3, [&] { freeSurf_3D(po.data(), nrapad, nphpad, nthpad, nb); });
        if (nr > 0) {
            dim3 gR(MIN(nr, (int)ceil(nr / 1024.0f)), 1, 1), bR(MIN(nr, 1024), 1, 1);
            launch(gR, bR, [&] {
                extract_3D(row.data(), it, nr, nrapad, nphpad, nthpad, po.data(), cr->jx, cr->jy, cr->jz, cr->w000,
                           cr->w001, cr->w010, cr->w011, cr->w100, cr->w101, cr->w110, cr->w111);
            });
            memcpy(dat + (size_t)it * nr, row.data(), nr * sizeof(float));
        }
        if (snaps && P->jsnap > 0 && it % P->jsnap == 0) {
            if (P->bnds)
                memcpy(snaps + isnap * npad, po.data(), npad * sizeof(float));
            else {
                cut3d_sph(po.data(), oslice, fdm, ath, ara, aph);
                memcpy(snaps + isnap * (size_t)nra * nth * nph, oslice[0][0],
                       (size_t)nra * nth * nph * sizeof(float));
            }
            isnap++;
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// sfAWEFDspher3Dgpu adj=y (MAWEFDspher3Dgpu.cu:449-566): data [nt][nr] go back
// in at the receivers through inject_sources_3D_adj at row nt-it-1, no
// extraction, frames at it % jsnap == 0 and at it == nt-kt, and after step
// nt-kt the model window of po is the image.  inject_sources_3D_adj reads its
// data sample before testing its thread index, so the data sit in a buffer
// with slack behind them (threads past nr read it and drop it).  Returns the
// frames written.
int gpuref_spher3d_adj(const gpuref_par *P, const float *vel, const float *data, int nr, const float *rec, int kt,
                       float *image, float *snaps) {
    using namespace ref_spher;
    const int nra = P->n1, nth = P->n2, nph = P->n3, nt = P->nt;
    const float dra = P->d1, dth = P->d2, dph = P->d3, dt = P->dt;
    if (kt < 1 || kt > nt) return -1;
    int nb = P->nb < NOP ? NOP : P->nb;
    sf_axis ara = sf_maxa(nra, P->o1, dra), ath = sf_maxa(nth, P->o2, dth), aph = sf_maxa(nph, P->o3, dph);
    fdm3d fdm = fdutil3d_init(false, P->fsrf, ath, ara, aph, nb, 1);
    const float oth = fdm->ozpad, ora = fdm->oxpad, oph = fdm->oypad;
    const int nrapad = fdm->nxpad, nthpad = fdm->nzpad, nphpad = fdm->nypad;
    const size_t npad = (size_t)nrapad * nthpad * nphpad;
    std::vector<float> tt1(vel, vel + (size_t)nra * nth * nph), h_vel(npad);
    expand_cpu_3D(tt1.data(), h_vel.data(), fdm->nb, nra, nrapad, nph, nphpad, nth, nthpad);
    pt3d *rr = (pt3d *)calloc(nr > 0 ? nr : 1, sizeof(pt3d));
    for (int i = 0; i < nr; i++) {
        rr[i].x = rec[3 * i];
        rr[i].y = rec[3 * i + 1];
        rr[i].z = rec[3 * i + 2];
    }
    lint3d cr = lint3d_make(nr, rr, fdm);
    std::vector<float> ww((size_t)nt * nr + 1024, 0.f);
    memcpy(ww.data(), data, (size_t)nt * nr * sizeof(float));
    std::vector<float> ppo(npad + kSlack, 0.f), po(npad + kSlack, 0.f), fpo(npad + kSlack, 0.f);
    float ***oslice = sf_floatalloc3(nra, nth, nph);
    const dim3 g3((unsigned)ceil(nrapad / 8.0f), (unsigned)ceil(nphpad / 8.0f), (unsigned)ceil(nthpad / 8.0f)),
        b3(8, 8, 8);
    size_t isnap = 0;
    for (int it = 0; it < nt; it++) {
        const int adjt = nt - it - 1;
        dim3 gS(MIN(nr, (int)ceil(nr / 1024.0f)), 1, 1), bS(MIN(nr, 1024), 1, 1);
        launch(gS, bS, [&] {
            inject_sources_3D_adj(po.data(), ww.data(), cr->w000, cr->w001, cr->w010, cr->w011, cr->w100, cr->w101,
                                  cr->w110, cr->w111, cr->jx, cr->jy, cr->jz, adjt, nr, nrapad, nphpad, nthpad);
        });
        launch(g3, b3, [&] {
            solve_3D(fpo.data(), po.data(), ppo.data(), h_vel.data(), dra, dph, dth, ora, oph, oth, dt, nrapad,
                     nphpad, nthpad);
        });
        launch(g3, b3, [&] { shift_3D(fpo.data(), po.data(), ppo.data(), nrapad, nphpad, nthpad); });
        launch(g3, b3, [&] { spongeKernel_3D(po.data(), nrapad, nphpad, nthpad, nb); });
        launch(g3, b3, [&] { spongeKernel_3D(ppo.data(), nrapad, nphpad, nthpad, nb); });
        if (P->fsrf) launch(g3, b3, [&] { freeSurf_3D(po.data(), nrapad, nphpad, nthpad, nb); });
        if (snaps && P->jsnap > 0 && (it % P->jsnap == 0 || it == nt - kt)) {
            if (P->bnds)
                memcpy(snaps + isnap * npad, po.data(), npad * sizeof(float));
            else {
                cut3d_sph(po.data(), oslice, fdm, ath, ara, aph);
                memcpy(snaps + isnap * (size_t)nra * nth * nph, oslice[0][0],
                       (size_t)nra * nth * nph * sizeof(float));
            }
            isnap++;
        }
        if (it == nt - kt) {
            cut3d_sph(po.data(), oslice, fdm, ath, ara, aph);
            memcpy(image, oslice[0][0], (size_t)nra * nth * nph * sizeof(float));
            break;
        }
    }
    return (int)isnap;
}

// ---------------------------------------------------------------------------
// sfDYNAWEFDcart2Dgpu (MDYNAWEFDcart2Dgpu.cu:296-432): vel [nx][nz]; sou
// ns*nst and rec nr*nrt (x, z) points; the kernels of dyn_cart_kernels.cu
// pick entry k*(it+1) of each table.  Traces of every step go to row it
// (the program's buffer holds nt/jdata rows: jdata must be 1).
int gpuref_dyncart2d(const gpuref_par *P, const float *vel, const float *wav, int ns, int nst, const float *sou,
                     int nr, int nrt, const float *rec, float *dat, float *snaps) {
    using namespace ref_dyn;
    const int nz = P->n1, nx = P->n2, nt = P->nt;
    const float dz = P->d1, dx = P->d2, dt = P->dt;
    if (P->jdata != 1) return 2;
    int nb = P->nb < NOP ? NOP : P->nb;
    sf_axis az = sf_maxa(nz, P->o1, dz), ax = sf_maxa(nx, P->o2, dx);
    fdm2d fdm = fdutil_init(false, P->fsrf, az, ax, nb, 1);
    const int nxpad = fdm->nxpad, nzpad = fdm->nzpad;
    std::vector<float> h_vel((size_t)nxpad * nzpad);
    std::vector<float> tt1(vel, vel + (size_t)nx * nz);
    expand_cpu_2d(tt1.data(), h_vel.data(), fdm->nb, nz, nzpad, nx, nxpad);
    std::vector<float> bzl(nxpad), bzh(nxpad), bxl(nzpad), bxh(nzpad);
    for (int ix = 0; ix < nxpad; ix++) {  // MDYNAWEFDcart2Dgpu.cu:275-289
        float d = h_vel[NOP * nxpad + ix] * (dt / dz);
        bzl[ix] = (1 - d) / (1 + d);
        d = h_vel[(nzpad - NOP - 1) * nxpad + ix] * (dt / dz);
        bzh[ix] = (1 - d) / (1 + d);
    }
    for (int iz = 0; iz < nzpad; iz++) {
        float d = h_vel[iz * nxpad + NOP] * (dt / dx);
        bxl[iz] = (1 - d) / (1 + d);
        d = h_vel[iz * nxpad + nxpad - NOP - 1] * (dt / dx);
        bxh[iz] = (1 - d) / (1 + d);
    }
    const int nse = ns * nst, nre = nr * nrt;
    pt2d *ss = (pt2d *)calloc(nse > 0 ? nse : 1, sizeof(pt2d)), *rr = (pt2d *)calloc(nre > 0 ? nre : 1, sizeof(pt2d));
    for (int i = 0; i < nse; i++) {
        ss[i].x = sou[2 * i];
        ss[i].z = sou[2 * i + 1];
    }
    for (int i = 0; i < nre; i++) {
        rr[i].x = rec[2 * i];
        rr[i].z = rec[2 * i + 1];
    }
    lint2d cs = lint2d_make(nse, ss, fdm), cr = lint2d_make(nre, rr, fdm);
    const size_t npad = (size_t)nxpad * nzpad;
    std::vector<float> ppo(npad + kSlack, 0.f), po(npad + kSlack, 0.f), fpo(npad + kSlack, 0.f);
    float **pz = sf_floatalloc2(nzpad, nxpad), **oslice = sf_floatalloc2(nz, nx);
    std::vector<float> dd((size_t)nt * nr + nr, 0.f);
    const dim3 g2((unsigned)ceil(nxpad / 8.0f), (unsigned)ceil(nzpad / 8.0f)), b2(8, 8);
    float *pww = const_cast<float *>(wav);
    size_t isnap = 0;
    for (int it = 0; it < nt; it++) {
        if (ns > 0) {
            dim3 gS(MIN(ns, (int)ceil(ns / 1024.0f)), 1), bS(MIN(ns, 1024), 1);
            launch(gS, bS, [&] {
                inject_sources_2D_dyn(po.data(), pww, cs->w00, cs->w01, cs->w10, cs->w11, cs->jx, cs->jz, it, ns,
                                      nxpad, nzpad);
            });
        }
        launch(g2, b2, [&] { solve_2D(fpo.data(), po.data(), ppo.data(), h_vel.data(), dx, dz, dt, nxpad, nzpad); });
        launch(g2, b2, [&] { shift_2D(fpo.data(), po.data(), ppo.data(), nxpad, nzpad); });
        launch_ordered(
            g2, b2,
            [&] {
                onewayBC_2D(po.data(), ppo.data(), bzl.data(), bzh.data(), bxl.data(), bxh.data(), nxpad, nzpad);
            },
            [&](long long, long long y, long long) { return facedist(y, nzpad); });
        launch(g2, b2, [&] { spongeKernel_2D(po.data(), nxpad, nzpad, nb); });
        launch(g2, b2, [&] { spongeKernel_2D(ppo.data(), nxpad, nzpad, nb); });
        if (P->fsrf) launch(g2, b2, [&] { freeSurf_2D(po.data(), nxpad, nzpad, nb); });
        if (snaps && P->jsnap > 0 && it % P->jsnap == 0) {
            for (int x = 0; x < nxpad; x++)
                for (int z = 0; z < nzpad; z++) pz[x][z] = po[(size_t)z * nxpad + x];
            if (P->bnds) {
                memcpy(snaps + isnap * npad, pz[0], npad * sizeof(float));
            } else {
                cut2d(pz, oslice, fdm, az, ax);
                memcpy(snaps + isnap * (size_t)nz * nx, oslice[0], (size_t)nz * nx * sizeof(float));
            }
            isnap++;
        }
        if (nr > 0) {
            dim3 gR(MIN(nr, (int)ceil(nr / 1024.0f)), 1), bR(MIN(nr, 1024), 1);
            launch(gR, bR, [&] {
                extract_2D_dyn(dd.data(), it, nr, nxpad, nzpad, po.data(), cr->jx, cr->jz, cr->w00, cr->w01,
                               cr->w10, cr->w11);
            });
        }
    }
    memcpy(dat, dd.data(), (size_t)nt * nr * sizeof(float));
    return 0;
}

}  // extern "C"
