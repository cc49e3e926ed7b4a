// Kernels for the scheme of the reference's GPU programs
// (CODE/MAWEFD{cart,spher}{2D,3D}gpu.cu over cart_kernels.cu / spher_kernels.cu):
// 2nd-order Laplacian (cartesian, polar, or spherical with metric terms),
// injection into the current level before the update, one-way boundary,
// quadratic-alpha sponge on both time levels, free-surface masks.
//
// Two buffers hold the time levels.  The reference shifts three (ppo <- po,
// po <- fpo) and then sponges both po and ppo; here the new level overwrites
// the previous one in place and the sponge of the level that becomes
// "previous" is applied when it is next read, the same float operation on the
// same value.  Cells that the one-way boundary rewrites or reads (the
// `shell`) are stored unsponged by the step kernel and finished by a two-phase
// boundary pass: phase 1 computes the boundary values from the unmodified
// fields (every read sees the field before the pass - the race-free reading
// of the reference's boundary kernels), phase 2 writes them with the sponge
// and masks.
#include <cuda_runtime.h>

#include "awe_internal.h"
#include "fp_exact.cuh"
#include "gsum.cuh"

namespace awe {

// reference sponge factor, FP64 as in spongeKernel_2D/3D
template <bool EXACT>
__device__ __forceinline__ float damp_a(float v, int i, const double *__restrict__ dtab,
                                        const float *__restrict__ ftab) {
    if (i == 0) return v;
    if constexpr (EXACT) return (float)((double)v * dtab[i]);
    else return v * ftab[i];
}

// sponge index: priority over memory axes pri[0..nd-1] (the kernel's x, y, z)
__device__ __forceinline__ int sponge_index(const int *c, const int *n, const StepAParams &p) {
    const int nb = p.nb;
    bool low = false, high = false;
    for (int k = 0; k < p.nd; k++) {
        const int a = p.pri[k];
        low = low || c[a] < nb;
        high = high || c[a] > n[a] - nb;
    }
    if (low) {
        for (int k = 0; k < p.nd; k++) {
            const int a = p.pri[k];
            if (c[a] < nb) return nb - c[a];
        }
    }
    if (high) {
        for (int k = 0; k < p.nd; k++) {
            const int a = p.pri[k];
            if (c[a] > n[a] - nb) return c[a] - (n[a] - nb);
        }
    }
    return 0;
}

// free-surface masks (value forced to zero), see StepAParams::mask
__device__ __forceinline__ bool masked(const int *c, const int *n, const StepAParams &p) {
    switch (p.mask) {
        case 1:  // cart 2D: x > nxpad - nb, plus the next-row spill of the rounded-up grid
            return c[1] > n[1] - p.nb || (c[1] < p.spill && c[0] >= 1);
        case 2:  // cart 3D (before the boundary): z < nb
            return c[0] < p.nb;
        case 3:  // polar / spherical: r > nrapad - nb, plus the next-line spill
            return c[0] > n[0] - p.nb || (c[0] < p.spill && (c[1] >= 1 || c[2] >= 1));
    }
    return false;
}

__device__ __forceinline__ bool in_shell(const int *c, const int *n, const StepAParams &p) {
    if (p.shell_axes == 0) return false;
    for (int a = 0; a < 3; a++)
        if ((p.shell_axes >> a) & 1)
            if (c[a] < p.shell || c[a] >= n[a] - p.shell) return true;
    return false;
}

template <int GEOM, bool EXACT>
__device__ __forceinline__ float laplacian(const float *__restrict__ A, long long i, const int *c,
                                           const StepAParams &p) {
    const long long s2 = p.g.n1, s3 = (long long)p.g.n1 * p.g.n2;
    const float u = A[i];
    const float u2 = fadd<EXACT>(u, u);  // 2*p, exact
    auto d2 = [&](float m, float pl) {   // (p[+1] - 2 p) + p[-1]
        return fadd<EXACT>(fsub<EXACT>(pl, u2), m);
    };
    // AWE_EXACT divides as the reference; AWE_FAST multiplies by the reciprocal
    auto div = [&](float a, float b, float rb) { return EXACT ? __fdiv_rn(a, b) : a * rb; };
    if constexpr (GEOM == 0) {  // cart 2D (x = axis 2, z = axis 1): pxx + pzz
        const float pxx = div(d2(A[i - s2], A[i + s2]), p.dd2, p.rd[1]);
        const float pzz = div(d2(A[i - 1], A[i + 1]), p.dd1, p.rd[0]);
        return fadd<EXACT>(pxx, pzz);
    } else if constexpr (GEOM == 1) {  // cart 3D: (pxx + pyy) + pzz
        const float pxx = div(d2(A[i - s2], A[i + s2]), p.dd2, p.rd[1]);
        const float pyy = div(d2(A[i - s3], A[i + s3]), p.dd3, p.rd[2]);
        const float pzz = div(d2(A[i - 1], A[i + 1]), p.dd1, p.rd[0]);
        return fadd<EXACT>(fadd<EXACT>(pxx, pyy), pzz);
    } else if constexpr (GEOM == 2) {  // polar (r = axis 1, theta = axis 2)
        const int ir = c[0];
        const float am = __ldg(p.tr0 + ir), ap = __ldg(p.tr1 + ir), b = __ldg(p.tr2 + ir), b0 = __ldg(p.tr3 + ir);
        const float compra =
            fadd<EXACT>(fadd<EXACT>(fmul<EXACT>(am, A[i - 1]), fmul<EXACT>(p.a0, u)), fmul<EXACT>(ap, A[i + 1]));
        const float compth =
            fadd<EXACT>(fadd<EXACT>(fmul<EXACT>(b, A[i - s2]), fmul<EXACT>(b0, u)), fmul<EXACT>(b, A[i + s2]));
        return fadd<EXACT>(compra, compth);
    } else {  // spherical (r = axis 1, theta = axis 2, phi = axis 3)
        const int ir = c[0];
        const float pra = div(fsub<EXACT>(A[i + 1], A[i - 1]), p.dd1, p.rd[0]);    // / (2 dra)
        const float ppra = div(d2(A[i - 1], A[i + 1]), p.dd2, p.rd[1]);              // / dra^2
        const float pth = div(fsub<EXACT>(A[i + s2], A[i - s2]), p.dd3, p.rd[2]);  // / (2 dth)
        const float ppth = div(d2(A[i - s2], A[i + s2]), p.dd4, p.rd[3]);            // / dth^2
        const float ppph = div(d2(A[i - s3], A[i + s3]), p.dd5, p.rd[4]);            // / dph^2
        const long long t = (long long)c[1] * p.g.n1 + ir;
        const float A2 = __ldg(p.tr0 + ir), Cr = __ldg(p.tr1 + ir), B = __ldg(p.tt0 + t), D = __ldg(p.tt1 + t);
        float lap = fadd<EXACT>(fmul<EXACT>(A2, pra), ppra);
        lap = fadd<EXACT>(lap, fmul<EXACT>(B, pth));
        lap = fadd<EXACT>(lap, fmul<EXACT>(Cr, ppth));
        return fadd<EXACT>(lap, fmul<EXACT>(D, ppph));
    }
}

// One step: nxt (previous level, sponge pending) <- new level.
template <int GEOM, bool EXACT>
__global__ void __launch_bounds__(256) k_stepA(const float *__restrict__ cur, float *__restrict__ nxt,
                                               const float *__restrict__ vel, const StepAParams p) {
    const int i1 = blockIdx.x * blockDim.x + threadIdx.x;
    const int i2 = blockIdx.y * blockDim.y + threadIdx.y;
    const int i3 = blockIdx.z;
    const Grid g = p.g;
    if (i1 >= g.n1 || i2 >= g.n2) return;
    const int c[3] = {i1, i2, i3}, n[3] = {g.n1, g.n2, g.n3};
    const long long i = ((long long)i3 * g.n2 + i2) * g.n1 + i1;
    const int si = sponge_index(c, n, p);
    const float q = damp_a<EXACT>(nxt[i], si, p.dtab, p.ftab);  // previous level, its sponge applied now
    bool interior = true;
    for (int a = 0; a < p.nd; a++) interior = interior && c[a] >= 4 && c[a] < n[a] - 4;
    const float lap = interior ? laplacian<GEOM, EXACT>(cur, i, c, p) : 0.f;
    const float v = __ldg(vel + i), u = cur[i];
    // cart: (dt*dt)*(v*v*lap) + 2p - pp ; polar/spherical: (dt*dt)*(v*v)*lap + 2p - pp
    float a;
    if constexpr (GEOM <= 1)
        a = fmul<EXACT>(p.dt2, fmul<EXACT>(fmul<EXACT>(v, v), lap));
    else
        a = fmul<EXACT>(fmul<EXACT>(p.dt2, fmul<EXACT>(v, v)), lap);
    float f = fsub<EXACT>(fadd<EXACT>(a, fadd<EXACT>(u, u)), q);
    if (!in_shell(c, n, p)) {
        if (p.mask && masked(c, n, p)) f = 0.f;
        f = damp_a<EXACT>(f, si, p.dtab, p.ftab);
    }
    nxt[i] = f;
}

// Spherical step, AWE_FAST: each thread owns one (r, theta) column and marches
// along phi through a chunk of planes.  The phi neighbours stay in registers,
// the per-radius and per-(theta, r) metric tables are read once per column,
// and the r / theta neighbours come through L1 from the lanes and warps that
// load the same plane.  Same formula and operation order as k_stepA<3>,
// with fused multiply-adds and reciprocal multiplies.
constexpr int kSphChunk = 16;

// prv: the previous level (the same buffer as nxt for the in-place step)
__global__ void __launch_bounds__(256) k_stepA_sph_march(const float *__restrict__ cur, const float *prv, float *nxt,
                                                         const float *__restrict__ vel, const StepAParams p) {
    const int i1 = blockIdx.x * blockDim.x + threadIdx.x;
    const int i2 = blockIdx.y * blockDim.y + threadIdx.y;
    const Grid g = p.g;
    if (i1 >= g.n1 || i2 >= g.n2) return;
    const int n[3] = {g.n1, g.n2, g.n3};
    const long long s2 = g.n1, s3 = (long long)g.n1 * g.n2;
    const int p0 = blockIdx.z * kSphChunk, p1 = min(p0 + kSphChunk, g.n3);
    const bool in12 = i1 >= 4 && i1 < g.n1 - 4 && i2 >= 4 && i2 < g.n2 - 4;
    const long long t = (long long)i2 * g.n1 + i1;
    const float A2 = __ldg(p.tr0 + i1), Cr = __ldg(p.tr1 + i1), B = __ldg(p.tt0 + t), D = __ldg(p.tt1 + t);
    const long long base = (long long)i2 * s2 + i1;
    float um = p0 > 0 ? cur[base + (p0 - 1) * s3] : 0.f;
    float uc = cur[base + p0 * s3];
    for (int i3 = p0; i3 < p1; i3++) {
        const long long i = base + i3 * s3;
        const float up = i3 + 1 < g.n3 ? cur[i + s3] : 0.f;
        const int c[3] = {i1, i2, i3};
        const int si = sponge_index(c, n, p);
        const float q = damp_a<false>(prv[i], si, p.dtab, p.ftab);
        float lap = 0.f;
        if (in12 && i3 >= 4 && i3 < g.n3 - 4) {
            const float u2 = uc + uc;
            const float rm = cur[i - 1], rp = cur[i + 1], tm = cur[i - s2], tp = cur[i + s2];
            const float pra = (rp - rm) * p.rd[0];
            const float ppra = ((rp - u2) + rm) * p.rd[1];
            const float pth = (tp - tm) * p.rd[2];
            const float ppth = ((tp - u2) + tm) * p.rd[3];
            const float ppph = ((up - u2) + um) * p.rd[4];
            lap = fmaf(A2, pra, ppra);
            lap = fmaf(B, pth, lap);
            lap = fmaf(Cr, ppth, lap);
            lap = fmaf(D, ppph, lap);
        }
        const float v = __ldg(vel + i);
        float f = fmaf(p.dt2 * (v * v), lap, uc + uc) - q;
        if (!in_shell(c, n, p)) {
            if (p.mask && masked(c, n, p)) f = 0.f;
            f = damp_a<false>(f, si, p.dtab, p.ftab);
        }
        nxt[i] = f;
        um = uc;
        uc = up;
    }
}

// sponge_index for a 3D grid with the coordinates in registers (no indexed
// arrays): the all-interior case first, then the priority walk
__device__ __forceinline__ int sel3(int a, int v0, int v1, int v2) { return a == 0 ? v0 : (a == 1 ? v1 : v2); }

__device__ __forceinline__ int sponge_index3(int c0, int c1, int c2, int n0, int n1, int n2, const StepAParams &p) {
    const int nb = p.nb;
    if (c0 >= nb && c0 <= n0 - nb && c1 >= nb && c1 <= n1 - nb && c2 >= nb && c2 <= n2 - nb) return 0;
    const bool low = c0 < nb || c1 < nb || c2 < nb;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int a = p.pri[k];
        const int c = sel3(a, c0, c1, c2), n = sel3(a, n0, n1, n2);
        if (low) {
            if (c < nb) return nb - c;
        }
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int a = p.pri[k];
        const int c = sel3(a, c0, c1, c2), n = sel3(a, n0, n1, n2);
        if (!low && c > n - nb) return c - (n - nb);
    }
    return 0;
}

// The same march with two consecutive radii per thread (n1 even): 8-byte
// loads and packed FP32x2 arithmetic (fma.rn.f32x2 / add.f32x2 / mul.f32x2).
__global__ void __launch_bounds__(256) k_stepA_sph_march2(const float *__restrict__ cur, const float *prv, float *nxt,
                                                          const float *__restrict__ vel, const StepAParams p) {
    // (the shot offset below is applied to cur and nxt, never to the shared model)
    const int i1 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int i2 = blockIdx.y * blockDim.y + threadIdx.y;
    const Grid g = p.g;
    if (i1 >= g.n1 || i2 >= g.n2) return;
    const long long s2 = g.n1, s3 = (long long)g.n1 * g.n2;
    // blockIdx.z enumerates (shot, phi chunk); shots' fields lie back to back
    const int nchunk = (g.n3 + kSphChunk - 1) / kSphChunk;
    const int shot = blockIdx.z / nchunk;
    cur += shot * p.shot_cells;
    prv += shot * p.shot_cells;
    nxt += shot * p.shot_cells;
    const int p0 = (blockIdx.z % nchunk) * kSphChunk, p1 = min(p0 + kSphChunk, g.n3);
    const bool th_in = i2 >= 4 && i2 < g.n2 - 4;
    const bool r0_in = i1 >= 4 && i1 < g.n1 - 4, r1_in = i1 + 1 >= 4 && i1 + 1 < g.n1 - 4;
    const long long t = (long long)i2 * g.n1 + i1;
    const float2 A2 = *reinterpret_cast<const float2 *>(p.tr0 + i1), Cr = *reinterpret_cast<const float2 *>(p.tr1 + i1);
    const float2 B = *reinterpret_cast<const float2 *>(p.tt0 + t), D = *reinterpret_cast<const float2 *>(p.tt1 + t);
    const float2 r0 = make_float2(p.rd[0], p.rd[0]), r1 = make_float2(p.rd[1], p.rd[1]);
    const float2 r2 = make_float2(p.rd[2], p.rd[2]), r3 = make_float2(p.rd[3], p.rd[3]);
    const float2 r4 = make_float2(p.rd[4], p.rd[4]), m1 = make_float2(-1.f, -1.f), m2 = make_float2(-2.f, -2.f);
    const long long base = (long long)i2 * s2 + i1;
    auto ld2 = [&](long long j) { return *reinterpret_cast<const float2 *>(cur + j); };
    float2 um = p0 > 0 ? ld2(base + (p0 - 1) * s3) : make_float2(0.f, 0.f);
    float2 uc = ld2(base + p0 * s3);
    for (int i3 = p0; i3 < p1; i3++) {
        const long long i = base + i3 * s3;
        const float2 up = i3 + 1 < g.n3 ? ld2(i + s3) : make_float2(0.f, 0.f);
        const float2 pv = *reinterpret_cast<const float2 *>(prv + i);
        const float2 vv = *reinterpret_cast<const float2 *>(vel + i);
        float2 lap = make_float2(0.f, 0.f);
        const bool ph_in = i3 >= 4 && i3 < g.n3 - 4;
        if (th_in && ph_in && (r0_in || r1_in)) {
            const float rm = i1 > 0 ? cur[i - 1] : 0.f, rp = i1 + 2 < g.n1 ? cur[i + 2] : 0.f;
            const float2 mi = make_float2(rm, uc.x), pl = make_float2(uc.y, rp);  // r - 1 and r + 1 of both cells
            const float2 tm = ld2(i - s2), tp = ld2(i + s2);
            const float2 pra = __fmul2_rn(__ffma2_rn(mi, m1, pl), r0);
            const float2 ppra = __fmul2_rn(__fadd2_rn(__ffma2_rn(uc, m2, pl), mi), r1);
            const float2 pth = __fmul2_rn(__ffma2_rn(tm, m1, tp), r2);
            const float2 ppth = __fmul2_rn(__fadd2_rn(__ffma2_rn(uc, m2, tp), tm), r3);
            const float2 ppph = __fmul2_rn(__fadd2_rn(__ffma2_rn(uc, m2, up), um), r4);
            lap = __ffma2_rn(A2, pra, ppra);
            lap = __ffma2_rn(B, pth, lap);
            lap = __ffma2_rn(Cr, ppth, lap);
            lap = __ffma2_rn(D, ppph, lap);
            if (!r0_in) lap.x = 0.f;
            if (!r1_in) lap.y = 0.f;
        }
        const float2 a = __fmul2_rn(make_float2(p.dt2, p.dt2), __fmul2_rn(vv, vv));
        const float2 f2 = __ffma2_rn(a, lap, __fadd2_rn(uc, uc));
        float f[2] = {f2.x, f2.y};
        const float pr[2] = {pv.x, pv.y};
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int si = sponge_index3(i1 + j, i2, i3, g.n1, g.n2, g.n3, p);
            float v = f[j] - damp_a<false>(pr[j], si, p.dtab, p.ftab);
            // the spherical program has no one-way boundary (no shell); free-surface mask
            if (p.mask == 3 && (i1 + j > g.n1 - p.nb || (i1 + j < p.spill && (i2 >= 1 || i3 >= 1)))) v = 0.f;
            f[j] = damp_a<false>(v, si, p.dtab, p.ftab);
        }
        *reinterpret_cast<float2 *>(nxt + i) = make_float2(f[0], f[1]);
        um = uc;
        uc = up;
    }
}

template <bool EXACT>
static void step_geom(int geom, const float *cur, const float *prv, float *nxt, const float *vel, const StepAParams &p,
                      cudaStream_t s) {
    dim3 block(64, 4, 1), grid((p.g.n1 + 63) / 64, (p.g.n2 + 3) / 4, p.g.n3);
    if (!EXACT && geom == 3) {
        if (p.g.n1 % 2 == 0) {
            const int nchunk = (p.g.n3 + kSphChunk - 1) / kSphChunk;
            dim3 b2(32, 8, 1), g2((p.g.n1 / 2 + 31) / 32, (p.g.n2 + 7) / 8, nchunk * (p.nshot > 0 ? p.nshot : 1));
            k_stepA_sph_march2<<<g2, b2, 0, s>>>(cur, prv, nxt, vel, p);
        } else {
            dim3 mg((p.g.n1 + 63) / 64, (p.g.n2 + 3) / 4, (p.g.n3 + kSphChunk - 1) / kSphChunk);
            k_stepA_sph_march<<<mg, block, 0, s>>>(cur, prv, nxt, vel, p);
        }
        return;
    }
    switch (geom) {
        case 0: k_stepA<0, EXACT><<<grid, block, 0, s>>>(cur, nxt, vel, p); break;
        case 1: k_stepA<1, EXACT><<<grid, block, 0, s>>>(cur, nxt, vel, p); break;
        case 2: k_stepA<2, EXACT><<<grid, block, 0, s>>>(cur, nxt, vel, p); break;
        default: k_stepA<3, EXACT><<<grid, block, 0, s>>>(cur, nxt, vel, p); break;
    }
}

void launch_stepA(int geom, bool exact, const float *cur, float *nxt, const float *vel, const StepAParams &p,
                  cudaStream_t s) {
    if (exact) step_geom<true>(geom, cur, nxt, nxt, vel, p, s);
    else step_geom<false>(geom, cur, nxt, nxt, vel, p, s);
}

bool stepA_out_of_place(int geom, bool exact) { return geom == 3 && !exact; }

void launch_stepA_oop(int geom, bool exact, const float *cur, const float *prv, float *out, const float *vel,
                      const StepAParams &p, cudaStream_t s) {
    if (stepA_out_of_place(geom, exact)) step_geom<false>(geom, cur, prv, out, vel, p, s);
}

// ---------------------------------------------------------------------------
// One-way boundary, phase 1: boundary values from the unmodified fields.
// um = the level that just became "previous" (before its sponge), uo = the
// new level as stored by the step kernel (unsponged inside the shell).
template <bool EXACT>
__device__ __forceinline__ float oneway(float um_n, float um_c, float uo_n, float b) {
    return fadd<EXACT>(um_n, fmul<EXACT>(fsub<EXACT>(um_c, uo_n), b));
}

// 2D programs: rows 1..4 and n-5..n-2 of the swept axis, read from the last
// sample of the other axis (the reference kernel's loop leaves that one).
// geom 0: swept axis z (axis 1), other axis x (axis 2), rows limited to < nxpad
// geom 2: swept axis theta (axis 2), other axis r (axis 1)
template <bool EXACT>
__global__ void k_bcA2_phase1(const float *__restrict__ um, const float *__restrict__ uo, float *__restrict__ aux,
                              const StepAParams p) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const Grid g = p.g;
    const bool cart = p.geom == 0;
    const int nsw = cart ? g.n1 : g.n2, noth = cart ? g.n2 : g.n1;
    if (t >= 8 * noth) return;
    const int k = t / noth, o = t % noth;  // k: 0..3 top rows 1..4, 4..7 bottom rows n-5..n-2
    const int row = k < 4 ? 1 + k : nsw - 5 + (k - 4);
    if (cart && row >= g.n2) return;  // the kernel's `iz < nxpad` test
    auto at = [&](int r, int oo) -> long long {
        return cart ? (long long)oo * g.n1 + r : (long long)r * g.n1 + oo;
    };
    const int nbr = k < 4 ? row + 1 : row - 1;
    const float b = k < 4 ? p.b2lo : p.b2hi;
    aux[at(row, o)] = oneway<EXACT>(um[at(nbr, noth - 1)], um[at(row, o)], uo[at(nbr, noth - 1)], b);
}

// cart 3D (onewayBC_3D): cells within 4 (low) / 5 (high) of a face; the last
// applicable face formula wins; neighbours read masked (z < nb zeroed).
template <bool EXACT>
__global__ void k_bcA3_phase1(const float *__restrict__ um, const float *__restrict__ uo, float *__restrict__ aux,
                              const StepAParams p) {
    const int i1 = blockIdx.x * blockDim.x + threadIdx.x;  // z
    const int i2 = blockIdx.y, i3 = blockIdx.z;           // x, y
    const Grid g = p.g;
    if (i1 >= g.n1) return;
    const int iz = i1, ix = i2, iy = i3;
    const bool zl = iz <= 4, zh = iz >= g.n1 - 5, xl = ix <= 4, xh = ix >= g.n2 - 5, yl = iy <= 4, yh = iy >= g.n3 - 5;
    if (!(zl || zh || xl || xh || yl || yh)) return;
    const long long s2 = g.n1, s3 = (long long)g.n1 * g.n2, c = iy * s3 + ix * s2 + iz;
    auto ps = [&](long long n, int nz) { return nz < p.nb ? 0.f : uo[n]; };  // freeSurf_3D before the boundary
    const int nx = g.n2, nz = g.n1;
    float val = 0.f;
    if (zl) val = oneway<EXACT>(um[c + 1], um[c], ps(c + 1, iz + 1), p.tb[0][iy * nx + ix]);
    if (zh) val = oneway<EXACT>(um[c - 1], um[c], ps(c - 1, iz - 1), p.tb[1][iy * nx + ix]);
    if (xl) val = oneway<EXACT>(um[c + s2], um[c], ps(c + s2, iz), p.tb[2][iy * nz + iz]);
    if (xh) val = oneway<EXACT>(um[c - s2], um[c], ps(c - s2, iz), p.tb[1][iy * nz + iz]);  // the z-high table, as the reference
    if (yl) val = oneway<EXACT>(um[c + s3], um[c], ps(c + s3, iz), p.tb[4][iz * nx + ix]);
    if (yh) val = oneway<EXACT>(um[c - s3], um[c], ps(c - s3, iz), p.tb[5][iz * nx + ix]);
    aux[c] = val;
}

// phase 2: every shell cell gets its final value: the boundary value where
// the boundary applies, else the (masked) new level; then sponge and masks.
template <bool EXACT>
__global__ void k_bcA_phase2(float *__restrict__ uo, const float *__restrict__ aux, const StepAParams p) {
    const int i1 = blockIdx.x * blockDim.x + threadIdx.x;
    const int i2 = blockIdx.y, i3 = blockIdx.z;
    const Grid g = p.g;
    if (i1 >= g.n1) return;
    const int c[3] = {i1, i2, i3}, n[3] = {g.n1, g.n2, g.n3};
    if (!in_shell(c, n, p)) return;
    const long long i = ((long long)i3 * g.n2 + i2) * g.n1 + i1;
    bool bc;
    if (p.geom == 0) bc = ((i1 >= 1 && i1 <= 4) || (i1 >= g.n1 - 5 && i1 <= g.n1 - 2)) && i1 < g.n2;
    else if (p.geom == 2) bc = (i2 >= 1 && i2 <= 4) || (i2 >= g.n2 - 5 && i2 <= g.n2 - 2);
    else bc = i1 <= 4 || i1 >= g.n1 - 5 || i2 <= 4 || i2 >= g.n2 - 5 || i3 <= 4 || i3 >= g.n3 - 5;
    float v = uo[i];
    if (p.geom == 1 && masked(c, n, p)) v = 0.f;  // cart 3D: free surface before the boundary
    if (bc) v = aux[i];
    v = damp_a<EXACT>(v, sponge_index(c, n, p), p.dtab, p.ftab);
    if (p.geom != 1 && p.mask && masked(c, n, p)) v = 0.f;  // 2D programs: free surface after the sponge
    uo[i] = v;
}

void launch_bcA(bool exact, const float *um, float *uo, float *aux, const StepAParams &p, cudaStream_t s) {
    const Grid &g = p.g;
    const int T = 128;
    if (p.geom == 0 || p.geom == 2) {
        const int noth = p.geom == 0 ? g.n2 : g.n1;
        const int n = 8 * noth;
        if (exact) k_bcA2_phase1<true><<<(n + T - 1) / T, T, 0, s>>>(um, uo, aux, p);
        else k_bcA2_phase1<false><<<(n + T - 1) / T, T, 0, s>>>(um, uo, aux, p);
    } else {
        dim3 grid((g.n1 + T - 1) / T, g.n2, g.n3);
        if (exact) k_bcA3_phase1<true><<<grid, T, 0, s>>>(um, uo, aux, p);
        else k_bcA3_phase1<false><<<grid, T, 0, s>>>(um, uo, aux, p);
    }
    dim3 grid2((g.n1 + T - 1) / T, g.n2, g.n3);
    if (exact) k_bcA_phase2<true><<<grid2, T, 0, s>>>(uo, aux, p);
    else k_bcA_phase2<false><<<grid2, T, 0, s>>>(uo, aux, p);
}

// ---------------------------------------------------------------------------
// Injection into the current level before the update
// (inject_sources_{2D,3D}{_const,,_refl}): u[node] += (wa * w) [* scale],
// sources and corners in order; the per-corner scale (reflectivity) is
// constant over time and prepared on the host.
template <bool EXACT>
__global__ void k_injectA(float *u, const GeoPoint *__restrict__ pts, const float *__restrict__ scale, int ns,
                          const float *__restrict__ wav, int it, int ncs, int ncorner, int scaled,
                          const long long *__restrict__ off, int stride) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int s = 0; s < ns; s++) {
        // one wavelet for every source (ncs = 1), or one per source (the
        // back-injected traces of sfAWEFDspher3Dgpu adj=y, row it of [nt][ns])
        const float wa = wav[(long long)it * ncs + (ncs == 1 ? 0 : s)];
        const GeoPoint pt = pts[(long long)s * stride];
        for (int c = 0; c < ncorner; c++) {
            const long long n = pt.base + off[c];
            float a = fmul<EXACT>(wa, pt.w[c]);
            if (scaled) a = fmul<EXACT>(a, scale[s * 8 + c]);
            u[n] = fadd<EXACT>(u[n], a);
        }
    }
}

void launch_injectA(bool exact, int ndim, float *u, const GeoPoint *pts, const float *scale, int ns, const float *wav,
                    int it, bool scaled, const long long *off, cudaStream_t s, int stride, int ncs) {
    if (ns <= 0) return;
    const int nc = ndim == 3 ? 8 : 4;
    if (exact) k_injectA<true><<<1, 32, 0, s>>>(u, pts, scale, ns, wav, it, ncs, nc, scaled, off, stride);
    else k_injectA<false><<<1, 32, 0, s>>>(u, pts, scale, ns, wav, it, ncs, nc, scaled, off, stride);
}

// polar snapshots are theta-fastest ([r][theta]) as sfAWEFDspher2Dgpu writes them
__global__ void k_snapshot_transpose2(const float *__restrict__ u, float *__restrict__ dst, Grid g, int f1, int f2,
                                      int m1, int m2) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m1 * m2) return;
    const int j2 = (int)(t % m2), j1 = (int)(t / m2);  // dst[j1][j2], j2 (theta) fastest
    dst[t] = u[(long long)(f2 + j2) * g.n1 + (f1 + j1)];
}

void launch_snapshot_transpose2(const float *u, float *dst, const Grid &g, int f1, int f2, int m1, int m2,
                                cudaStream_t s) {
    const long long n = (long long)m1 * m2;
    k_snapshot_transpose2<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(u, dst, g, f1, f2, m1, m2);
}

// ---------------------------------------------------------------------------
// Adjoint of the spherical step (AWE_FAST).  The forward map of one step is
//   U_{k+1} = W M (c L A_k + 2 A_k - W A_{k-1}),   c = dt^2 v^2,
// A_k the current level after the injection, L the metric Laplacian on the
// interior (zero in the 4-cell ring), W the sponge factor, M the free-surface
// mask.  Its transpose, with X = z_{j+1} and Y = z_{j+2}:
//   Y <- z_j = W M (L^T (I c X) + 2 X - W Y)
//   G += X L(A_j) on the interior (A == nullptr: no gradient term).
// L is not symmetric: each neighbour n of the cell contributes I c X at n
// times the weight of this cell in n's stencil, so the r neighbours use their
// own 2/r and the theta neighbours their own cos/(r^2 sin).  One thread per
// (r, theta) column marching a chunk of phi; the phi neighbours of I c X and
// of A stay in registers.
__global__ void __launch_bounds__(256) k_adjA_sph(const float *__restrict__ X, float *__restrict__ Y,
                                                  const float *__restrict__ A, const float *__restrict__ vel,
                                                  float2 *__restrict__ G, const StepAParams p, int xcorr) {
    const int i1 = blockIdx.x * blockDim.x + threadIdx.x;
    const int i2 = blockIdx.y * blockDim.y + threadIdx.y;
    const Grid g = p.g;
    if (i1 >= g.n1 || i2 >= g.n2) return;
    const long long s2 = g.n1, s3 = (long long)g.n1 * g.n2;
    const int p0 = blockIdx.z * kSphChunk, p1 = min(p0 + kSphChunk, g.n3);
    auto rin = [&](int r) { return r >= 4 && r < g.n1 - 4; };
    auto tin = [&](int t) { return t >= 4 && t < g.n2 - 4; };
    auto pin = [&](int f) { return f >= 4 && f < g.n3 - 4; };
    const bool c_in = rin(i1) && tin(i2);
    const bool rm_in = rin(i1 - 1) && tin(i2), rp_in = rin(i1 + 1) && tin(i2);
    const bool tm_in = rin(i1) && tin(i2 - 1), tp_in = rin(i1) && tin(i2 + 1);
    const long long t = (long long)i2 * g.n1 + i1;
    const float rd0 = p.rd[0], rd1 = p.rd[1], rd2 = p.rd[2], rd3 = p.rd[3], rd4 = p.rd[4];
    const float A2 = __ldg(p.tr0 + i1), Cr = __ldg(p.tr1 + i1), B = __ldg(p.tt0 + t), D = __ldg(p.tt1 + t);
    // this cell's weight in each neighbour's stencil (0 where the neighbour has no stencil)
    const float w_rm = rm_in ? fmaf(__ldg(p.tr0 + i1 - 1), rd0, rd1) : 0.f;
    const float w_rp = rp_in ? fmaf(-__ldg(p.tr0 + i1 + 1), rd0, rd1) : 0.f;
    const float w_tm = tm_in ? fmaf(__ldg(p.tt0 + t - s2), rd2, Cr * rd3) : 0.f;
    const float w_tp = tp_in ? fmaf(-__ldg(p.tt0 + t + s2), rd2, Cr * rd3) : 0.f;
    const float w_c = -2.f * (rd1 + Cr * rd3 + D * rd4), w_ph = D * rd4;
    const float dt2 = p.dt2;
    auto ycx = [&](long long j) {  // c X at cell j
        const float v = __ldg(vel + j);
        return (dt2 * (v * v)) * X[j];
    };
    const long long base = (long long)i2 * s2 + i1;
    // phi - 1 and phi of I c X and A for the column
    float ym = (p0 > 0 && c_in && pin(p0 - 1)) ? ycx(base + (p0 - 1) * s3) : 0.f;
    float yc = (c_in && pin(p0)) ? ycx(base + p0 * s3) : 0.f;
    float am = 0.f, ac = 0.f;
    if (A) {
        am = p0 > 0 ? A[base + (p0 - 1) * s3] : 0.f;
        ac = A[base + p0 * s3];
    }
    for (int i3 = p0; i3 < p1; i3++) {
        const long long i = base + i3 * s3;
        const bool ph = pin(i3);
        const float yp = (i3 + 1 < g.n3 && c_in && pin(i3 + 1)) ? ycx(i + s3) : 0.f;
        const float ap = (A && i3 + 1 < g.n3) ? A[i + s3] : 0.f;
        float lt = w_ph * (ym + yp);
        if (ph) {
            lt = fmaf(w_c, yc, lt);
            if (rm_in) lt = fmaf(w_rm, ycx(i - 1), lt);
            if (rp_in) lt = fmaf(w_rp, ycx(i + 1), lt);
            if (tm_in) lt = fmaf(w_tm, ycx(i - s2), lt);
            if (tp_in) lt = fmaf(w_tp, ycx(i + s2), lt);
        }
        const float xc = X[i];
        const int si = sponge_index3(i1, i2, i3, g.n1, g.n2, g.n3, p);
        const float yv = Y[i];
        float mu = fmaf(-damp_a<false>(1.f, si, p.dtab, p.ftab), yv, fmaf(2.f, xc, lt));
        if (p.mask == 3 && (i1 > g.n1 - p.nb || (i1 < p.spill && (i2 >= 1 || i3 >= 1)))) mu = 0.f;
        Y[i] = damp_a<false>(mu, si, p.dtab, p.ftab);
        if (A && c_in && ph && xcorr) {
            G[i] = gsum_add(G[i], __fmul_rn(xc, ac));  // zero-lag cross-correlation image
        } else if (A && c_in && ph) {  // the forward's Laplacian of A at this cell
            const float u2 = ac + ac;
            const float rm = A[i - 1], rp = A[i + 1], tm = A[i - s2], tp = A[i + s2];
            const float pra = (rp - rm) * rd0;
            const float ppra = ((rp - u2) + rm) * rd1;
            const float pth = (tp - tm) * rd2;
            const float ppth = ((tp - u2) + tm) * rd3;
            const float ppph = ((ap - u2) + am) * rd4;
            float lap = fmaf(A2, pra, ppra);
            lap = fmaf(B, pth, lap);
            lap = fmaf(Cr, ppth, lap);
            lap = fmaf(D, ppph, lap);
            G[i] = gsum_add(G[i], __fmul_rn(xc, lap));
        }
        ym = yc;
        yc = yp;
        am = ac;
        ac = ap;
    }
}

// The same adjoint with two consecutive radii per thread (n1 even): 8-byte
// loads and packed FP32x2 arithmetic; the r neighbours outside the pair come
// from scalar loads, those inside it from the thread's own cells.
__global__ void __launch_bounds__(256) k_adjA_sph2(const float *__restrict__ X, float *__restrict__ Y,
                                                   const float *__restrict__ A, const float *__restrict__ vel,
                                                   float2 *__restrict__ G, const StepAParams p, int xcorr) {
    const int i1 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int i2 = blockIdx.y * blockDim.y + threadIdx.y;
    const Grid g = p.g;
    if (i1 >= g.n1 || i2 >= g.n2) return;
    const long long s2 = g.n1, s3 = (long long)g.n1 * g.n2;
    const int p0 = blockIdx.z * kSphChunk, p1 = min(p0 + kSphChunk, g.n3);
    auto rin = [&](int r) { return r >= 4 && r < g.n1 - 4; };
    auto pin = [&](int f) { return f >= 4 && f < g.n3 - 4; };
    const bool t_in = i2 >= 4 && i2 < g.n2 - 4;
    const bool tm_ok = i2 - 1 >= 4 && i2 - 1 < g.n2 - 4, tp_ok = i2 + 1 >= 4 && i2 + 1 < g.n2 - 4;
    const bool r0 = rin(i1), r1 = rin(i1 + 1);
    const bool c0 = r0 && t_in, c1 = r1 && t_in;
    const long long t = (long long)i2 * g.n1 + i1;
    const float rd0 = p.rd[0], rd1 = p.rd[1], rd2 = p.rd[2], rd3 = p.rd[3], rd4 = p.rd[4];
    const float2 A2 = *reinterpret_cast<const float2 *>(p.tr0 + i1), Cr = *reinterpret_cast<const float2 *>(p.tr1 + i1);
    const float2 B = *reinterpret_cast<const float2 *>(p.tt0 + t), D = *reinterpret_cast<const float2 *>(p.tt1 + t);
    // weights of the two cells in their neighbours' stencils (0: no stencil there)
    // r - 1: cell 0's neighbour i1 - 1 (outside the pair), cell 1's is cell 0
    const float wrm0 = (rin(i1 - 1) && t_in) ? fmaf(__ldg(p.tr0 + i1 - 1), rd0, rd1) : 0.f;
    const float wrm1 = c0 ? fmaf(A2.x, rd0, rd1) : 0.f;
    // r + 1: cell 0's neighbour is cell 1, cell 1's is i1 + 2 (outside)
    const float wrp0 = c1 ? fmaf(-A2.y, rd0, rd1) : 0.f;
    const float wrp1 = (rin(i1 + 2) && t_in) ? fmaf(-__ldg(p.tr0 + i1 + 2), rd0, rd1) : 0.f;
    float2 wtm = make_float2(0.f, 0.f), wtp = wtm;
    if (tm_ok) {
        const float2 Bm = *reinterpret_cast<const float2 *>(p.tt0 + t - s2);
        wtm = make_float2(r0 ? fmaf(Bm.x, rd2, Cr.x * rd3) : 0.f, r1 ? fmaf(Bm.y, rd2, Cr.y * rd3) : 0.f);
    }
    if (tp_ok) {
        const float2 Bp = *reinterpret_cast<const float2 *>(p.tt0 + t + s2);
        wtp = make_float2(r0 ? fmaf(-Bp.x, rd2, Cr.x * rd3) : 0.f, r1 ? fmaf(-Bp.y, rd2, Cr.y * rd3) : 0.f);
    }
    const float2 wc = make_float2(-2.f * (rd1 + Cr.x * rd3 + D.x * rd4), -2.f * (rd1 + Cr.y * rd3 + D.y * rd4));
    const float2 wph = make_float2(D.x * rd4, D.y * rd4);
    const float dt2 = p.dt2;
    const float2 dt22 = make_float2(dt2, dt2);
    auto ld2 = [](const float *b, long long j) { return *reinterpret_cast<const float2 *>(b + j); };
    auto ycx2 = [&](long long j) {  // c X at cells j, j + 1
        const float2 v = ld2(vel, j);
        return __fmul2_rn(__fmul2_rn(dt22, __fmul2_rn(v, v)), ld2(X, j));
    };
    auto ycx1 = [&](long long j) {
        const float v = __ldg(vel + j);
        return (dt2 * (v * v)) * X[j];
    };
    auto own = [&](float2 y, int f) {  // I c X of the own cells at plane f
        const bool ph = f >= 0 && f < g.n3 && pin(f);
        return make_float2(c0 && ph ? y.x : 0.f, c1 && ph ? y.y : 0.f);
    };
    const long long base = (long long)i2 * s2 + i1;
    float2 ym = p0 > 0 ? own(ycx2(base + (p0 - 1) * s3), p0 - 1) : make_float2(0.f, 0.f);
    float2 yc = own(ycx2(base + p0 * s3), p0);
    float2 am = make_float2(0.f, 0.f), ac = am;
    if (A) {
        am = p0 > 0 ? ld2(A, base + (p0 - 1) * s3) : am;
        ac = ld2(A, base + p0 * s3);
    }
    const float2 r0v = make_float2(rd0, rd0), r1v = make_float2(rd1, rd1), r2v = make_float2(rd2, rd2);
    const float2 r3v = make_float2(rd3, rd3), r4v = make_float2(rd4, rd4), m1 = make_float2(-1.f, -1.f),
                 m2 = make_float2(-2.f, -2.f);
    for (int i3 = p0; i3 < p1; i3++) {
        const long long i = base + i3 * s3;
        const bool ph = pin(i3);
        const float2 yp = i3 + 1 < g.n3 ? own(ycx2(i + s3), i3 + 1) : make_float2(0.f, 0.f);
        const float2 ap = (A && i3 + 1 < g.n3) ? ld2(A, i + s3) : make_float2(0.f, 0.f);
        float2 lt = __fmul2_rn(wph, __fadd2_rn(ym, yp));
        if (ph) {
            lt = __ffma2_rn(wc, yc, lt);
            const float yrm = wrm0 != 0.f ? ycx1(i - 1) : 0.f, yrp = wrp1 != 0.f ? ycx1(i + 2) : 0.f;
            lt = __ffma2_rn(make_float2(wrm0, wrm1), make_float2(yrm, yc.x), lt);
            lt = __ffma2_rn(make_float2(wrp0, wrp1), make_float2(yc.y, yrp), lt);
            if (tm_ok) lt = __ffma2_rn(wtm, ycx2(i - s2), lt);
            if (tp_ok) lt = __ffma2_rn(wtp, ycx2(i + s2), lt);
        }
        const float2 xc = ld2(X, i), yv = ld2(Y, i);
        const float2 mu2 = __ffma2_rn(make_float2(2.f, 2.f), xc, lt);
        float out[2] = {mu2.x, mu2.y};
        const float yy[2] = {yv.x, yv.y};
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int si = sponge_index3(i1 + j, i2, i3, g.n1, g.n2, g.n3, p);
            float m = fmaf(-damp_a<false>(1.f, si, p.dtab, p.ftab), yy[j], out[j]);
            if (p.mask == 3 && (i1 + j > g.n1 - p.nb || (i1 + j < p.spill && (i2 >= 1 || i3 >= 1)))) m = 0.f;
            out[j] = damp_a<false>(m, si, p.dtab, p.ftab);
        }
        *reinterpret_cast<float2 *>(Y + i) = make_float2(out[0], out[1]);
        if (A && (c0 || c1) && ph && xcorr) {  // zero-lag cross-correlation image
            const float4 gq = *reinterpret_cast<const float4 *>(G + i);
            float2 g0 = make_float2(gq.x, gq.y), g1 = make_float2(gq.z, gq.w);
            if (c0) g0 = gsum_add(g0, __fmul_rn(xc.x, ac.x));
            if (c1) g1 = gsum_add(g1, __fmul_rn(xc.y, ac.y));
            *reinterpret_cast<float4 *>(G + i) = make_float4(g0.x, g0.y, g1.x, g1.y);
        } else if (A && (c0 || c1) && ph) {  // the forward's Laplacian of A at the two cells
            const float rm = A[i - 1], rp = A[i + 2];
            const float2 mi = make_float2(rm, ac.x), pl = make_float2(ac.y, rp);
            const float2 tm = ld2(A, i - s2), tp = ld2(A, i + s2);
            const float2 pra = __fmul2_rn(__ffma2_rn(mi, m1, pl), r0v);
            const float2 ppra = __fmul2_rn(__fadd2_rn(__ffma2_rn(ac, m2, pl), mi), r1v);
            const float2 pth = __fmul2_rn(__ffma2_rn(tm, m1, tp), r2v);
            const float2 ppth = __fmul2_rn(__fadd2_rn(__ffma2_rn(ac, m2, tp), tm), r3v);
            const float2 ppph = __fmul2_rn(__fadd2_rn(__ffma2_rn(ac, m2, ap), am), r4v);
            float2 lap = __ffma2_rn(A2, pra, ppra);
            lap = __ffma2_rn(B, pth, lap);
            lap = __ffma2_rn(Cr, ppth, lap);
            lap = __ffma2_rn(D, ppph, lap);
            const float4 gq = *reinterpret_cast<const float4 *>(G + i);
            float2 g0 = make_float2(gq.x, gq.y), g1 = make_float2(gq.z, gq.w);
            if (c0) g0 = gsum_add(g0, __fmul_rn(xc.x, lap.x));
            if (c1) g1 = gsum_add(g1, __fmul_rn(xc.y, lap.y));
            *reinterpret_cast<float4 *>(G + i) = make_float4(g0.x, g0.y, g1.x, g1.y);
        }
        ym = yc;
        yc = yp;
        am = ac;
        ac = ap;
    }
}

void launch_adjA_sph(const float *X, float *Y, const float *A, const float *vel, float2 *G, const StepAParams &p,
                     cudaStream_t s, bool xcorr) {
    const int nchunk = (p.g.n3 + kSphChunk - 1) / kSphChunk;
    if (p.g.n1 % 2 == 0) {
        dim3 b2(32, 8, 1), g2((p.g.n1 / 2 + 31) / 32, (p.g.n2 + 7) / 8, nchunk);
        k_adjA_sph2<<<g2, b2, 0, s>>>(X, Y, A, vel, G, p, xcorr ? 1 : 0);
        return;
    }
    dim3 block(64, 4, 1), grid((p.g.n1 + 63) / 64, (p.g.n2 + 3) / 4, nchunk);
    k_adjA_sph<<<grid, block, 0, s>>>(X, Y, A, vel, G, p, xcorr ? 1 : 0);
}

// receiver term of the spherical adjoint: z += W M (w r) at every corner
__global__ void k_rec_adjA(float *z, const GeoPoint *__restrict__ pts, int nr, const float *__restrict__ r,
                           const StepAParams p, const long long *__restrict__ off) {
    const int ir = blockIdx.x * blockDim.x + threadIdx.x;
    if (ir >= nr) return;
    const GeoPoint pt = pts[ir];
    const float rv = r[ir];
    const Grid g = p.g;
    for (int k = 0; k < 8; k++) {
        const long long j = pt.base + off[k];
        const int c0 = (int)(j % g.n1), c1 = (int)((j / g.n1) % g.n2), c2 = (int)(j / ((long long)g.n1 * g.n2));
        if (p.mask == 3 && (c0 > g.n1 - p.nb || (c0 < p.spill && (c1 >= 1 || c2 >= 1)))) continue;
        const int si = sponge_index3(c0, c1, c2, g.n1, g.n2, g.n3, p);
        atomicAdd(z + j, damp_a<false>(pt.w[k] * rv, si, p.dtab, p.ftab));
    }
}

void launch_rec_adjA(float *z, const GeoPoint *pts, int nr, const float *r, const StepAParams &p, const long long *off,
                     cudaStream_t s) {
    if (nr > 0) k_rec_adjA<<<(nr + 127) / 128, 128, 0, s>>>(z, pts, nr, r, p, off);
}

}  // namespace awe
