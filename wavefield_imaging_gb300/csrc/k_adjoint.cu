// Adjoint of the CPU-program scheme's time step and the imaging-condition
// gradient accumulator (no counterpart in the reference, which has only the
// forward map of MAWEFDcart{2D,3D}cpu.c).
//
// Forward step k (V_k = level k after its own sponge; W = sponge factor, I =
// cells at least nop from every face, vel2 = v^2 dt^2):
//   N = I (2 V_k + vel2 L V_k - W V_{k-1}) + (1 - I) W V_{k-1} + S_k
//   N' = ABC(N; um = V_k)  (3D, abcone3d_apply),  V_{k+1} = W N'
//   d_k = R (W V_k)
// Adjoint step k, with mu = W lambda_{k+1} held in the buffer that becomes nu_k:
//   nu_k, kappa_k = ABC^T(mu)
//   lambda_k = 2 I nu_k + L(I vel2 nu_k) + kappa_k + W (1 - 2 I) nu_{k+1} + W R^T r_k
//   the new buffer holds mu_k = W lambda_k
//   dJ/dvel2 += I nu_k L(V_k)  (+ nu_k wav w at the source corners), summed per
//   cell as a compensated FP32 pair (gsum.cuh) and folded in FP64.
// The stencil is symmetric, so L^T is the same stencil applied to I vel2 nu.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "awe_internal.h"
#include "gsum.cuh"

namespace awe {

__device__ __forceinline__ float wcell(const AdjParams &p, int i1, int i2, int i3) {
    if (!p.w1) return 1.f;
    float w = __ldg(p.w1 + i1) * __ldg(p.w2 + i2);
    if (p.nd == 3) w *= __ldg(p.w3 + i3);
    return w;
}

template <int NOP, int NDIM>
__device__ __forceinline__ bool interior(const Grid &g, int i1, int i2, int i3) {
    bool in = i1 >= NOP && i1 < g.n1 - NOP && i2 >= NOP && i2 < g.n2 - NOP;
    if (NDIM == 3) in = in && i3 >= NOP && i3 < g.n3 - NOP;
    return in;
}

// main adjoint step, one thread per cell.  X = nu_k (stencil), Y = nu_{k+1}
// in / mu_k out (same cell only), V = V_k (stencil), G += I nu L(V) (compensated)
// (p.xcorr: G += I nu V, the cross-correlation imaging condition).
template <int NOP, int NDIM>
__global__ void __launch_bounds__(256) k_adjB(const float *__restrict__ X, float *__restrict__ Y,
                                              const float *__restrict__ V, const float *__restrict__ vel,
                                              float2 *__restrict__ G, const AdjParams p) {
    // programmatic dependent launch (2D): wait for the previous grid, then let the next be scheduled
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;");
    const int i1 = blockIdx.x * blockDim.x + threadIdx.x;
    const int i2 = blockIdx.y * blockDim.y + threadIdx.y;
    const int i3 = (NDIM == 3) ? (int)blockIdx.z : 0;
    const Grid g = p.g;
    if (i1 >= g.n1 || i2 >= g.n2) return;
    const long long s2 = g.n1, s3 = (long long)g.n1 * g.n2;
    const long long i = i3 * s3 + i2 * s2 + i1;
    const bool in = interior<NOP, NDIM>(g, i1, i2, i3);
    const float x = X[i];
    // L(I vel2 nu) at i: neighbours outside the interior (or the grid) contribute 0
    auto f = [&](long long j, int j1, int j2, int j3) -> float {
        return interior<NOP, NDIM>(g, j1, j2, j3) ? __ldg(vel + j) * __ldg(X + j) : 0.f;
    };
    float lt = in ? p.k.c0 * (__ldg(vel + i) * x) : 0.f;
#pragma unroll
    for (int k = 1; k <= NOP; k++) {
        float t = f(i - k, i1 - k, i2, i3) + f(i + k, i1 + k, i2, i3);
        lt = fmaf(t, p.k.c[0][k], lt);
        t = f(i - k * s2, i1, i2 - k, i3) + f(i + k * s2, i1, i2 + k, i3);
        lt = fmaf(t, p.k.c[1][k], lt);
        if constexpr (NDIM == 3) {
            t = f(i - k * s3, i1, i2, i3 - k) + f(i + k * s3, i1, i2, i3 + k);
            lt = fmaf(t, p.k.c[2][k], lt);
        }
    }
    const float w = wcell(p, i1, i2, i3);
    const float lam = (in ? 2.f * x : 0.f) + lt + (in ? -w : w) * Y[i];
    float mu = w * lam;
    if (p.rrow) {  // receiver residuals at this cell, in (receiver, corner) order
        for (int e = p.rc_start[i], e1 = p.rc_start[i + 1]; e < e1; e++) {
            const int2 en = p.rc_ent[e];
            mu = __fadd_rn(mu, __fmul_rn(w, __fmul_rn(w, __fmul_rn(__int_as_float(en.y), p.rrow[en.x]))));
        }
    }
    Y[i] = mu;
    if (in && p.xcorr) {
        G[i] = gsum_add(G[i], __fmul_rn(x, V[i]));  // FP32 product, compensated sum
    } else if (in) {
        float lap = V[i] * p.k.c0;
#pragma unroll
        for (int k = 1; k <= NOP; k++) {
            float t = fmaf(__ldg(V + i - k) + __ldg(V + i + k), p.k.c[0][k],
                           (__ldg(V + i - k * s2) + __ldg(V + i + k * s2)) * p.k.c[1][k]);
            if constexpr (NDIM == 3) t = fmaf(__ldg(V + i - k * s3) + __ldg(V + i + k * s3), p.k.c[2][k], t);
            lap += t;
        }
        G[i] = gsum_add(G[i], __fmul_rn(x, lap));
    }
    if (p.wav && !p.xcorr) {  // source term, in (source, corner) order
        for (int e = p.sc_start[i], e1 = p.sc_start[i + 1]; e < e1; e++) {
            const int2 en = p.sc_ent[e];
            const float dd = p.one_wavelet ? p.wav[(long long)p.it * p.ncs] : p.wav[(long long)p.it * p.ncs + en.x];
            G[i] = gsum_add_prod(G[i], x, dd * __int_as_float(en.y));
        }
    }
}

template <int NDIM>
static void adj_dispatch_nop(int nop, const float *X, float *Y, const float *V, const float *vel, float2 *G,
                             const AdjParams &p, cudaStream_t s) {
    dim3 block(64, 4, 1);
    dim3 grid((p.g.n1 + 63) / 64, (p.g.n2 + 3) / 4, NDIM == 3 ? p.g.n3 : 1);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = NDIM == 2 ? 1 : 0;  // launch-bound 2D steps: hide the launch gap
    switch (nop) {
#define CASE(N) \
    case N: cudaLaunchKernelEx(&cfg, k_adjB<N, NDIM>, X, Y, V, vel, G, p); break;
        CASE(1) CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8) CASE(9) CASE(10)
#undef CASE
        default: break;
    }
}

void launch_adjB(const float *X, float *Y, const float *V, const float *vel, float2 *G, const AdjParams &p,
                 cudaStream_t s) {
    if (p.nd == 3) adj_dispatch_nop<3>(p.nop, X, Y, V, vel, G, p, s);
    else adj_dispatch_nop<2>(p.nop, X, Y, V, vel, G, p, s);
}

// g = I vel2 nu, four cells per thread (n1 % 4 == 0)
__global__ void k_adj_g(const float4 *__restrict__ nu, const float4 *__restrict__ vel2, float4 *__restrict__ g, Grid gr,
                        int nop) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n4 = (long long)gr.n1 * gr.n2 * gr.n3 / 4;
    if (t >= n4) return;
    const long long c = 4 * t;
    const int i1 = (int)(c % gr.n1), i2 = (int)((c / gr.n1) % gr.n2), i3 = (int)(c / ((long long)gr.n1 * gr.n2));
    const bool rest = i2 >= nop && i2 < gr.n2 - nop && (gr.n3 == 1 || (i3 >= nop && i3 < gr.n3 - nop));
    const float4 a = nu[t], v = vel2[t];
    float4 o;
    o.x = (rest && i1 >= nop && i1 < gr.n1 - nop) ? v.x * a.x : 0.f;
    o.y = (rest && i1 + 1 >= nop && i1 + 1 < gr.n1 - nop) ? v.y * a.y : 0.f;
    o.z = (rest && i1 + 2 >= nop && i1 + 2 < gr.n1 - nop) ? v.z * a.z : 0.f;
    o.w = (rest && i1 + 3 >= nop && i1 + 3 < gr.n1 - nop) ? v.w * a.w : 0.f;
    g[t] = o;
}

void launch_adj_g(const float *nu, const float *vel2, float *g, const Grid &gr, int nop, cudaStream_t s) {
    const long long n4 = gr.cells() / 4;
    k_adj_g<<<(unsigned)((n4 + 255) / 256), 256, 0, s>>>((const float4 *)nu, (const float4 *)vel2, (float4 *)g, gr,
                                                         nop);
}

// ---------------------------------------------------------------------------
// Transpose of abcone3d_apply (fdutil.c:2085-2177).  The forward runs three
// passes (axis-1, axis-2, axis-3 faces); each updates, per line and outward,
// uo[i] = um[a] + (um[i] - uo[b]) * c with a = b = the inward neighbour.  The
// transpose visits the passes and the updates in reverse order:
//   t = mu[i]; mu[i] = 0; mu[b] -= c t; kap[a] += t; kap[i] += c t.
template <int AXIS>
__global__ void k_abc_adj(float *mu, float *kap, const float *__restrict__ bl, const float *__restrict__ bh, Grid g,
                          int nop, int top) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long base, st;
    int n;
    if (AXIS == 1) {  // line (i3, i2), coefficients [n3][n2]
        if (t >= (long long)g.n2 * g.n3) return;
        base = t * g.n1;
        st = 1;
        n = g.n1;
    } else if (AXIS == 2) {  // line (i3, i1), coefficients [n3][n1]
        if (t >= (long long)g.n1 * g.n3) return;
        base = (t / g.n1) * g.n1 * (long long)g.n2 + t % g.n1;
        st = g.n1;
        n = g.n2;
    } else {  // line (i2, i1), coefficients [n2][n1]
        if (t >= (long long)g.n1 * g.n2) return;
        base = t;
        st = (long long)g.n1 * g.n2;
        n = g.n3;
    }
    const float cl = bl[t], ch = bh[t];
    for (int jj = 0; jj < nop; jj++) {
        const int iop = nop - 1 - jj;
        long long i = base + (long long)(n - nop + iop - 1) * st, b = i - st;
        float v = mu[i];
        mu[i] = 0.f;
        mu[b] -= ch * v;
        kap[b] += v;
        kap[i] += ch * v;
        if (top) {
            i = base + (long long)(nop - iop) * st;
            b = i + st;
            v = mu[i];
            mu[i] = 0.f;
            mu[b] -= cl * v;
            kap[b] += v;
            kap[i] += cl * v;
        }
    }
}

// Axis-1 faces with nop = 4 and n1 % 4 == 0 (the layout of k_abc_axis1_v4):
// one thread per line keeps the eight cells at each end of mu and kap in
// registers (two float4 each) and runs the transposed recurrence there,
// instead of the dependent global read-modify-writes of k_abc_adj<1>.
__device__ __forceinline__ void abc_adj_cell(float &mi, float &mb, float &kb, float &ki, float c) {
    const float v = mi;
    mi = 0.f;
    mb -= c * v;
    kb += v;
    ki += c * v;
}

__global__ void k_abc_adj1_v4(float *__restrict__ mu, float *__restrict__ kap, const float *__restrict__ bl,
                              const float *__restrict__ bh, Grid g, int top) {
    const long long line = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= (long long)g.n2 * g.n3) return;
    const int q = g.n1 / 4;
    float4 *M = reinterpret_cast<float4 *>(mu + line * g.n1);
    float4 *K = reinterpret_cast<float4 *>(kap + line * g.n1);
    {  // i = n1-2, n1-3, n1-4, n1-5 (the forward's last update first), b = i - 1
        const float h = bh[line];
        float4 ma = M[q - 2], mb = M[q - 1], ka = K[q - 2], kb = K[q - 1];
        abc_adj_cell(mb.z, mb.y, kb.y, kb.z, h);
        abc_adj_cell(mb.y, mb.x, kb.x, kb.y, h);
        abc_adj_cell(mb.x, ma.w, ka.w, kb.x, h);
        abc_adj_cell(ma.w, ma.z, ka.z, ka.w, h);
        M[q - 2] = ma;
        M[q - 1] = mb;
        K[q - 2] = ka;
        K[q - 1] = kb;
    }
    if (top) {  // i = 1, 2, 3, 4, b = i + 1
        const float l = bl[line];
        float4 ma = M[0], mb = M[1], ka = K[0], kb = K[1];
        abc_adj_cell(ma.y, ma.z, ka.z, ka.y, l);
        abc_adj_cell(ma.z, ma.w, ka.w, ka.z, l);
        abc_adj_cell(ma.w, mb.x, kb.x, ka.w, l);
        abc_adj_cell(mb.x, mb.y, kb.y, kb.x, l);
        M[0] = ma;
        M[1] = mb;
        K[0] = ka;
        K[1] = kb;
    }
}

void launch_abc_adjB(int nop, int fsrf, float *mu, float *kap, const AbcB &a, const Grid &g, cudaStream_t s) {
    const int T = 128;
    long long n = (long long)g.n1 * g.n2;
    k_abc_adj<3><<<(unsigned)((n + T - 1) / T), T, 0, s>>>(mu, kap, a.yl, a.yh, g, nop, 1);
    n = (long long)g.n1 * g.n3;
    k_abc_adj<2><<<(unsigned)((n + T - 1) / T), T, 0, s>>>(mu, kap, a.xl, a.xh, g, nop, 1);
    n = (long long)g.n2 * g.n3;
    if (nop == 4 && g.n1 % 4 == 0 && g.n1 >= 16)
        k_abc_adj1_v4<<<(unsigned)((n + T - 1) / T), T, 0, s>>>(mu, kap, a.zl, a.zh, g, !fsrf);
    else
        k_abc_adj<1><<<(unsigned)((n + T - 1) / T), T, 0, s>>>(mu, kap, a.zl, a.zh, g, nop, !fsrf);
}

// mu += W kap on the faces the transpose ABC touched (the outer nop+2 cells of
// every axis), clearing kap for the next step.  The three slabs are disjoint:
// axis-1 ends of every line; axis-2 bands without them; axis-3 bands without both.
__global__ void k_kap_fold(float *mu, float *kap, AdjParams p, int width) {
    const Grid g = p.g;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int W = width;
    const long long n_a = (long long)g.n2 * g.n3 * 2 * W;
    const int in1 = g.n1 - 2 * W;
    const long long n_b = (long long)in1 * 2 * W * g.n3;
    const int in2 = g.n2 - 2 * W;
    const long long n_c = (long long)in1 * in2 * 2 * W;
    int i1, i2, i3;
    if (t < n_a) {
        const long long line = t / (2 * W);
        const int k = (int)(t - line * 2 * W);
        i1 = k < W ? k : g.n1 - 2 * W + k;
        i2 = (int)(line % g.n2);
        i3 = (int)(line / g.n2);
    } else if (t < n_a + n_b) {
        const long long u = t - n_a;
        i1 = W + (int)(u % in1);
        const long long r = u / in1;
        const int k = (int)(r % (2 * W));
        i2 = k < W ? k : g.n2 - 2 * W + k;
        i3 = (int)(r / (2 * W));
    } else if (t < n_a + n_b + n_c) {
        const long long u = t - n_a - n_b;
        i1 = W + (int)(u % in1);
        const long long r = u / in1;
        i2 = W + (int)(r % in2);
        const int k = (int)(r / in2);
        i3 = k < W ? k : g.n3 - 2 * W + k;
    } else {
        return;
    }
    const long long i = ((long long)i3 * g.n2 + i2) * g.n1 + i1;
    const float kv = kap[i];
    if (kv != 0.f) {
        mu[i] += wcell(p, i1, i2, i3) * kv;
        kap[i] = 0.f;
    }
}

void launch_kap_fold(float *mu, float *kap, const AdjParams &p, cudaStream_t s) {
    const Grid g = p.g;
    const int W = p.nop + 2;
    const long long n = (long long)g.n2 * g.n3 * 2 * W + (long long)(g.n1 - 2 * W) * 2 * W * g.n3 +
                        (long long)(g.n1 - 2 * W) * (g.n2 - 2 * W) * 2 * W;
    k_kap_fold<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(mu, kap, p, W);
}

// W R^T r: receiver residuals into mu (scaled by W twice: once from the
// gather of W V, once from mu = W lambda).  Coincident corners add atomically.
__global__ void k_rec_adj(float *mu, const GeoPoint *__restrict__ pts, int nr, const float *__restrict__ r,
                          AdjParams p, const long long *__restrict__ off) {
    const int ir = blockIdx.x * blockDim.x + threadIdx.x;
    if (ir >= nr) return;
    const GeoPoint pt = pts[ir];
    const float rv = r[ir];
    const Grid g = p.g;
    const int nc = p.nd == 3 ? 8 : 4;
    for (int c = 0; c < nc; c++) {
        const long long n = pt.base + off[c];
        const int i1 = (int)(n % g.n1), i2 = (int)((n / g.n1) % g.n2), i3 = (int)(n / ((long long)g.n1 * g.n2));
        const float w = wcell(p, i1, i2, i3);
        atomicAdd(mu + n, w * (w * (pt.w[c] * rv)));
    }
}

void launch_rec_adj(float *mu, const GeoPoint *pts, int nr, const float *r, const AdjParams &p, const long long *off,
                    cudaStream_t s) {
    if (nr > 0) k_rec_adj<<<(nr + 127) / 128, 128, 0, s>>>(mu, pts, nr, r, p, off);
}

// source term of the gradient: dJ/dvel2[node] += nu[node] * wav * w (one
// thread, sources and corners in order)
__global__ void k_src_grad(float2 *G, const float *__restrict__ nu, const GeoPoint *__restrict__ pts, int ns,
                           const float *__restrict__ wav, int it, int ncs, int one_wavelet, int nc,
                           const long long *__restrict__ off) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int s = 0; s < ns; s++) {
        const float dd = one_wavelet ? wav[(long long)it * ncs] : wav[(long long)it * ncs + s];
        const GeoPoint pt = pts[s];
        for (int c = 0; c < nc; c++) {
            const long long n = pt.base + off[c];
            G[n] = gsum_add_prod(G[n], nu[n], dd * pt.w[c]);
        }
    }
}

void launch_src_grad(float2 *G, const float *nu, const GeoPoint *pts, int ns, const float *wav, int it, int ncs,
                     bool one_wavelet, int nd, const long long *off, cudaStream_t s) {
    if (ns > 0) k_src_grad<<<1, 1, 0, s>>>(G, nu, pts, ns, wav, it, ncs, one_wavelet, nd == 3 ? 8 : 4, off);
}

// ---------------------------------------------------------------------------
// Residual and misfit: r = d - dobs per row; per-row sums of r^2 in FP64
// (one block per row, fixed reduction order).
__global__ void k_residual(const float *__restrict__ d, const float *__restrict__ dobs, float *__restrict__ r, int nr,
                           double *__restrict__ row_sum) {
    const int row = blockIdx.x;
    __shared__ double part[256];
    double acc = 0;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
        const long long j = (long long)row * nr + i;
        const float v = d[j] - dobs[j];
        r[j] = v;
        acc += (double)v * (double)v;
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) row_sum[row] = part[0];
}

void launch_residual(const float *d, const float *dobs, float *r, int nrows, int nr, double *row_sum, cudaStream_t s) {
    if (nrows > 0) k_residual<<<nrows, 256, 0, s>>>(d, dobs, r, nr, row_sum);
}

// ---------------------------------------------------------------------------
// Checkpoints: BF16 or FP16 with one FP32 scale per level (the level's
// max |v|), or plain FP32 copies.
__global__ void k_absmax(const float *__restrict__ u, long long n, unsigned int *out) {
    float m = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(u[i]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));  // non-negative floats order as unsigned
}

__device__ __forceinline__ void to16(float x, __nv_bfloat16 &q) { q = __float2bfloat16_rn(x); }
__device__ __forceinline__ void to16(float x, __half &q) { q = __float2half_rn(x); }
__device__ __forceinline__ float from16(__nv_bfloat16 q) { return __bfloat162float(q); }
__device__ __forceinline__ float from16(__half q) { return __half2float(q); }

// q = round(u / scale) with scale = max |u| (1 for an all-zero level): the
// values land in [-1, 1], inside FP16's normal range down to 6e-5 of the max
template <typename Q>
__global__ void k_quant16(const float *__restrict__ u, long long n, const unsigned int *__restrict__ amax,
                          Q *__restrict__ q, float *__restrict__ scale_out) {
    const float a = __uint_as_float(*amax);
    const float scale = a > 0.f ? a : 1.f;
    const float inv = 1.f / scale;
    if (blockIdx.x == 0 && threadIdx.x == 0) *scale_out = scale;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        to16(u[i] * inv, q[i]);
}

template <typename Q>
__global__ void k_dequant16(const Q *__restrict__ q, long long n, const float *__restrict__ scale,
                            float *__restrict__ u) {
    const float sc = *scale;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        u[i] = from16(q[i]) * sc;
}

void launch_ckpt_store16(bool fp16, const float *u, long long n, unsigned int *amax, void *q, float *scale, int grid,
                         cudaStream_t s) {
    cudaMemsetAsync(amax, 0, sizeof(unsigned int), s);
    k_absmax<<<grid, 256, 0, s>>>(u, n, amax);
    if (fp16) k_quant16<__half><<<grid, 256, 0, s>>>(u, n, amax, (__half *)q, scale);
    else k_quant16<__nv_bfloat16><<<grid, 256, 0, s>>>(u, n, amax, (__nv_bfloat16 *)q, scale);
}

void launch_ckpt_load16(bool fp16, const void *q, long long n, const float *scale, float *u, int grid,
                        cudaStream_t s) {
    if (fp16) k_dequant16<__half><<<grid, 256, 0, s>>>((const __half *)q, n, scale, u);
    else k_dequant16<__nv_bfloat16><<<grid, 256, 0, s>>>((const __nv_bfloat16 *)q, n, scale, u);
}

// Block floating point: each block of 64 consecutive cells keeps 16-bit
// integers q = round(v / s) and one FP32 scale s = max|v| / 32767 of the
// block, so the error is at most s/2 - relative to the block's largest value
// 2^-16, against BF16's 2^-9 per value.  One warp per block: lane l holds
// cells l and l + 32 (coalesced 128-byte loads, 64-byte stores); the
// division and the reciprocal are IEEE round-to-nearest so a host
// restatement gets the same integers.  Unlike the per-level formats no
// separate max pass over the level is needed.
__global__ void k_bfp_store(const float *__restrict__ u, long long n, short *__restrict__ q,
                            float *__restrict__ scale) {
    const int lane = threadIdx.x & 31;
    const long long nblk = (n + kBfpBlock - 1) / kBfpBlock;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long b = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < nblk; b += warps) {
        const long long i0 = b * kBfpBlock + lane, i1 = i0 + 32;
        const float v0 = i0 < n ? u[i0] : 0.f, v1 = i1 < n ? u[i1] : 0.f;
        float m = fmaxf(fabsf(v0), fabsf(v1));
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        // blocks at or below kBfpTiny store zeros (keeps s and 1/s normal floats)
        const float sc = m > kBfpTiny ? __fdiv_rn(m, 32767.f) : 0.f;
        const float inv = m > kBfpTiny ? __frcp_rn(sc) : 0.f;
        const int a0 = max(-32767, min(32767, __float2int_rn(__fmul_rn(v0, inv))));
        const int a1 = max(-32767, min(32767, __float2int_rn(__fmul_rn(v1, inv))));
        if (i0 < n) q[i0] = (short)a0;
        if (i1 < n) q[i1] = (short)a1;
        if (lane == 0) scale[b] = sc;
    }
}

__global__ void k_bfp_load(const short *__restrict__ q, const float *__restrict__ scale, long long n,
                           float *__restrict__ u) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        u[i] = __fmul_rn(__int2float_rn(q[i]), scale[i / kBfpBlock]);
}

void launch_ckpt_store_bfp(const float *u, long long n, short *q, float *scale, int grid, cudaStream_t s) {
    k_bfp_store<<<grid, 256, 0, s>>>(u, n, q, scale);
}

void launch_ckpt_load_bfp(const short *q, const float *scale, long long n, float *u, int grid, cudaStream_t s) {
    k_bfp_load<<<grid, 256, 0, s>>>(q, scale, n, u);
}

// ---------------------------------------------------------------------------
// dJ/dm on the model grid: dJ/dvel2 * (-vel2^2 / dt^2) per padded cell (vel2 =
// v^2 dt^2, m = 1/v^2; zero where vel2 is zero), summed over the padded cells
// that replicate each model cell (the transpose of the edge padding).
// padded cells that replicate model index j along one axis
__device__ __forceinline__ void fold_range(int j, int m, int npad, int nb, int &lo, int &hi) {
    lo = j == 0 ? 0 : j + nb;
    hi = j == m - 1 ? npad - 1 : j + nb;
}

__device__ __forceinline__ int edge_axes(int j1, int j2, int j3, int m1, int m2, int m3, int nd) {
    return (j1 == 0 || j1 == m1 - 1) + (j2 == 0 || j2 == m2 - 1) + (nd == 3 && (j3 == 0 || j3 == m3 - 1));
}

// skip_big: model cells on two or more edge axes (the model's edges and
// corners, whose replicas span (nb+1)^2 or (nb+1)^3 padded cells) are left
// to k_grad_fold_big
// vel2 holds c = v^2 dt^2 per padded cell, or (cscale > 0) the velocity v with c = cscale v^2
__device__ __forceinline__ double fold_c(const float *vel2, long long i, double cscale) {
    const double v = vel2[i];
    return cscale > 0 ? cscale * v * v : v;
}

__global__ void k_grad_fold(const float2 *__restrict__ G, const float *__restrict__ vel2, double inv_dt2, Grid g,
                            int nb, int m1, int m2, int m3, int nd, double *__restrict__ out, int skip_big,
                            double cscale) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m1 * m2 * m3) return;
    const int j1 = (int)(t % m1), j2 = (int)((t / m1) % m2), j3 = (int)(t / ((long long)m1 * m2));
    if (skip_big && edge_axes(j1, j2, j3, m1, m2, m3, nd) >= 2) return;
    auto range = [&](int j, int m, int npad, int &lo, int &hi) { fold_range(j, m, npad, nb, lo, hi); };
    int a1, b1, a2, b2, a3 = 0, b3 = 0;
    range(j1, m1, g.n1, a1, b1);
    range(j2, m2, g.n2, a2, b2);
    if (nd == 3) range(j3, m3, g.n3, a3, b3);
    double acc = 0;
    for (int i3 = a3; i3 <= b3; i3++)
        for (int i2 = a2; i2 <= b2; i2++)
            for (int i1 = a1; i1 <= b1; i1++) {
                const long long i = ((long long)i3 * g.n2 + i2) * g.n1 + i1;
                const double v2 = fold_c(vel2, i, cscale);
                acc += gsum_value(G[i]) * (-v2 * v2 * inv_dt2);
            }
    out[t] = acc;
}

__global__ void k_image_cut(const float2 *__restrict__ G, Grid g, int nb, int m1, int m2, int m3, int nd,
                            double *__restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m1 * m2 * m3) return;
    const int j1 = (int)(t % m1), j2 = (int)((t / m1) % m2), j3 = (int)(t / ((long long)m1 * m2));
    out[t] = gsum_value(G[((long long)(nd == 3 ? j3 + nb : 0) * g.n2 + j2 + nb) * g.n1 + j1 + nb]);
}

// dst += src (gradients of several shots)
__global__ void k_add_f64(double *__restrict__ dst, const double *__restrict__ src, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] += src[i];
}

void launch_add_f64(double *dst, const double *src, long long n, cudaStream_t s) {
    if (n > 0) k_add_f64<<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256, 0, s>>>(dst, src, n);
}

void launch_image_cut(const float2 *G, const Grid &g, int nb, const int *n, int nd, double *out, cudaStream_t s) {
    const long long m = (long long)n[0] * n[1] * (nd == 3 ? n[2] : 1);
    k_image_cut<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(G, g, nb, n[0], n[1], nd == 3 ? n[2] : 1, nd, out);
}

// The model's edge and corner cells, one block each: 2D the 4 corners; 3D
// the 4 edges along each axis (corners counted with the axis-1 edges).
__global__ void __launch_bounds__(256) k_grad_fold_big(const float2 *__restrict__ G, const float *__restrict__ vel2,
                                                       double inv_dt2, Grid g, int nb, int m1, int m2, int m3, int nd,
                                                       double *__restrict__ out, double cscale) {
    long long b = blockIdx.x;
    int j1, j2, j3 = 0;
    if (nd == 2) {
        j1 = (b & 1) ? m1 - 1 : 0;
        j2 = (b & 2) ? m2 - 1 : 0;
    } else if (b < 4LL * m1) {
        const int e = (int)(b / m1);
        j1 = (int)(b % m1);
        j2 = (e & 1) ? m2 - 1 : 0;
        j3 = (e & 2) ? m3 - 1 : 0;
    } else if ((b -= 4LL * m1) < 4LL * (m2 - 2)) {
        const int e = (int)(b / (m2 - 2));
        j2 = 1 + (int)(b % (m2 - 2));
        j1 = (e & 1) ? m1 - 1 : 0;
        j3 = (e & 2) ? m3 - 1 : 0;
    } else {
        b -= 4LL * (m2 - 2);
        const int e = (int)(b / (m3 - 2));
        j3 = 1 + (int)(b % (m3 - 2));
        j1 = (e & 1) ? m1 - 1 : 0;
        j2 = (e & 2) ? m2 - 1 : 0;
    }
    int a1, b1, a2, b2, a3 = 0, b3 = 0;
    fold_range(j1, m1, g.n1, nb, a1, b1);
    fold_range(j2, m2, g.n2, nb, a2, b2);
    if (nd == 3) fold_range(j3, m3, g.n3, nb, a3, b3);
    const long long w1 = b1 - a1 + 1, w2 = b2 - a2 + 1, vol = w1 * w2 * (b3 - a3 + 1);
    double acc = 0;
    for (long long k = threadIdx.x; k < vol; k += blockDim.x) {
        const long long i1 = a1 + k % w1, i2 = a2 + (k / w1) % w2, i3 = a3 + k / (w1 * w2);
        const long long i = (i3 * g.n2 + i2) * g.n1 + i1;
        const double v2 = fold_c(vel2, i, cscale);
        acc += gsum_value(G[i]) * (-v2 * v2 * inv_dt2);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += part[w];
        out[((long long)j3 * m2 + j2) * m1 + j1] = t;
    }
}

void launch_grad_fold(const float2 *G, const float *vel2, float dt, const Grid &g, int nb, const int *n, int nd,
                      double *out, cudaStream_t s, bool raw_v) {
    const double cscale = raw_v ? (double)dt * (double)dt : 0.0;
    const int m1 = n[0], m2 = n[1], m3 = nd == 3 ? n[2] : 1;
    const long long m = (long long)m1 * m2 * m3;
    const double inv = 1.0 / ((double)dt * (double)dt);
    // edges and corners go to one block each when every model axis has an interior
    const bool split = m1 >= 3 && m2 >= 3 && (nd == 2 || m3 >= 3);
    k_grad_fold<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(G, vel2, inv, g, nb, m1, m2, m3, nd, out, split ? 1 : 0,
                                                            cscale);
    if (split) {
        const long long nbig = nd == 2 ? 4 : 4LL * (m1 + m2 - 2 + m3 - 2);
        k_grad_fold_big<<<(unsigned)nbig, 256, 0, s>>>(G, vel2, inv, g, nb, m1, m2, m3, nd, out, cscale);
    }
}

}  // namespace awe
