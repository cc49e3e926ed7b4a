// The boundary work of one 3D step of the CPU-program scheme in one launch:
// the one-way ABC of the six faces (abcone3d_apply, fdutil.c:2085-2177), the
// sponge of the shell the step kernel left unsponged (sponge3d_apply,
// fdutil.c:2248-2310), the receiver gather of the level the step read
// (lint3d_extract, fdutil.c:1653-1670) and, when no source touches the shell,
// the injection (lint3d_inject1_with_vv, fdutil.c:1723-1740).
//
// The reference applies the ABC as three passes over the whole grid (axis-1
// lines, then axis-2 lines, then axis-3 lines, each an outward recurrence over
// the nop = 4 outer cells from the fifth), then the sponge.  The passes only
// meet in the shell (cells within 6 of a face), so the work splits into
// blocks that each own a whole chain of dependencies:
//  * a plane y in [6, n3-6) (no axis-3 face cell): its axis-1 line ends, then
//    (after a barrier) its axis-2 line ends, each sponged once it is final;
//  * a face block (planes 0..5 or n3-6..n3-1) x a 16-column x-range x a
//    64-cell z-range: the axis-1 pass of its lines, the axis-2 pass of its
//    z-range (x-ranges holding a face), the axis-3 pass of its columns, then
//    the sponge of all its cells;
//  * receiver blocks (256 receivers each) and one injection block, which read
//    or write cells no pass touches.
// Every cell is written by one block only, so the result does not depend on
// the order in which blocks run.
//
// The axis-1 ends (8 cells at each end of every line, 32 bytes of every
// n1*4-byte line) are the scattered part of the work.  Within a forward run
// each launch also writes the final ends of the new level to a compact
// [n3][n2][16] copy, and the next step's launch reads the ends of the level
// its step read (the same values) from that copy with coalesced loads
// instead of one scattered sector per line end.
#include <cuda_runtime.h>

#include "awe_internal.h"
#include "fp_exact.cuh"

namespace awe {

namespace b3 {
constexpr int SHELL = 6;  // nop + 2: cells the ABC writes (1..4) or reads (5), and the face cell 0
constexpr int XR = 16, ZR = 64;
constexpr int NT = 256;
}  // namespace b3

template <bool EXACT>
__device__ __forceinline__ float b3_abc(float um_in, float um_c, float uo_in, float b) {
    // uo = um[inner] + (um[c] - uo[inner]) * b
    return fadd<EXACT>(um_in, fmul<EXACT>(fsub<EXACT>(um_c, uo_in), b));
}

template <bool EXACT>
__device__ __forceinline__ float b3_damp(float v, float wz, float wx, float wy) {
    return fmul<EXACT>(fmul<EXACT>(fmul<EXACT>(v, wz), wx), wy);
}

// axis-1 low face of one line: cells 4, 3, 2, 1 from cell 5 (a = cells 0..3, b = 4..7)
template <bool EXACT>
__device__ __forceinline__ void b3_zlow(float4 &a, float4 &b, const float4 ma, const float4 mb, float c) {
    const float u4 = b3_abc<EXACT>(mb.y, mb.x, b.y, c);
    const float u3 = b3_abc<EXACT>(mb.x, ma.w, u4, c);
    const float u2 = b3_abc<EXACT>(ma.w, ma.z, u3, c);
    a.y = b3_abc<EXACT>(ma.z, ma.y, u2, c);
    a.z = u2;
    a.w = u3;
    b.x = u4;
}

// axis-1 high face: cells n1-5 .. n1-2 from n1-6 (a = cells n1-8..n1-5, b = n1-4..n1-1)
template <bool EXACT>
__device__ __forceinline__ void b3_zhigh(float4 &a, float4 &b, const float4 ma, const float4 mb, float c) {
    const float v5 = b3_abc<EXACT>(ma.z, ma.w, a.z, c);
    const float v4 = b3_abc<EXACT>(ma.w, mb.x, v5, c);
    const float v3 = b3_abc<EXACT>(mb.x, mb.y, v4, c);
    b.z = b3_abc<EXACT>(mb.y, mb.z, v3, c);
    a.w = v5;
    b.x = v4;
    b.y = v3;
}

template <bool EXACT>
__device__ __forceinline__ void b3_damp4(float4 &v, const float *w1, int z, float wx, float wy, unsigned mask) {
    const float4 wz = __ldg(reinterpret_cast<const float4 *>(w1 + z));
    if (mask & 1u) v.x = b3_damp<EXACT>(v.x, wz.x, wx, wy);
    if (mask & 2u) v.y = b3_damp<EXACT>(v.y, wz.y, wx, wy);
    if (mask & 4u) v.z = b3_damp<EXACT>(v.z, wz.z, wx, wy);
    if (mask & 8u) v.w = b3_damp<EXACT>(v.w, wz.w, wx, wy);
}

// one axis-2 face line (y, z): cells x = xa+dx .. xa+4dx from xa (outward),
// optionally sponged (cells xs .. xs+5 of the line, the axis-2 shell)
template <bool EXACT>
__device__ __forceinline__ void b3_xline(const Bnd3Params &p, long long c0, int y, int z, bool low, bool damp) {
    const long long s2 = p.g.n1;
    const int xa = low ? 5 : p.g.n2 - b3::SHELL, dx = low ? -1 : 1;
    const float b = __ldg((low ? p.xl : p.xh) + (long long)y * p.g.n1 + z);
    float v[6];  // cells xa .. xa + 5dx (the last one is the face cell 0 / n2-1)
#pragma unroll
    for (int k = 0; k < 6; k++) v[k] = p.uo[c0 + (long long)(xa + k * dx) * s2];
    float m[5];
#pragma unroll
    for (int k = 0; k < 5; k++) m[k] = __ldg(p.um + c0 + (long long)(xa + k * dx) * s2);
#pragma unroll
    for (int k = 1; k <= 4; k++) v[k] = b3_abc<EXACT>(m[k - 1], m[k], v[k - 1], b);
    if (damp) {
        const float wz = __ldg(p.w1 + z), wy = __ldg(p.w3 + y);
#pragma unroll
        for (int k = 0; k < 6; k++) v[k] = b3_damp<EXACT>(v[k], wz, __ldg(p.w2 + xa + k * dx), wy);
        p.uo[c0 + (long long)xa * s2] = v[0];
        p.uo[c0 + (long long)(xa + 5 * dx) * s2] = v[5];
    }
#pragma unroll
    for (int k = 1; k <= 4; k++) p.uo[c0 + (long long)(xa + k * dx) * s2] = v[k];
}

// float4 `part` of line `line`'s ends (parts 0, 1: cells 0..7; 2, 3: cells
// n1-8..n1-1) of the level the step read: from the compact copy of its line
// ends the previous step's launch wrote (em), else from the level itself
__device__ __forceinline__ float4 b3_mend(const Bnd3Params &p, long long line, int part) {
    if (p.em) return __ldg(reinterpret_cast<const float4 *>(p.em) + line * 4 + part);
    const float4 *m = reinterpret_cast<const float4 *>(p.um + line * p.g.n1);
    return __ldg(m + (part < 2 ? part : p.g.n1 / 4 - 4 + part));
}

// the compact copy of the new level's line ends (eo), read back from uo once
// the line's cells are final
__device__ __forceinline__ void b3_eput_from_uo(const Bnd3Params &p, long long line, int part) {
    const float4 *o = reinterpret_cast<const float4 *>(p.uo + line * p.g.n1);
    reinterpret_cast<float4 *>(p.eo)[line * 4 + part] = o[part < 2 ? part : p.g.n1 / 4 - 4 + part];
}

template <bool EXACT>
__global__ void __launch_bounds__(b3::NT, 4) k_bnd3(const Bnd3Params p) {
    using namespace b3;
    const int tid = threadIdx.x;
    const int n1 = p.g.n1, n2 = p.g.n2, n3 = p.g.n3;
    const long long s2 = n1, s3 = (long long)n1 * n2;
    int blk = blockIdx.x;

    if (blk < p.n_int) {  // ---- one plane without axis-3 face cells
        const int y = SHELL + blk;
        const float wy = p.w3 ? __ldg(p.w3 + y) : 1.f;
        const int q = n1 / 4;
        for (int x = tid; x < n2; x += NT) {
            const long long line = (long long)y * n2 + x;
            float4 *o = reinterpret_cast<float4 *>(p.uo + line * n1);
            // lines in the axis-2 shell are sponged by the axis-2 pass below
            const bool xshell = x < SHELL || x >= n2 - SHELL;
            const bool damp = p.w1 && !xshell;
            const float wx = damp ? __ldg(p.w2 + x) : 1.f;
            float4 lo0 = make_float4(0.f, 0.f, 0.f, 0.f), lo1 = lo0;  // cells 0..7 as left
            if (p.top || damp) {
                lo0 = o[0];
                lo1 = o[1];
                if (p.top) b3_zlow<EXACT>(lo0, lo1, b3_mend(p, line, 0), b3_mend(p, line, 1), __ldg(p.zl + line));
                if (damp) {
                    b3_damp4<EXACT>(lo0, p.w1, 0, wx, wy, 15u);
                    b3_damp4<EXACT>(lo1, p.w1, 4, wx, wy, 3u);
                }
                o[0] = lo0;
                o[1] = lo1;
            }
            float4 a = o[q - 2], b = o[q - 1];
            b3_zhigh<EXACT>(a, b, b3_mend(p, line, 2), b3_mend(p, line, 3), __ldg(p.zh + line));
            if (damp) {
                b3_damp4<EXACT>(a, p.w1, n1 - 8, wx, wy, 12u);
                b3_damp4<EXACT>(b, p.w1, n1 - 4, wx, wy, 15u);
            }
            o[q - 2] = a;
            o[q - 1] = b;
            // final unless the axis-2 pass changes the line (the axis-2 shell);
            // without a sponge and with a free surface the low end is not
            // read (nor needed: the next step's low-end ABC is off)
            if (p.eo && !xshell) {
                float4 *e = reinterpret_cast<float4 *>(p.eo) + line * 4;
                e[0] = lo0;
                e[1] = lo1;
                e[2] = a;
                e[3] = b;
            }
        }
        __syncthreads();  // the axis-2 pass reads the axis-1 results of lines x = 1..5
        for (int z = tid; z < n1; z += NT) {
            const long long c0 = (long long)y * s3 + z;
            b3_xline<EXACT>(p, c0, y, z, true, p.w1 != nullptr);
            b3_xline<EXACT>(p, c0, y, z, false, p.w1 != nullptr);
        }
        if (p.eo) {  // the axis-2 shell lines' ends, final now
            __syncthreads();
            for (int l = tid; l < 2 * SHELL * 4; l += NT) {
                const int k = l >> 2, x = k < SHELL ? k : n2 - 2 * SHELL + k;
                b3_eput_from_uo(p, (long long)y * n2 + x, l & 3);
            }
        }
        return;
    }
    blk -= p.n_int;
    if (blk < 2 * p.nxr * p.nzr) {  // ---- face block
        const int f = blk / (p.nxr * p.nzr), r = blk % (p.nxr * p.nzr), xr = r / p.nzr, zr = r % p.nzr;
        const int xa = xr * XR, xb = xr == p.nxr - 1 ? n2 : xa + XR;
        const int za = zr * ZR, zb = zr == p.nzr - 1 ? n1 : za + ZR;
        const int ya = f == 0 ? 0 : n3 - SHELL;  // planes [ya, ya + 6)
        const int ncol = xb - xa, nz = zb - za, q = n1 / 4;
        // axis 1: the line ends inside this z-range
        const bool zlo = zr == 0 && p.top, zhi = zr == p.nzr - 1;
        if (zlo || zhi)
            for (int l = tid; l < SHELL * ncol; l += NT) {
                const int y = ya + l / ncol, x = xa + l % ncol;
                const long long line = (long long)y * n2 + x;
                float4 *o = reinterpret_cast<float4 *>(p.uo + line * n1);
                if (zlo) {
                    float4 a = o[0], b = o[1];
                    b3_zlow<EXACT>(a, b, b3_mend(p, line, 0), b3_mend(p, line, 1), __ldg(p.zl + line));
                    o[0] = a;
                    o[1] = b;
                }
                if (zhi) {
                    float4 a = o[q - 2], b = o[q - 1];
                    b3_zhigh<EXACT>(a, b, b3_mend(p, line, 2), b3_mend(p, line, 3), __ldg(p.zh + line));
                    o[q - 2] = a;
                    o[q - 1] = b;
                }
            }
        __syncthreads();
        // axis 2: the x-ranges holding a face, lines (y, z) of this z-range
        const bool xlo = xr == 0, xhi = xr == p.nxr - 1;
        if (xlo || xhi)
            for (int l = tid; l < SHELL * nz; l += NT) {
                const int y = ya + l / nz, z = za + l % nz;
                const long long c0 = (long long)y * s3 + z;
                if (xlo) b3_xline<EXACT>(p, c0, y, z, true, false);
                if (xhi) b3_xline<EXACT>(p, c0, y, z, false, false);
            }
        __syncthreads();
        // axis 3: columns (x, z), planes 4..1 from 5 or n3-5..n3-2 from n3-6
        for (int l = tid; l < ncol * nz; l += NT) {
            const int x = xa + l / nz, z = za + l % nz;
            const long long c0 = (long long)x * s2 + z;
            const int y0 = f == 0 ? 5 : n3 - SHELL, dy = f == 0 ? -1 : 1;
            const float b = __ldg((f == 0 ? p.yl : p.yh) + (long long)x * n1 + z);
            float v = p.uo[c0 + (long long)y0 * s3], mprev = __ldg(p.um + c0 + (long long)y0 * s3);
#pragma unroll
            for (int k = 1; k <= 4; k++) {
                const long long c = c0 + (long long)(y0 + k * dy) * s3;
                const float mc = __ldg(p.um + c);
                v = b3_abc<EXACT>(mprev, mc, v, b);
                p.uo[c] = v;
                mprev = mc;
            }
        }
        if (p.w1) {
            __syncthreads();
            // sponge of every cell of the block (all lie in the axis-3 shell)
            const int nq = nz / 4;
            for (int l = tid; l < SHELL * ncol * nq; l += NT) {
                const int y = ya + l / (ncol * nq), k = l % (ncol * nq), x = xa + k / nq, z = za + 4 * (k % nq);
                float4 *c = reinterpret_cast<float4 *>(p.uo + (long long)y * s3 + (long long)x * s2 + z);
                float4 v = *c;
                b3_damp4<EXACT>(v, p.w1, z, __ldg(p.w2 + x), __ldg(p.w3 + y), 15u);
                *c = v;
            }
        }
        if (p.eo && (zr == 0 || zr == p.nzr - 1)) {  // the line ends this block holds, final now
            __syncthreads();
            for (int l = tid; l < SHELL * ncol * 4; l += NT) {
                const int k = l >> 2, part = l & 3;
                if (part < 2 ? zr != 0 : zr != p.nzr - 1) continue;
                b3_eput_from_uo(p, (long long)(ya + k / ncol) * n2 + xa + k % ncol, part);
            }
        }
        return;
    }
    blk -= 2 * p.nxr * p.nzr;
    if (blk < p.rec_blocks) {  // ---- receiver gather of um (its pending sponge applied)
        const int r = blk * NT + tid;
        if (r >= p.nr) return;
        const GeoPoint pt = p.rec[(long long)r * p.rec_stride];
        float acc = 0.f;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const long long n = pt.base + ((c & 1) ? 1 : 0) + ((c & 2) ? s2 : 0) + ((c & 4) ? s3 : 0);
            float v = __ldg(p.um + n);
            if (p.w1) {
                const int i3 = (int)(n / s3), rem = (int)(n % s3);
                v = fmul<EXACT>(v, __ldg(p.w1 + rem % n1));
                v = fmul<EXACT>(v, __ldg(p.w2 + rem / n1));
                v = fmul<EXACT>(v, __ldg(p.w3 + i3));
            }
            const float t = fmul<EXACT>(v, pt.w[c]);
            acc = (c == 0) ? t : fadd<EXACT>(acc, t);
        }
        p.rec_row[r] = acc;
        return;
    }
    blk -= p.rec_blocks;
    if (blk == 0 && p.ns > 0 && tid == 0) {  // ---- injection, sources and corners in order
        for (int s = 0; s < p.ns; s++) {
            const float dd = p.one_wavelet ? p.wav[(long long)p.it * p.ncs] : p.wav[(long long)p.it * p.ncs + s];
            const GeoPoint pt = p.src[(long long)s * p.src_stride];
            for (int c = 0; c < 8; c++) {
                const long long n = pt.base + ((c & 1) ? 1 : 0) + ((c & 2) ? s2 : 0) + ((c & 4) ? s3 : 0);
                p.uo[n] = fadd<EXACT>(p.uo[n], fmul<EXACT>(fmul<EXACT>(dd, pt.w[c]), p.vel[n]));
            }
        }
    }
}

bool bnd3_eligible(int nop, const Grid &g) {
    return nop == 4 && g.n1 % 4 == 0 && g.n1 >= 16 && g.n2 >= 2 * b3::SHELL && g.n3 >= 2 * b3::SHELL;
}

void launch_bnd3(bool exact, Bnd3Params p, cudaStream_t s) {
    using namespace b3;
    p.n_int = p.g.n3 - 2 * SHELL;
    p.nxr = p.g.n2 / XR > 0 ? p.g.n2 / XR : 1;
    p.nzr = p.g.n1 / ZR > 0 ? p.g.n1 / ZR : 1;
    p.rec_blocks = p.rec_row ? (p.nr + NT - 1) / NT : 0;
    const int grid = p.n_int + 2 * p.nxr * p.nzr + p.rec_blocks + (p.ns > 0 ? 1 : 0);
    if (exact) k_bnd3<true><<<grid, NT, 0, s>>>(p);
    else k_bnd3<false><<<grid, NT, 0, s>>>(p);
}

// ---------------------------------------------------------------------------
// The boundary work before one adjoint step of the 3D gradient in one launch:
//  1. fold the previous adjoint step's kappa into mu on the shell (mu += W
//     kappa, kappa = 0; cells within nop + 2 of a face),
//  2. the transpose of the one-way ABC (abcone3d_apply, fdutil.c:2085-2177),
//     passes in reverse order (axis 3, axis 2, axis 1) and updates within a
//     line in reverse order: t = mu[i]; mu[i] = 0; mu[b] -= c t;
//     kappa[b] += t; kappa[i] += c t (b the inward neighbour of i),
//  3. g = I vel2 mu on every cell (I: at least nop from every face), the
//     field the adjoint step's stencil reads.
// Block roles as in k_bnd3, so each cell's chain runs in one block: a plane y
// in [6, n3-6) folds its axis-2 bands, runs the axis-2 lines, then folds and
// transposes its axis-1 line ends together, then forms g for the plane; a
// face block (6 axis-3 face planes x 16 columns x 64 cells of axis 1) folds
// all its cells, runs the axis-3, axis-2 and axis-1 lines it holds, then
// forms g.  The result does not depend on block order.
namespace b3a {
__device__ __forceinline__ void tcell(float &mi, float &mb, float &kb, float &ki, float c) {
    const float v = mi;
    mi = 0.f;
    mb -= c * v;
    kb += v;
    ki += c * v;
}

__device__ __forceinline__ float wcell3(const Bnd3AdjParams &p, int z, int x, int y) {
    if (!p.w1) return 1.f;
    return __ldg(p.w1 + z) * __ldg(p.w2 + x) * __ldg(p.w3 + y);
}

// mu += W kappa, kappa = 0 (cells whose kappa is 0 keep their value)
__device__ __forceinline__ void fold(const Bnd3AdjParams &p, long long i, int z, int x, int y) {
    const float kv = p.kap[i];
    if (kv != 0.f) {
        p.mu[i] += wcell3(p, z, x, y) * kv;
        p.kap[i] = 0.f;
    }
}

// transpose of one line's ABC updates: cells base + j*st, j = 0..n-1;
// high face i = n-2 .. n-5 (b = i-1), low face i = 1 .. 4 (b = i+1)
__device__ __forceinline__ void tline(const Bnd3AdjParams &p, long long base, long long st, int n, float cl, float ch,
                                      bool low) {
    for (int i = n - 2; i >= n - 5; i--) {
        const long long ci = base + i * st, cb = ci - st;
        float mi = p.mu[ci], mb = p.mu[cb], kb = p.kap[cb], ki = p.kap[ci];
        tcell(mi, mb, kb, ki, ch);
        p.mu[ci] = mi;
        p.mu[cb] = mb;
        p.kap[cb] = kb;
        p.kap[ci] = ki;
    }
    if (low)
        for (int i = 1; i <= 4; i++) {
            const long long ci = base + i * st, cb = ci + st;
            float mi = p.mu[ci], mb = p.mu[cb], kb = p.kap[cb], ki = p.kap[ci];
            tcell(mi, mb, kb, ki, cl);
            p.mu[ci] = mi;
            p.mu[cb] = mb;
            p.kap[cb] = kb;
            p.kap[ci] = ki;
        }
}

// axis-1 ends of line `line` (n1 % 4 == 0): optionally fold cells 0..5 and
// n1-6..n1-1 first, then the transposed updates, in registers
__device__ __forceinline__ void zends(const Bnd3AdjParams &p, long long line, int x, int y, bool dofold) {
    const int n1 = p.g.n1, q = n1 / 4;
    float4 *M = reinterpret_cast<float4 *>(p.mu + line * n1);
    float4 *K = reinterpret_cast<float4 *>(p.kap + line * n1);
    auto fold4 = [&](float4 &m, float4 &k, int z0, unsigned mask) {
        float *mv = &m.x, *kv = &k.x;
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (((mask >> j) & 1u) && kv[j] != 0.f) {
                mv[j] += wcell3(p, z0 + j, x, y) * kv[j];
                kv[j] = 0.f;
            }
    };
    {  // high end: cells n1-8 .. n1-1
        float4 ma = M[q - 2], mb = M[q - 1], ka = K[q - 2], kb = K[q - 1];
        if (dofold) {
            fold4(ma, ka, n1 - 8, 12u);
            fold4(mb, kb, n1 - 4, 15u);
        }
        const float h = __ldg(p.zh + line);
        tcell(mb.z, mb.y, kb.y, kb.z, h);
        tcell(mb.y, mb.x, kb.x, kb.y, h);
        tcell(mb.x, ma.w, ka.w, kb.x, h);
        tcell(ma.w, ma.z, ka.z, ka.w, h);
        M[q - 2] = ma;
        M[q - 1] = mb;
        K[q - 2] = ka;
        K[q - 1] = kb;
    }
    {  // low end: cells 0 .. 7
        float4 ma = M[0], mb = M[1], ka = K[0], kb = K[1];
        if (dofold) {
            fold4(ma, ka, 0, 15u);
            fold4(mb, kb, 4, 3u);
        }
        if (p.top) {
            const float l = __ldg(p.zl + line);
            tcell(ma.y, ma.z, ka.z, ka.y, l);
            tcell(ma.z, ma.w, ka.w, ka.z, l);
            tcell(ma.w, mb.x, kb.x, ka.w, l);
            tcell(mb.x, mb.y, kb.y, kb.x, l);
        }
        M[0] = ma;
        M[1] = mb;
        K[0] = ka;
        K[1] = kb;
    }
}

// g = I vel2 mu on the 4 cells z .. z+3 of line (y, x) (z % 4 == 0), from
// loaded values
__device__ __forceinline__ void gstore(const Bnd3AdjParams &p, int y, int z, int x, float4 m, float4 v) {
    const int n1 = p.g.n1, n2 = p.g.n2, n3 = p.g.n3;
    const long long c = ((long long)y * n2 + x) * n1 + z;
    const bool rest = x >= 4 && x < n2 - 4 && y >= 4 && y < n3 - 4;
    float4 o;
    o.x = (rest && z >= 4 && z < n1 - 4) ? v.x * m.x : 0.f;
    o.y = (rest && z + 1 >= 4 && z + 1 < n1 - 4) ? v.y * m.y : 0.f;
    o.z = (rest && z + 2 >= 4 && z + 2 < n1 - 4) ? v.z * m.z : 0.f;
    o.w = (rest && z + 3 >= 4 && z + 3 < n1 - 4) ? v.w * m.w : 0.f;
    __stcs(reinterpret_cast<float4 *>(p.gout + c), o);
}

__device__ __forceinline__ void gcells(const Bnd3AdjParams &p, int y, int z, int x) {
    const long long c = ((long long)y * p.g.n2 + x) * p.g.n1 + z;
    gstore(p, y, z, x, *reinterpret_cast<const float4 *>(p.mu + c), __ldg(reinterpret_cast<const float4 *>(p.vel2 + c)));
}

// g of a whole plane y, four groups of 4 cells per thread in flight
__device__ __forceinline__ void gplane(const Bnd3AdjParams &p, int y, int tid) {
    const int n1 = p.g.n1, n2 = p.g.n2, nq = n1 / 4, total = n2 * nq;
    const long long base = (long long)y * n2 * n1;
    for (int l0 = tid; l0 < total; l0 += 4 * b3::NT) {
        float4 m[4], v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int l = l0 + u * b3::NT;
            if (l < total) {
                const long long c = base + 4LL * l;  // line l / nq, cells 4 (l % nq) ..: contiguous in the plane
                m[u] = *reinterpret_cast<const float4 *>(p.mu + c);
                v[u] = __ldg(reinterpret_cast<const float4 *>(p.vel2 + c));
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int l = l0 + u * b3::NT;
            if (l < total) gstore(p, y, 4 * (l % nq), l / nq, m[u], v[u]);
        }
    }
}
}  // namespace b3a

__global__ void __launch_bounds__(b3::NT) k_bnd3_adj(const Bnd3AdjParams p) {
    using namespace b3;
    using namespace b3a;
    const int tid = threadIdx.x;
    const int n1 = p.g.n1, n2 = p.g.n2, n3 = p.g.n3;
    const long long s2 = n1, s3 = (long long)n1 * n2;
    int blk = blockIdx.x;

    if (blk < p.n_int) {  // ---- one plane without axis-3 face cells
        const int y = SHELL + blk;
        // fold the axis-2 bands (x < 6, x >= n2-6), every z
        for (int l = tid; l < 2 * SHELL * n1; l += NT) {
            const int k = l / n1, z = l % n1, x = k < SHELL ? k : n2 - 2 * SHELL + k;
            fold(p, (long long)y * s3 + (long long)x * s2 + z, z, x, y);
        }
        __syncthreads();
        // axis-2 lines (y, z)
        for (int z = tid; z < n1; z += NT) {
            const long long line = (long long)y * n1 + z;
            tline(p, (long long)y * s3 + z, s2, n2, __ldg(p.xl + line), __ldg(p.xh + line), true);
        }
        __syncthreads();
        // axis-1 ends, folded here for the lines outside the axis-2 bands
        for (int x = tid; x < n2; x += NT) zends(p, (long long)y * n2 + x, x, y, x >= SHELL && x < n2 - SHELL);
        __syncthreads();
        gplane(p, y, tid);
        return;
    }
    blk -= p.n_int;
    if (blk < 2 * p.nxr * p.nzr) {  // ---- face block
        const int f = blk / (p.nxr * p.nzr), r = blk % (p.nxr * p.nzr), xr = r / p.nzr, zr = r % p.nzr;
        const int xa = xr * XR, xb = xr == p.nxr - 1 ? n2 : xa + XR;
        const int za = zr * ZR, zb = zr == p.nzr - 1 ? n1 : za + ZR;
        const int ya = f == 0 ? 0 : n3 - SHELL;
        const int ncol = xb - xa, nz = zb - za;
        for (int l = tid; l < SHELL * ncol * nz; l += NT) {  // fold every cell (all in the axis-3 shell)
            const int y = ya + l / (ncol * nz), k = l % (ncol * nz), x = xa + k / nz, z = za + k % nz;
            fold(p, (long long)y * s3 + (long long)x * s2 + z, z, x, y);
        }
        __syncthreads();
        // axis 3: columns (x, z) of this block, the face planes only
        for (int l = tid; l < ncol * nz; l += NT) {
            const int x = xa + l / nz, z = za + l % nz;
            const long long c0 = (long long)x * s2 + z;
            const float b = __ldg((f == 0 ? p.yl : p.yh) + (long long)x * n1 + z);
            if (f == 0) {
                for (int i = 1; i <= 4; i++) {
                    const long long ci = c0 + i * s3, cb = ci + s3;
                    float mi = p.mu[ci], mb = p.mu[cb], kb = p.kap[cb], ki = p.kap[ci];
                    tcell(mi, mb, kb, ki, b);
                    p.mu[ci] = mi;
                    p.mu[cb] = mb;
                    p.kap[cb] = kb;
                    p.kap[ci] = ki;
                }
            } else {
                for (int i = n3 - 2; i >= n3 - 5; i--) {
                    const long long ci = c0 + i * s3, cb = ci - s3;
                    float mi = p.mu[ci], mb = p.mu[cb], kb = p.kap[cb], ki = p.kap[ci];
                    tcell(mi, mb, kb, ki, b);
                    p.mu[ci] = mi;
                    p.mu[cb] = mb;
                    p.kap[cb] = kb;
                    p.kap[ci] = ki;
                }
            }
        }
        __syncthreads();
        // axis 2: the x-ranges holding a face, lines (y, z) of this z-range
        const bool xlo = xr == 0, xhi = xr == p.nxr - 1;
        if (xlo || xhi)
            for (int l = tid; l < SHELL * nz; l += NT) {
                const int y = ya + l / nz, z = za + l % nz;
                const long long line = (long long)y * n1 + z, c0 = (long long)y * s3 + z;
                // a line's two faces belong to the first and the last x-range
                if (xlo && xhi) {
                    tline(p, c0, s2, n2, __ldg(p.xl + line), __ldg(p.xh + line), true);
                } else if (xhi) {
                    tline(p, c0, s2, n2, 0.f, __ldg(p.xh + line), false);
                } else {  // low face only: i = 1 .. 4
                    const float cl = __ldg(p.xl + line);
                    for (int i = 1; i <= 4; i++) {
                        const long long ci = c0 + i * s2, cb = ci + s2;
                        float mi = p.mu[ci], mb = p.mu[cb], kb = p.kap[cb], ki = p.kap[ci];
                        tcell(mi, mb, kb, ki, cl);
                        p.mu[ci] = mi;
                        p.mu[cb] = mb;
                        p.kap[cb] = kb;
                        p.kap[ci] = ki;
                    }
                }
            }
        __syncthreads();
        // axis 1: the line ends inside this z-range (already folded)
        const bool zlo = zr == 0, zhi = zr == p.nzr - 1;
        if (zlo && zhi) {
            for (int l = tid; l < SHELL * ncol; l += NT) {
                const int y = ya + l / ncol, x = xa + l % ncol;
                zends(p, (long long)y * n2 + x, x, y, false);
            }
        } else if (zlo || zhi) {
            for (int l = tid; l < SHELL * ncol; l += NT) {
                const int y = ya + l / ncol, x = xa + l % ncol;
                const long long line = (long long)y * n2 + x;
                if (zhi) {
                    tline(p, line * n1, 1, n1, 0.f, __ldg(p.zh + line), false);
                } else if (p.top) {
                    const float cl = __ldg(p.zl + line);
                    for (int i = 1; i <= 4; i++) {
                        const long long ci = line * n1 + i, cb = ci + 1;
                        float mi = p.mu[ci], mb = p.mu[cb], kb = p.kap[cb], ki = p.kap[ci];
                        tcell(mi, mb, kb, ki, cl);
                        p.mu[ci] = mi;
                        p.mu[cb] = mb;
                        p.kap[cb] = kb;
                        p.kap[ci] = ki;
                    }
                }
            }
        }
        __syncthreads();
        const int nq = nz / 4;
        for (int l = tid; l < SHELL * ncol * nq; l += NT) {
            const int y = ya + l / (ncol * nq), k = l % (ncol * nq);
            gcells(p, y, za + 4 * (k % nq), xa + k / nq);
        }
    }
}

void launch_bnd3_adj(Bnd3AdjParams p, cudaStream_t s) {
    using namespace b3;
    p.n_int = p.g.n3 - 2 * SHELL;
    p.nxr = p.g.n2 / XR > 0 ? p.g.n2 / XR : 1;
    p.nzr = p.g.n1 / ZR > 0 ? p.g.n1 / ZR : 1;
    k_bnd3_adj<<<p.n_int + 2 * p.nxr * p.nzr, NT, 0, s>>>(p);
}

}  // namespace awe
