// Kernels for the scheme of the reference's cartesian CPU programs
// (CODE/MAWEFDcart{2D,3D}cpu.c + ts_kernel.c + fdutil.c): 2N-order
// Laplacian, leapfrog in place over two time levels, Gaussian sponge,
// Clayton-Engquist one-way ABC, v^2 dt^2-scaled injection.
//
// Time levels.  The reference keeps u0 (previous, overwritten by the new
// level) and u1 (current); after the update and injection it applies the
// ABC to u0 and the sponge to both u0 and u1, then swaps.  Here the sponge of
// u1 is not written back: u1 is still being read by neighbouring cells, so
// its sponge is applied when the value is next read (as "prev" in the next
// step, or by the receiver gather / snapshot of this step).  The product is
// the same float multiplication on the same value, so results are unchanged.
// The new level is sponged in the step kernel except in the `shell` of cells
// that the one-way ABC rewrites or reads, which the boundary kernels finish.
#include <cuda_runtime.h>

#include "awe_internal.h"
#include "fp_exact.cuh"

namespace awe {

template <bool EXACT, int NDIM>
__device__ __forceinline__ float damp_cell(float v, int i1, int i2, int i3, const float *__restrict__ w1,
                                           const float *__restrict__ w2, const float *__restrict__ w3) {
    // sponge3d_apply order: axis-1 faces, then axis 2, then axis 3
    v = fmul<EXACT>(v, __ldg(w1 + i1));
    v = fmul<EXACT>(v, __ldg(w2 + i2));
    if constexpr (NDIM == 3) v = fmul<EXACT>(v, __ldg(w3 + i3));
    return v;
}

// One time step, one thread per cell (grid: x = axis-1 tiles, y = axis 2, z = axis 3).
template <int NOP, int NDIM, bool EXACT, bool RHO>
__global__ void __launch_bounds__(256) k_stepB(const float *__restrict__ cur, float *__restrict__ nxt,
                                               const float *__restrict__ vel, const float *__restrict__ rho,
                                               const StepBParams p) {
    // programmatic dependent launch (2D): wait for the previous grid before
    // touching memory (a no-op for an ordinary launch), then let the next
    // step's grid be scheduled once every block of this one has started
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;");
    const Grid g = p.g;
    const long long s2 = g.n1, s3 = (long long)g.n1 * g.n2;
    if (NDIM == 2 && p.ext_n > 0) {
        const int rows = (g.n2 + (int)blockDim.y - 1) / (int)blockDim.y;  // blocks of cells
        if ((int)blockIdx.y >= rows) {  // receiver gather of `cur`, lint2d_extract's order
            const int r = (((int)blockIdx.y - rows) * (int)gridDim.x + (int)blockIdx.x) * (int)(blockDim.x * blockDim.y) +
                          (int)(threadIdx.y * blockDim.x + threadIdx.x);
            if (r >= p.ext_n) return;
            const GeoPoint pt = p.ext[(long long)r * p.ext_stride];
            float acc = 0.f;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const long long n = pt.base + (c & 1) + (c >> 1) * s2;
                float v = __ldg(cur + n);
                if (p.damp_prev) v = damp_cell<EXACT, 2>(v, (int)(n % s2), (int)(n / s2), 0, p.w1, p.w2, p.w3);
                const float t = fmul<EXACT>(v, pt.w[c]);
                acc = (c == 0) ? t : fadd<EXACT>(acc, t);
            }
            p.ext_row[r] = acc;
            return;
        }
    }
    const int i1 = blockIdx.x * blockDim.x + threadIdx.x;
    const int i2 = blockIdx.y * blockDim.y + threadIdx.y;
    const int i3 = (NDIM == 3) ? (int)blockIdx.z : 0;
    if (i1 >= g.n1 || i2 >= g.n2) return;
    const long long i = i3 * s3 + i2 * s2 + i1;

    float prv = p.prv ? p.prv[i] : nxt[i];  // out of place when p.prv is set
    if (p.damp_prev) prv = damp_cell<EXACT, NDIM>(prv, i1, i2, i3, p.w1, p.w2, p.w3);

    bool interior = i1 >= NOP && i1 < g.n1 - NOP && i2 >= NOP && i2 < g.n2 - NOP;
    if (NDIM == 3) interior = interior && i3 >= NOP && i3 < g.n3 - NOP;
    float out = prv;
    if (interior) {
        const float u = cur[i];
        // ts_kernel.c:140-144 / :286-291: lap = u*c0 + sum_k [(z pair)*cz + (x pair)*cx (+ (y pair)*cy)]
        float lap = fmul<EXACT>(u, p.k.c0);
#pragma unroll
        for (int k = 1; k <= NOP; k++) {
            float t = fadd<EXACT>(fmul<EXACT>(fadd<EXACT>(__ldg(cur + i - k), __ldg(cur + i + k)), p.k.c[0][k]),
                                  fmul<EXACT>(fadd<EXACT>(__ldg(cur + i - k * s2), __ldg(cur + i + k * s2)),
                                              p.k.c[1][k]));
            if constexpr (NDIM == 3)
                t = fadd<EXACT>(
                    t, fmul<EXACT>(fadd<EXACT>(__ldg(cur + i - k * s3), __ldg(cur + i + k * s3)), p.k.c[2][k]));
            lap = fadd<EXACT>(lap, t);
        }
        if constexpr (RHO) {
            // variable density, ts_kernel.c:145-155 / :292-305
            float duz = 0.f, dux = 0.f, duy = 0.f, drz = 0.f, drx = 0.f, dry = 0.f;
#pragma unroll
            for (int k = 1; k <= NOP; k++) {
                duz = fadd<EXACT>(duz, fmul<EXACT>(fsub<EXACT>(__ldg(cur + i + k), __ldg(cur + i - k)), p.k.b[0][k]));
                dux = fadd<EXACT>(
                    dux, fmul<EXACT>(fsub<EXACT>(__ldg(cur + i + k * s2), __ldg(cur + i - k * s2)), p.k.b[1][k]));
                drz = fadd<EXACT>(drz, fmul<EXACT>(fsub<EXACT>(__ldg(rho + i + k), __ldg(rho + i - k)), p.k.b[0][k]));
                drx = fadd<EXACT>(
                    drx, fmul<EXACT>(fsub<EXACT>(__ldg(rho + i + k * s2), __ldg(rho + i - k * s2)), p.k.b[1][k]));
                if constexpr (NDIM == 3) {
                    duy = fadd<EXACT>(
                        duy, fmul<EXACT>(fsub<EXACT>(__ldg(cur + i + k * s3), __ldg(cur + i - k * s3)), p.k.b[2][k]));
                    dry = fadd<EXACT>(
                        dry, fmul<EXACT>(fsub<EXACT>(__ldg(rho + i + k * s3), __ldg(rho + i - k * s3)), p.k.b[2][k]));
                }
            }
            float dot = fadd<EXACT>(fmul<EXACT>(duz, drz), fmul<EXACT>(dux, drx));
            if constexpr (NDIM == 3) dot = fadd<EXACT>(dot, fmul<EXACT>(duy, dry));
            float q = EXACT ? __fdiv_rn(dot, __ldg(rho + i)) : dot / __ldg(rho + i);
            lap = fsub<EXACT>(lap, q);
        }
        const float q = fmul<EXACT>(__ldg(vel + i), lap);
        if constexpr (EXACT)
            out = sum3_rn(q, __fadd_rn(u, u), -prv);
        else
            out = fmaf(__ldg(vel + i), lap, 2.f * u - prv);
    }
    if (p.sponge_new) {
        bool raw = false;
        if (p.shell > 0) {
            const int s = p.shell;
            raw = i1 < s || i1 >= g.n1 - s || i2 < s || i2 >= g.n2 - s;
            if (NDIM == 3) raw = raw || i3 < s || i3 >= g.n3 - s;
        }
        if (!raw) out = damp_cell<EXACT, NDIM>(out, i1, i2, i3, p.w1, p.w2, p.w3);
    }
    if (NDIM == 2 && p.inj_n > 0) {  // lint2d_inject_with_vv, sources and corners in order
        for (int sidx = 0; sidx < p.inj_n; sidx++) {
            const long long b0 = p.inj[(long long)sidx * p.inj_stride].base - i;
            if (b0 < -(s2 + 1) || b0 > 0) continue;  // corners are base + {0, 1, s2, s2 + 1}
            const GeoPoint pt = p.inj[(long long)sidx * p.inj_stride];
            const float dd = p.inj_one ? p.inj_wav[(long long)p.inj_it * p.inj_ncs]
                                       : p.inj_wav[(long long)p.inj_it * p.inj_ncs + sidx];
#pragma unroll
            for (int c = 0; c < 4; c++)
                if (pt.base + (c & 1) + (c >> 1) * s2 == i)
                    out = fadd<EXACT>(out, fmul<EXACT>(fmul<EXACT>(dd, pt.w[c]), __ldg(vel + i)));
        }
    }
    nxt[i] = out;
}

template <int NOP, int NDIM, bool EXACT>
static void dispatch_rho(bool rho, const float *cur, float *nxt, const float *vel, const float *den,
                         const StepBParams &p, cudaStream_t s) {
    dim3 block(64, 4, 1);
    dim3 grid((p.g.n1 + 63) / 64, (p.g.n2 + 3) / 4, NDIM == 3 ? p.g.n3 : 1);
    if (NDIM == 2 && p.ext_n > 0)  // extra rows of blocks gather the receivers
        grid.y += (unsigned)((p.ext_n + grid.x * 256 - 1) / (grid.x * 256));
    if (NDIM == 2) {  // launch-bound steps: programmatic dependent launch hides the launch gap
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = grid;
        cfg.blockDim = block;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if (rho) cudaLaunchKernelEx(&cfg, k_stepB<NOP, NDIM, EXACT, true>, cur, nxt, vel, den, p);
        else cudaLaunchKernelEx(&cfg, k_stepB<NOP, NDIM, EXACT, false>, cur, nxt, vel, den, p);
        return;
    }
    if (rho)
        k_stepB<NOP, NDIM, EXACT, true><<<grid, block, 0, s>>>(cur, nxt, vel, den, p);
    else
        k_stepB<NOP, NDIM, EXACT, false><<<grid, block, 0, s>>>(cur, nxt, vel, den, p);
}

template <int NOP>
static void dispatch_dim(int ndim, bool exact, bool rho, const float *cur, float *nxt, const float *vel,
                         const float *den, const StepBParams &p, cudaStream_t s) {
    if (ndim == 3) {
        if (exact) dispatch_rho<NOP, 3, true>(rho, cur, nxt, vel, den, p, s);
        else dispatch_rho<NOP, 3, false>(rho, cur, nxt, vel, den, p, s);
    } else {
        if (exact) dispatch_rho<NOP, 2, true>(rho, cur, nxt, vel, den, p, s);
        else dispatch_rho<NOP, 2, false>(rho, cur, nxt, vel, den, p, s);
    }
}

void launch_stepB(int ndim, int nop, bool exact, bool rho, const float *cur, float *nxt, const float *vel,
                  const float *den, const StepBParams &p, cudaStream_t s) {
    switch (nop) {
        case 1: dispatch_dim<1>(ndim, exact, rho, cur, nxt, vel, den, p, s); break;
        case 2: dispatch_dim<2>(ndim, exact, rho, cur, nxt, vel, den, p, s); break;
        case 3: dispatch_dim<3>(ndim, exact, rho, cur, nxt, vel, den, p, s); break;
        case 4: dispatch_dim<4>(ndim, exact, rho, cur, nxt, vel, den, p, s); break;
        case 5: dispatch_dim<5>(ndim, exact, rho, cur, nxt, vel, den, p, s); break;
        case 6: dispatch_dim<6>(ndim, exact, rho, cur, nxt, vel, den, p, s); break;
        case 7: dispatch_dim<7>(ndim, exact, rho, cur, nxt, vel, den, p, s); break;
        case 8: dispatch_dim<8>(ndim, exact, rho, cur, nxt, vel, den, p, s); break;
        case 9: dispatch_dim<9>(ndim, exact, rho, cur, nxt, vel, den, p, s); break;
        case 10: dispatch_dim<10>(ndim, exact, rho, cur, nxt, vel, den, p, s); break;
        default: break;
    }
}

// ---------------------------------------------------------------------------
// One-way ABC, abcone3d_apply (fdutil.c:2085-2177): three passes (axis 1,
// axis 2, axis 3 faces), each a sequential sweep outward per line, as the
// reference; a pass completes before the next reads its corners.
template <bool EXACT>
__device__ __forceinline__ float abc_update(float um_in, float um_c, float uo_in, float b) {
    // uo = um[inner] + (um[c] - uo[inner]) * b
    return fadd<EXACT>(um_in, fmul<EXACT>(fsub<EXACT>(um_c, uo_in), b));
}

template <bool EXACT>
__global__ void k_abc_axis1(float *__restrict__ uo, const float *__restrict__ um, const float *__restrict__ bl,
                            const float *__restrict__ bh, Grid g, int nop, int top) {
    const int line = blockIdx.x * blockDim.x + threadIdx.x;  // (i3, i2)
    if (line >= g.n2 * g.n3) return;
    const long long c = (long long)line * g.n1;
    const float l = bl[line], h = bh[line];
    // the sweep keeps the value it just wrote in a register (the next cell
    // reads it), so each face costs one pass over its nop+2 samples; the two
    // faces touch disjoint samples, so their order does not matter
    if (top) {
        float next = uo[c + nop + 1];
        for (int iz = nop; iz >= 1; iz--) {
            next = abc_update<EXACT>(um[c + iz + 1], um[c + iz], next, l);
            uo[c + iz] = next;
        }
    }
    float prev = uo[c + g.n1 - nop - 2];
    for (int iz = g.n1 - nop - 1; iz <= g.n1 - 2; iz++) {
        prev = abc_update<EXACT>(um[c + iz - 1], um[c + iz], prev, h);
        uo[c + iz] = prev;
    }
}

// The same sweep for nop == 4 and n1 % 4 == 0, n1 >= 16, with 16-byte
// accesses: a face reads and writes inside the first (last) two float4 of
// its line; the one sample of those float4s the face does not update is
// stored back unchanged (no other thread of the launch touches the line).
// With sponge tables given (w1 != null), lines at least `band` from the
// axis-2 and axis-3 faces - which the later ABC passes neither read nor
// write - also get the sponge of their axis-1 ends (the first and last
// `band` <= 8 samples) here, as the band sponge would after the ABC.
template <bool EXACT>
__device__ __forceinline__ void damp_end(float4 &v, int i1, int lo, int hi, int i2, int i3, const float *w1,
                                         const float *w2, const float *w3) {
    float *e = &v.x;
#pragma unroll
    for (int j = 0; j < 4; j++)
        if (i1 + j >= lo && i1 + j < hi) e[j] = damp_cell<EXACT, 3>(e[j], i1 + j, i2, i3, w1, w2, w3);
}

template <bool EXACT>
__global__ void k_abc_axis1_v4(float *__restrict__ uo, const float *__restrict__ um, const float *__restrict__ bl,
                               const float *__restrict__ bh, Grid g, int top, const float *__restrict__ w1,
                               const float *__restrict__ w2, const float *__restrict__ w3, int band) {
    const int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= g.n2 * g.n3) return;
    const int q = g.n1 / 4, i2 = line % g.n2, i3 = line / g.n2;
    const bool sp = w1 && i2 >= band && i2 < g.n2 - band && i3 >= band && i3 < g.n3 - band;
    const float4 *m = reinterpret_cast<const float4 *>(um + (long long)line * g.n1);
    float4 *o = reinterpret_cast<float4 *>(uo + (long long)line * g.n1);
    if (top || sp) {  // iz = 4, 3, 2, 1 from uo[5]
        float4 oa = o[0], ob = o[1];
        if (top) {
            const float l = bl[line];
            const float4 ma = m[0], mb = m[1];
            const float u4 = abc_update<EXACT>(mb.y, mb.x, ob.y, l);
            const float u3 = abc_update<EXACT>(mb.x, ma.w, u4, l);
            const float u2 = abc_update<EXACT>(ma.w, ma.z, u3, l);
            const float u1 = abc_update<EXACT>(ma.z, ma.y, u2, l);
            oa = make_float4(oa.x, u1, u2, u3);
            ob = make_float4(u4, ob.y, ob.z, ob.w);
        }
        if (sp) {
            damp_end<EXACT>(oa, 0, 0, band, i2, i3, w1, w2, w3);
            damp_end<EXACT>(ob, 4, 0, band, i2, i3, w1, w2, w3);
        }
        o[0] = oa;
        o[1] = ob;
    }
    {  // iz = n1-5 .. n1-2 from uo[n1-6]
        const float h = bh[line];
        const float4 ma = m[q - 2], mb = m[q - 1];
        const float4 oa = o[q - 2], ob = o[q - 1];
        const float v5 = abc_update<EXACT>(ma.z, ma.w, oa.z, h);
        const float v4 = abc_update<EXACT>(ma.w, mb.x, v5, h);
        const float v3 = abc_update<EXACT>(mb.x, mb.y, v4, h);
        const float v2 = abc_update<EXACT>(mb.y, mb.z, v3, h);
        float4 na = make_float4(oa.x, oa.y, oa.z, v5), nb = make_float4(v4, v3, v2, ob.w);
        if (sp) {
            damp_end<EXACT>(na, g.n1 - 8, g.n1 - band, g.n1, i2, i3, w1, w2, w3);
            damp_end<EXACT>(nb, g.n1 - 4, g.n1 - band, g.n1, i2, i3, w1, w2, w3);
        }
        o[q - 2] = na;
        o[q - 1] = nb;
    }
}

// axis-2 faces: one thread per (i3, i1); coefficients [n3][n1]
template <bool EXACT>
__global__ void k_abc_axis2(float *uo, const float *__restrict__ um, const float *__restrict__ bl,
                            const float *__restrict__ bh, Grid g, int nop) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.n1 * g.n3) return;
    const long long i3 = t / g.n1, i1 = t % g.n1;
    const long long s2 = g.n1, base = i3 * g.n1 * (long long)g.n2 + i1;
    const float l = bl[t], h = bh[t];
    for (int iop = 0; iop < nop; iop++) {
        long long c = base + (long long)(nop - iop) * s2;
        uo[c] = abc_update<EXACT>(um[c + s2], um[c], uo[c + s2], l);
        c = base + (long long)(g.n2 - nop + iop - 1) * s2;
        uo[c] = abc_update<EXACT>(um[c - s2], um[c], uo[c - s2], h);
    }
}

// axis-3 faces: one thread per (i2, i1); coefficients [n2][n1]
template <bool EXACT>
__global__ void k_abc_axis3(float *uo, const float *__restrict__ um, const float *__restrict__ bl,
                            const float *__restrict__ bh, Grid g, int nop) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.n1 * g.n2) return;
    const long long s3 = (long long)g.n1 * g.n2;
    const float l = bl[t], h = bh[t];
    for (int iop = 0; iop < nop; iop++) {
        long long c = (long long)(nop - iop) * s3 + t;
        uo[c] = abc_update<EXACT>(um[c + s3], um[c], uo[c + s3], l);
        c = (long long)(g.n3 - nop + iop - 1) * s3 + t;
        uo[c] = abc_update<EXACT>(um[c - s3], um[c], uo[c - s3], h);
    }
}

bool abc_zfused(int nop, const Grid &g, int band) {
    return nop == 4 && g.n1 % 4 == 0 && g.n1 >= 16 && band > 0 && band <= 8;
}

void launch_abconeB(int ndim, int nop, bool exact, int fsrf, float *uo, const float *um, const AbcB &a,
                    const Grid &g, cudaStream_t s, const float *w1, const float *w2, const float *w3, int band) {
    const int T = 128;
    long long n = (long long)g.n2 * g.n3;
    if (nop == 4 && g.n1 % 4 == 0 && g.n1 >= 16) {
        if (!abc_zfused(nop, g, band)) w1 = nullptr;
        if (exact)
            k_abc_axis1_v4<true><<<(n + T - 1) / T, T, 0, s>>>(uo, um, a.zl, a.zh, g, !fsrf, w1, w2, w3, band);
        else
            k_abc_axis1_v4<false><<<(n + T - 1) / T, T, 0, s>>>(uo, um, a.zl, a.zh, g, !fsrf, w1, w2, w3, band);
    } else if (exact) {
        k_abc_axis1<true><<<(n + T - 1) / T, T, 0, s>>>(uo, um, a.zl, a.zh, g, nop, !fsrf);
    } else {
        k_abc_axis1<false><<<(n + T - 1) / T, T, 0, s>>>(uo, um, a.zl, a.zh, g, nop, !fsrf);
    }
    n = (long long)g.n1 * g.n3;
    if (exact) k_abc_axis2<true><<<(n + T - 1) / T, T, 0, s>>>(uo, um, a.xl, a.xh, g, nop);
    else k_abc_axis2<false><<<(n + T - 1) / T, T, 0, s>>>(uo, um, a.xl, a.xh, g, nop);
    if (ndim == 3) {
        n = (long long)g.n1 * g.n2;
        if (exact) k_abc_axis3<true><<<(n + T - 1) / T, T, 0, s>>>(uo, um, a.yl, a.yh, g, nop);
        else k_abc_axis3<false><<<(n + T - 1) / T, T, 0, s>>>(uo, um, a.yl, a.yh, g, nop);
    }
}

// ---------------------------------------------------------------------------
// Hybrid one-way ABC (apply_abc, MAWEFDcart2Dcpu.c:553-614 and
// MAWEFDcart3Dcpu.c:533-625): the A1 update on the outer nop layers, then a
// blend of the A1 value and the field over the next nbd-nop layers with
// weights damp[ib]; free surface zeroes the first nbd+1 samples of axis 1.
template <bool EXACT>
__device__ __forceinline__ float blend(float bc, float u, float d) {
    return fadd<EXACT>(fmul<EXACT>(bc, fsub<EXACT>(1.f, d)), fmul<EXACT>(u, d));
}

template <bool EXACT>
__global__ void k_hybrid_axis(float *u2, const float *__restrict__ u1, const float *__restrict__ bl,
                              const float *__restrict__ bh, const float *__restrict__ damp, Grid g, int axis,
                              int nop, int nbd, int fsrf) {
    // one thread per line along `axis`; line index enumerates the other two axes
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long nlines, base, stride;
    int n;
    if (axis == 1) {
        nlines = (long long)g.n2 * g.n3;
        if (t >= nlines) return;
        base = t * g.n1;
        stride = 1;
        n = g.n1;
    } else if (axis == 2) {
        nlines = (long long)g.n1 * g.n3;
        if (t >= nlines) return;
        base = (t / g.n1) * g.n1 * (long long)g.n2 + t % g.n1;
        stride = g.n1;
        n = g.n2;
    } else {
        nlines = (long long)g.n1 * g.n2;
        if (t >= nlines) return;
        base = t;
        stride = (long long)g.n1 * g.n2;
        n = g.n3;
    }
    const float l = bl[t], h = bh[t];
#define AT(a, k) a[base + (long long)(k) * stride]
    for (int ib = nbd - nop; ib < nbd; ib++) {
        int k = nbd - ib - 1;
        AT(u2, k) = abc_update<EXACT>(AT(u1, k + 1), AT(u1, k), AT(u2, k + 1), l);
        k = n - nbd + ib;
        AT(u2, k) = abc_update<EXACT>(AT(u1, k - 1), AT(u1, k), AT(u2, k - 1), h);
    }
    if (damp)
        for (int ib = 0; ib < nbd - nop; ib++) {
            const float d = damp[ib];
            int k = nbd - ib - 1;
            float bc = abc_update<EXACT>(AT(u1, k + 1), AT(u1, k), AT(u2, k + 1), l);
            AT(u2, k) = blend<EXACT>(bc, AT(u2, k), d);
            k = n - nbd + ib;
            bc = abc_update<EXACT>(AT(u1, k - 1), AT(u1, k), AT(u2, k - 1), h);
            AT(u2, k) = blend<EXACT>(bc, AT(u2, k), d);
        }
    if (axis == 1 && fsrf)
        for (int k = 0; k < nbd + 1; k++) AT(u2, k) = 0.f;
#undef AT
}

void launch_hybridB(int ndim, int nop, int nbd, bool exact, int fsrf, float *uo, const float *um, const AbcB &a,
                    const float *damp, const Grid &g, cudaStream_t s) {
    const int T = 128;
    const float *lo[3] = {a.zl, a.xl, a.yl}, *hi[3] = {a.zh, a.xh, a.yh};
    long long nl[3] = {(long long)g.n2 * g.n3, (long long)g.n1 * g.n3, (long long)g.n1 * g.n2};
    for (int ax = 1; ax <= ndim; ax++) {
        long long n = nl[ax - 1];
        if (exact)
            k_hybrid_axis<true><<<(n + T - 1) / T, T, 0, s>>>(uo, um, lo[ax - 1], hi[ax - 1], damp, g, ax, nop, nbd,
                                                              fsrf);
        else
            k_hybrid_axis<false><<<(n + T - 1) / T, T, 0, s>>>(uo, um, lo[ax - 1], hi[ax - 1], damp, g, ax, nop,
                                                               nbd, fsrf);
    }
}

// ---------------------------------------------------------------------------
// Sponge over the cells within `width` of any face, each cell exactly once:
// axis-1 slabs (every line), then axis-2 slabs (axis-1 interior), then
// axis-3 slabs (axis-1 and axis-2 interior).  32-bit index arithmetic; the
// axis-2 and axis-3 parts run along axis 1 so their accesses coalesce.
template <bool EXACT, int NDIM>
__global__ void k_sponge_slab1(float *u, const float *__restrict__ w1, const float *__restrict__ w2,
                               const float *__restrict__ w3, Grid g, int W) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int per = 2 * W;
    if (t >= g.n2 * g.n3 * per) return;
    const int line = t / per, k = t - line * per;
    const int i1 = k < W ? k : g.n1 - per + k, i2 = line % g.n2, i3 = line / g.n2;
    const long long i = (long long)line * g.n1 + i1;
    u[i] = damp_cell<EXACT, NDIM>(u[i], i1, i2, i3, w1, w2, w3);
}

template <bool EXACT, int NDIM>
__global__ void k_sponge_slab2(float *u, const float *__restrict__ w1, const float *__restrict__ w2,
                               const float *__restrict__ w3, Grid g, int W) {
    const int i1 = W + blockIdx.x * blockDim.x + threadIdx.x;
    if (i1 >= g.n1 - W) return;
    const int k = blockIdx.y, i2 = k < W ? k : g.n2 - 2 * W + k, i3 = blockIdx.z;
    const long long i = ((long long)i3 * g.n2 + i2) * g.n1 + i1;
    u[i] = damp_cell<EXACT, NDIM>(u[i], i1, i2, i3, w1, w2, w3);
}

template <bool EXACT>
__global__ void k_sponge_slab3(float *u, const float *__restrict__ w1, const float *__restrict__ w2,
                               const float *__restrict__ w3, Grid g, int W) {
    const int i1 = W + blockIdx.x * blockDim.x + threadIdx.x;
    if (i1 >= g.n1 - W) return;
    const int i2 = W + blockIdx.y, k = blockIdx.z, i3 = k < W ? k : g.n3 - 2 * W + k;
    const long long i = ((long long)i3 * g.n2 + i2) * g.n1 + i1;
    u[i] = damp_cell<EXACT, 3>(u[i], i1, i2, i3, w1, w2, w3);
}

// The same three slabs with 16-byte accesses (n1 % 4 == 0): one thread per
// float4, lanes outside the slab's axis-1 range are stored back unchanged
// (no other thread of the launch touches them).
template <bool EXACT, int NDIM>
__device__ __forceinline__ void damp4(float4 &v, int i1, int lo, int hi, int i2, int i3, const float *w1,
                                      const float *w2, const float *w3) {
    float *e = &v.x;
#pragma unroll
    for (int j = 0; j < 4; j++)
        if (i1 + j >= lo && i1 + j < hi) e[j] = damp_cell<EXACT, NDIM>(e[j], i1 + j, i2, i3, w1, w2, w3);
}

template <bool EXACT, int NDIM>
__global__ void k_sponge_slab1_v4(float *u, const float *__restrict__ w1, const float *__restrict__ w2,
                                  const float *__restrict__ w3, Grid g, int W, int zfused) {
    // per line: chunks [0, c) cover axis-1 cells [0, W), chunks [q - c, q) cover [n1 - W, n1)
    const int q = g.n1 / 4, c = (W + 3) / 4;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.n2 * g.n3 * 2 * c) return;
    const int line = (int)(t / (2 * c)), k = (int)(t - (long long)line * 2 * c);
    const int chunk = k < c ? k : q - 2 * c + k;
    const int i2 = line % g.n2, i3 = line / g.n2, i1 = 4 * chunk;
    // lines away from the axis-2/3 bands were finished by the fused axis-1 ABC pass
    if (zfused && i2 >= W && i2 < g.n2 - W && i3 >= W && i3 < g.n3 - W) return;
    float4 *p = reinterpret_cast<float4 *>(u + (long long)line * g.n1) + chunk;
    float4 v = *p;
    if (k < c) damp4<EXACT, NDIM>(v, i1, 0, W, i2, i3, w1, w2, w3);
    else damp4<EXACT, NDIM>(v, i1, g.n1 - W, g.n1, i2, i3, w1, w2, w3);
    *p = v;
}

// slab2 (NDIM 3: axis-2 bands; NDIM 2: the same) and slab3 (axis-3 bands)
// over axis-1 cells [W, n1 - W), chunk-aligned
template <bool EXACT, int NDIM, int SLAB>
__global__ void k_sponge_slab23_v4(float *u, const float *__restrict__ w1, const float *__restrict__ w2,
                                   const float *__restrict__ w3, Grid g, int W) {
    const int c0 = W / 4, c1 = (g.n1 - W + 3) / 4;
    const int chunk = c0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (chunk >= c1) return;
    int i2, i3;
    if (SLAB == 2) {
        const int k = blockIdx.y;
        i2 = k < W ? k : g.n2 - 2 * W + k;
        i3 = blockIdx.z;
    } else {
        i2 = W + blockIdx.y;
        const int k = blockIdx.z;
        i3 = k < W ? k : g.n3 - 2 * W + k;
    }
    float4 *p = reinterpret_cast<float4 *>(u + ((long long)i3 * g.n2 + i2) * g.n1) + chunk;
    float4 v = *p;
    damp4<EXACT, NDIM>(v, 4 * chunk, W, g.n1 - W, i2, i3, w1, w2, w3);
    *p = v;
}

template <bool EXACT, int NDIM>
static void band_sponge_t(int W, float *u, const float *w1, const float *w2, const float *w3, const Grid &g,
                          cudaStream_t s, int zfused) {
    const int T = 128;
    if (g.n1 % 4 == 0 && g.n1 >= 2 * W + 8) {
        const int c = (W + 3) / 4;
        const long long n1tot = (long long)g.n2 * g.n3 * 2 * c;
        k_sponge_slab1_v4<EXACT, NDIM><<<(unsigned)((n1tot + 255) / 256), 256, 0, s>>>(u, w1, w2, w3, g, W,
                                                                                       NDIM == 3 ? zfused : 0);
        const int nch = (g.n1 - W + 3) / 4 - W / 4;
        k_sponge_slab23_v4<EXACT, NDIM, 2><<<dim3((nch + 63) / 64, 2 * W, g.n3), 64, 0, s>>>(u, w1, w2, w3, g, W);
        if (NDIM == 3 && g.n2 - 2 * W > 0)
            k_sponge_slab23_v4<EXACT, 3, 3><<<dim3((nch + 63) / 64, g.n2 - 2 * W, 2 * W), 64, 0, s>>>(u, w1, w2, w3,
                                                                                                   g, W);
        return;
    }
    const long long n1tot = (long long)g.n2 * g.n3 * 2 * W;
    k_sponge_slab1<EXACT, NDIM><<<(unsigned)((n1tot + 255) / 256), 256, 0, s>>>(u, w1, w2, w3, g, W);
    const int inner1 = g.n1 - 2 * W;
    if (inner1 <= 0) return;
    k_sponge_slab2<EXACT, NDIM><<<dim3((inner1 + T - 1) / T, 2 * W, g.n3), T, 0, s>>>(u, w1, w2, w3, g, W);
    if (NDIM == 3 && g.n2 - 2 * W > 0)
        k_sponge_slab3<EXACT><<<dim3((inner1 + T - 1) / T, g.n2 - 2 * W, 2 * W), T, 0, s>>>(u, w1, w2, w3, g, W);
}

void launch_band_sponge(int ndim, int width, bool exact, float *u, const float *w1, const float *w2, const float *w3,
                        const Grid &g, cudaStream_t s, int zfused) {
    if (ndim == 3) {
        if (exact) band_sponge_t<true, 3>(width, u, w1, w2, w3, g, s, zfused);
        else band_sponge_t<false, 3>(width, u, w1, w2, w3, g, s, zfused);
    } else {
        if (exact) band_sponge_t<true, 2>(width, u, w1, w2, w3, g, s, 0);
        else band_sponge_t<false, 2>(width, u, w1, w2, w3, g, s, 0);
    }
}

// ---------------------------------------------------------------------------
// Injection into the new level, lint{2,3}d_inject[1]_with_vv
// (fdutil.c:1688-1740): u[node] += (dd * w) * vel[node], sources and corners
// in the reference's order (one thread, so coincident nodes add in order).
template <bool EXACT>
__global__ void k_injectB(float *u, const float *__restrict__ vel, const GeoPoint *__restrict__ pts, int ns,
                          const float *__restrict__ wav, int it, int ncs, int one_wavelet, int ncorner,
                          const long long *__restrict__ off, int stride) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int s = 0; s < ns; s++) {
        const float dd = one_wavelet ? wav[(long long)it * ncs] : wav[(long long)it * ncs + s];
        const GeoPoint pt = pts[(long long)s * stride];
        for (int c = 0; c < ncorner; c++) {
            const long long n = pt.base + off[c];
            u[n] = fadd<EXACT>(u[n], fmul<EXACT>(fmul<EXACT>(dd, pt.w[c]), vel[n]));
        }
    }
}

// ---------------------------------------------------------------------------
// Receiver gather, lint{2,3}d_extract (fdutil.c:1596-1670):
// d = sum_c u[node_c] * w_c, summed in corner order.
template <bool EXACT, int NDIM>
__global__ void k_extract(const float *__restrict__ u, const GeoPoint *__restrict__ pts, int nr, float *dat,
                          const float *__restrict__ w1, const float *__restrict__ w2, const float *__restrict__ w3,
                          Grid g, const long long *__restrict__ off, int stride) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nr) return;
    const GeoPoint pt = pts[(long long)r * stride];
    constexpr int NC = NDIM == 3 ? 8 : 4;
    float acc = 0.f;
#pragma unroll
    for (int c = 0; c < NC; c++) {
        const long long n = pt.base + off[c];
        float v = __ldg(u + n);
        if (w1) {
            const long long s3 = (long long)g.n1 * g.n2;
            const int i3 = (int)(n / s3), rem = (int)(n % s3);
            v = damp_cell<EXACT, NDIM>(v, rem % g.n1, rem / g.n1, i3, w1, w2, w3);
        }
        const float t = fmul<EXACT>(v, pt.w[c]);
        acc = (c == 0) ? t : fadd<EXACT>(acc, t);
    }
    dat[r] = acc;
}

void launch_injectB_off(int ndim, bool exact, float *u, const float *vel, const GeoPoint *pts, int ns,
                        const float *wav, int it, int ncs, bool one_wavelet, const long long *off, cudaStream_t s,
                        int stride) {
    if (ns <= 0) return;
    const int nc = ndim == 3 ? 8 : 4;
    if (exact) k_injectB<true><<<1, 32, 0, s>>>(u, vel, pts, ns, wav, it, ncs, one_wavelet, nc, off, stride);
    else k_injectB<false><<<1, 32, 0, s>>>(u, vel, pts, ns, wav, it, ncs, one_wavelet, nc, off, stride);
}

void launch_extract_off(int ndim, bool exact, const float *u, const GeoPoint *pts, int nr, float *dat_row,
                        const float *w1, const float *w2, const float *w3, const Grid &g, const long long *off,
                        cudaStream_t s, int stride) {
    if (nr <= 0) return;
    const int T = 128, B = (nr + T - 1) / T;
    if (ndim == 3) {
        if (exact) k_extract<true, 3><<<B, T, 0, s>>>(u, pts, nr, dat_row, w1, w2, w3, g, off, stride);
        else k_extract<false, 3><<<B, T, 0, s>>>(u, pts, nr, dat_row, w1, w2, w3, g, off, stride);
    } else {
        if (exact) k_extract<true, 2><<<B, T, 0, s>>>(u, pts, nr, dat_row, w1, w2, w3, g, off, stride);
        else k_extract<false, 2><<<B, T, 0, s>>>(u, pts, nr, dat_row, w1, w2, w3, g, off, stride);
    }
}

// ---------------------------------------------------------------------------
// Snapshot: window [f .. f+m) of the padded grid (m = padded size for
// bnds=y), pending sponge applied.
template <int NDIM>
__global__ void k_snapshot(const float *__restrict__ u, float *__restrict__ dst, Grid g, int f1, int f2, int f3,
                           int m1, int m2, int m3, const float *__restrict__ w1, const float *__restrict__ w2,
                           const float *__restrict__ w3) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m1 * m2 * m3) return;
    const int j1 = (int)(t % m1), j2 = (int)((t / m1) % m2), j3 = (int)(t / ((long long)m1 * m2));
    const int i1 = f1 + j1, i2 = f2 + j2, i3 = f3 + j3;
    float v = u[((long long)i3 * g.n2 + i2) * g.n1 + i1];
    if (w1) v = damp_cell<true, NDIM>(v, i1, i2, i3, w1, w2, w3);
    dst[t] = v;
}

void launch_snapshot(int ndim, const float *u, float *dst, const Grid &g, int f1, int f2, int f3, int m1, int m2,
                     int m3, const float *w1, const float *w2, const float *w3, cudaStream_t s) {
    const long long n = (long long)m1 * m2 * m3;
    const int T = 256;
    if (ndim == 3) k_snapshot<3><<<(n + T - 1) / T, T, 0, s>>>(u, dst, g, f1, f2, f3, m1, m2, m3, w1, w2, w3);
    else k_snapshot<2><<<(n + T - 1) / T, T, 0, s>>>(u, dst, g, f1, f2, f3, m1, m2, m3, w1, w2, w3);
}

}  // namespace awe
