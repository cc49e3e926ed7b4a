// Model preparation of the CPU-program scheme on the device, from the model
// as the caller passes it ([n3][n2][n1], axis 1 fastest):
//  * padding by edge replication (expand2d / expand3d, fdutil.c:435-571): a
//    padded cell takes the model cell at its coordinates clamped to the model;
//  * v^2 dt^2 (MAWEFDcart2Dcpu.c:290-291) and, with a free surface, zero on
//    the first nb+1 samples of every axis-1 line (:292-295);
//  * the one-way ABC coefficients b = (1 - v dt/d) / (1 + v dt/d) at the first
//    interior sample of each face (abcone2d_make / abcone3d_make,
//    fdutil.c:1919-2019).
// Every value is formed with the same IEEE float operations in the same
// order as the host restatement (multiply, divide, subtract and add each
// rounded once, no contraction), so the tables are bit-identical to it.
#include <cuda_runtime.h>

#include "awe_internal.h"

namespace awe {

namespace {

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// model value at padded coordinates (i1, i2, i3)
__device__ __forceinline__ float model_at(const float *__restrict__ raw, const ModelPrep &m, int i1, int i2, int i3) {
    const int r1 = clampi(i1 - m.nb, 0, m.n1 - 1), r2 = clampi(i2 - m.nb, 0, m.n2 - 1);
    const int r3 = m.nd == 3 ? clampi(i3 - m.nb, 0, m.n3 - 1) : 0;
    return __ldg(raw + ((long long)r3 * m.n2 + r2) * m.n1 + r1);
}

__global__ void k_model_pad(const float *__restrict__ raw, float *__restrict__ out, const ModelPrep m, int vel2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long cells = (long long)m.g.n1 * m.g.n2 * m.g.n3;
    if (i >= cells) return;
    const int i1 = (int)(i % m.g.n1);
    const long long r = i / m.g.n1;
    const int i2 = (int)(r % m.g.n2), i3 = (int)(r / m.g.n2);
    float v = model_at(raw, m, i1, i2, i3);
    if (vel2) {
        v = __fmul_rn(v, __fmul_rn(v, m.dt2));
        if (i1 < m.zero1) v = 0.f;
    }
    out[i] = v;
}

__device__ __forceinline__ float abc_coef(float v, float dt, float dd) {
    const float q = __fdiv_rn(__fmul_rn(v, dt), dd);
    return __fdiv_rn(__fsub_rn(1.f, q), __fadd_rn(1.f, q));
}

// blockIdx.y: 0 the axis-1 faces over (i3, i2), 1 the axis-2 faces over
// (i3, i1), 2 the axis-3 faces over (i2, i1)
__global__ void k_model_abc(const float *__restrict__ raw, const ModelPrep m, float *zl, float *zh, float *xl,
                            float *xh, float *yl, float *yh) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const Grid g = m.g;
    const int nb = m.nb;
    if (blockIdx.y == 0) {
        if (t >= (long long)g.n2 * g.n3) return;
        const int i2 = (int)(t % g.n2), i3 = (int)(t / g.n2);
        zl[t] = abc_coef(model_at(raw, m, nb, i2, i3), m.dt, m.d1);
        zh[t] = abc_coef(model_at(raw, m, g.n1 - nb - 1, i2, i3), m.dt, m.d1);
    } else if (blockIdx.y == 1) {
        if (t >= (long long)g.n1 * g.n3) return;
        const int i1 = (int)(t % g.n1), i3 = (int)(t / g.n1);
        xl[t] = abc_coef(model_at(raw, m, i1, nb, i3), m.dt, m.d2);
        xh[t] = abc_coef(model_at(raw, m, i1, g.n2 - nb - 1, i3), m.dt, m.d2);
    } else {
        if (m.nd != 3 || t >= (long long)g.n1 * g.n2) return;
        const int i1 = (int)(t % g.n1), i2 = (int)(t / g.n1);
        yl[t] = abc_coef(model_at(raw, m, i1, i2, nb), m.dt, m.d3);
        yh[t] = abc_coef(model_at(raw, m, i1, i2, g.n3 - nb - 1), m.dt, m.d3);
    }
}

}  // namespace

void launch_model_pad(const float *raw, float *out, const ModelPrep &m, bool vel2, cudaStream_t s) {
    const long long cells = m.g.cells();
    k_model_pad<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(raw, out, m, vel2 ? 1 : 0);
}

void launch_model_abc(const float *raw, const ModelPrep &m, float *const abc[6], cudaStream_t s) {
    const Grid &g = m.g;
    long long n = (long long)g.n2 * g.n3;
    n = n > (long long)g.n1 * g.n3 ? n : (long long)g.n1 * g.n3;
    n = n > (long long)g.n1 * g.n2 ? n : (long long)g.n1 * g.n2;
    dim3 grid((unsigned)((n + 255) / 256), m.nd == 3 ? 3 : 2);
    k_model_abc<<<grid, 256, 0, s>>>(raw, m, abc[0], abc[1], abc[2], abc[3], abc[4], abc[5]);
}

}  // namespace awe
