// Batched 2D forward of the CPU-program scheme: many shots, each on its own
// window of one model, advanced one time step by one launch.
//
// A launch walks a flat list of work items: every (shot, tile) of the shots'
// padded grids, then every (shot, receiver block).  Tile items stage the
// current level's tile with its nop-wide halo in shared memory (16-byte
// loads), apply the 2N-order update with the sponge of the previous level on
// read, add the shot's source term and store the new level with its sponge
// (V_{k+1} = W (N + S), MAWEFDcart2Dcpu.c:297-339 with the order of the
// engine's single-shot path).  Receiver items gather R (W V_k) from the
// current level, which this launch does not write.  Shots share nz, the
// spacing, the sponge width and the time axis; they differ in nx and offset.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "awe_internal.h"
#include "gsum.cuh"

namespace awe {

template <int NOP, int TZ, int TX>
__global__ void __launch_bounds__(TZ / 4 * TX) k_batch2d(const BatchShot *__restrict__ shots,
                                                         const int4 *__restrict__ items, int nitems,
                                                         const BatchStep p) {
    constexpr int NT = TZ / 4 * TX;
    constexpr int SH = (NOP + 3) / 4 * 4;  // halo width along axis 1, rounded to 16 bytes
    constexpr int HX = TX + 2 * NOP;
    constexpr int HZP = TZ + 2 * SH;  // row pitch (floats), keeps rows 16-byte aligned
    constexpr int CH = HZP / 4;       // 16-byte chunks per halo row
    constexpr int NCH = (HX * CH + NT - 1) / NT;
    __shared__ __align__(16) float tile[HX][HZP];
    const int tid = threadIdx.x;
    const int zq = tid % (TZ / 4), xi = tid / (TZ / 4);
    const int n1 = p.n1;
    const float *prvb = p.prv ? p.prv : p.nxt;  // previous level: in place, or out of place
    // registers of the next tile item: its halo chunks and this thread's
    // previous-level and v^2 dt^2 strips (loaded while the current item computes)
    float4 hb[NCH], pb = make_float4(0.f, 0.f, 0.f, 0.f), vb = pb;
    auto fetch = [&](int w2) {
        const int4 it = items[w2];
        if (it.w != 0) return;
        const BatchShot sh = shots[it.x];
        const float *c = p.cur + sh.off;
#pragma unroll
        for (int j = 0; j < NCH; j++) {
            const int e = tid + j * NT;
            const int r = e / CH, q = e % CH;
            const int x = it.z - NOP + r, z = it.y - SH + 4 * q;
            hb[j] = make_float4(0.f, 0.f, 0.f, 0.f);
            // n1 % 4 == 0 and z % 4 == 0: a chunk is wholly inside or outside
            if (e < HX * CH && x >= 0 && x < sh.n2 && z >= 0 && z < n1)
                hb[j] = *reinterpret_cast<const float4 *>(c + (long long)x * n1 + z);
        }
        const int x = it.z + xi, zb = it.y + 4 * zq;
        if (x < sh.n2 && zb < n1) {
            const long long gi = sh.off + (long long)x * n1 + zb;
            pb = *reinterpret_cast<const float4 *>(prvb + gi);
            vb = *reinterpret_cast<const float4 *>(p.vel + gi);
        }
    };
    if (blockIdx.x < nitems) fetch(blockIdx.x);
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const int4 it = items[w];
        const BatchShot sh = shots[it.x];
        const int n2 = sh.n2;
        if (it.w == 0) {
            // ---- tile item: it.y = z0, it.z = x0
            const int z0 = it.y, x0 = it.z;
            __syncthreads();  // the previous item's readers are done with `tile`
#pragma unroll
            for (int j = 0; j < NCH; j++) {
                const int e = tid + j * NT;
                if (e < HX * CH) *reinterpret_cast<float4 *>(&tile[e / CH][4 * (e % CH)]) = hb[j];
            }
            const float4 pv = pb, vv = vb;
            __syncthreads();
            if (w + (int)gridDim.x < nitems) fetch(w + gridDim.x);
            const int x = x0 + xi, zb = z0 + 4 * zq;
            if (x >= n2 || zb >= n1) continue;
            const long long gi = sh.off + (long long)x * n1 + zb;
            const float wx = p.wx[sh.wx_off + x];
            float o[4];
            const float pr4[4] = {pv.x, pv.y, pv.z, pv.w}, v4[4] = {vv.x, vv.y, vv.z, vv.w};
            const bool xin = x >= NOP && x < n2 - NOP;
            // 16-byte shared loads (conflict-free): the z window of the strip and
            // the x neighbours' strips; packed FP32x2 arithmetic, two cells at a time
            const int tz0 = SH + 4 * zq;  // tile column of zb
            constexpr int NZW = 4 + 2 * SH;
            float zw[NZW];
#pragma unroll
            for (int j = 0; j < NZW / 4; j++) {
                const float4 t = *reinterpret_cast<const float4 *>(&tile[xi + NOP][tz0 - SH + 4 * j]);
                zw[4 * j] = t.x;
                zw[4 * j + 1] = t.y;
                zw[4 * j + 2] = t.z;
                zw[4 * j + 3] = t.w;
            }
            float2 l01 = __fmul2_rn(make_float2(zw[SH], zw[SH + 1]), make_float2(p.c0, p.c0));
            float2 l23 = __fmul2_rn(make_float2(zw[SH + 2], zw[SH + 3]), make_float2(p.c0, p.c0));
#pragma unroll
            for (int k = 1; k <= NOP; k++) {
                const float4 xm = *reinterpret_cast<const float4 *>(&tile[xi + NOP - k][tz0]);
                const float4 xp = *reinterpret_cast<const float4 *>(&tile[xi + NOP + k][tz0]);
                const float2 z01 = make_float2(zw[SH - k] + zw[SH + k], zw[SH + 1 - k] + zw[SH + 1 + k]);
                const float2 z23 = make_float2(zw[SH + 2 - k] + zw[SH + 2 + k], zw[SH + 3 - k] + zw[SH + 3 + k]);
                const float2 x01 = __fadd2_rn(make_float2(xm.x, xm.y), make_float2(xp.x, xp.y));
                const float2 x23 = __fadd2_rn(make_float2(xm.z, xm.w), make_float2(xp.z, xp.w));
                const float2 cz = make_float2(p.cz[k], p.cz[k]), cx = make_float2(p.cx[k], p.cx[k]);
                l01 = __ffma2_rn(z01, cz, l01);
                l23 = __ffma2_rn(z23, cz, l23);
                l01 = __ffma2_rn(x01, cx, l01);
                l23 = __ffma2_rn(x23, cx, l23);
            }
            const float lap[4] = {l01.x, l01.y, l23.x, l23.y};
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int z = zb + i;
                float pr = pr4[i];
                if (p.sponge) pr = (pr * p.wz[z]) * wx;
                float out = pr;
                if (xin && z >= NOP && z < n1 - NOP) out = fmaf(v4[i], lap[i], 2.f * zw[SH + i] - pr);
                o[i] = out;
            }
            // source corners of this shot that fall in this 4-cell strip
            if (sh.ns > 0) {
                const float dd = p.wav[p.it];
                for (int s = 0; s < sh.ns; s++) {
                    // corners lie within n1 + 1 of the base index
                    const long long b0 = p.src[sh.src0 + s].base - ((long long)x * n1 + zb);
                    if (b0 < -(long long)n1 - 1 || b0 > 3) continue;
                    const GeoPoint gp = p.src[sh.src0 + s];
#pragma unroll
                    for (int cc = 0; cc < 4; cc++) {
                        const long long n = gp.base + (cc & 1) + (cc >> 1) * (long long)n1;
                        const long long d = n - ((long long)x * n1 + zb);
#pragma unroll
                        for (int i = 0; i < 4; i++)
                            if (d == i) o[i] = o[i] + (dd * gp.w[cc]) * v4[i];
                    }
                }
            }
            if (p.sponge) {
#pragma unroll
                for (int i = 0; i < 4; i++) o[i] = (o[i] * p.wz[zb + i]) * wx;
            }
            *reinterpret_cast<float4 *>(p.nxt + gi) = make_float4(o[0], o[1], o[2], o[3]);
        } else {
            if (w + (int)gridDim.x < nitems) fetch(w + gridDim.x);
            if (p.row < 0) continue;
            // ---- receiver item: it.y = first receiver of the block
            const int r = it.y + tid;
            if (tid >= kBatchRecBlock || r >= sh.nr) continue;
            const GeoPoint gp = p.rec[sh.rec0 + r];
            const float *c = p.cur + sh.off;
            float acc = 0.f;
#pragma unroll
            for (int cc = 0; cc < 4; cc++) {
                const long long n = gp.base + (cc & 1) + (cc >> 1) * (long long)n1;
                float v = c[n];
                if (p.sponge) {
                    const int z = (int)(n % n1), xx = (int)(n / n1);
                    v = (v * p.wz[z]) * p.wx[sh.wx_off + xx];
                }
                acc = fmaf(v, gp.w[cc], acc);
            }
            p.dat[sh.dat_off + (long long)p.row * sh.nr + r] = acc;
        }
    }
}

template <int NOP, int TZ, int TX>
static void launch_t(const BatchShot *shots, const int4 *items, int nitems, int grid, const BatchStep &p,
                     cudaStream_t s) {
    k_batch2d<NOP, TZ, TX><<<grid, TZ / 4 * TX, 0, s>>>(shots, items, nitems, p);
}

// tile shapes the autotuner chooses from (TZ x TX cells; TZ/4 * TX threads)
const int kBatchTiles[kBatchNumTiles][2] = {{64, 16}, {128, 8}, {32, 32}, {64, 8}};

void launch_batch2d(int nop, int tile, const BatchShot *shots, const int4 *items, int nitems, int grid,
                    const BatchStep &p, cudaStream_t s) {
#define TILES(N)                                                          \
    case N:                                                               \
        if (tile == 0) launch_t<N, 64, 16>(shots, items, nitems, grid, p, s);  \
        else if (tile == 1) launch_t<N, 128, 8>(shots, items, nitems, grid, p, s); \
        else if (tile == 2) launch_t<N, 32, 32>(shots, items, nitems, grid, p, s); \
        else launch_t<N, 64, 8>(shots, items, nitems, grid, p, s);         \
        break;
    switch (nop) {
        TILES(1) TILES(2) TILES(3) TILES(4) TILES(5) TILES(6) TILES(7) TILES(8)
        default: break;
    }
#undef TILES
}

// ---------------------------------------------------------------------------
// Adjoint step of the batch (2D, sponge, no one-way ABC: the 2D CPU-program
// scheme applies none without the hybrid option).  Per tile item, with
// X = nu_k, Y = nu_{k+1} (overwritten by mu_k = W lambda_k), V = V_k:
//   lambda = 2 I nu + L(I vel2 nu) + W (1 - 2 I) nu_{k+1} + W R^T r_k
//   dJ/dvel2 += I nu L(V_k) + nu wav w (source corners), FP64 per shot.
// The halo tiles of g = I vel2 nu and of V_k are staged in shared memory; the
// receiver corners of the tile come from a per-tile list, so each cell is
// written by the one thread that owns it.
template <int NOP, int TZ, int TX>
__global__ void __launch_bounds__(TZ / 4 * TX) k_batch2d_adj(const BatchShot *__restrict__ shots,
                                                             const int4 *__restrict__ items, int nitems,
                                                             const BatchAdj p) {
    constexpr int NT = TZ / 4 * TX;
    constexpr int SH = (NOP + 3) / 4 * 4;
    constexpr int HX = TX + 2 * NOP;
    constexpr int HZP = TZ + 2 * SH;
    constexpr int CH = HZP / 4;
    constexpr int NCH = (HX * CH + NT - 1) / NT;
    __shared__ __align__(16) float gt[HX][HZP];
    __shared__ __align__(16) float vt[HX][HZP];
    const int tid = threadIdx.x;
    const int zq = tid % (TZ / 4), xi = tid / (TZ / 4);
    const int n1 = p.n1;
    // registers of the next item: g = I vel2 nu and V_k halo chunks, nu and
    // nu_{k+1} strips of this thread (loaded while the current item computes)
    float4 gb[NCH], vb[NCH], nb4 = make_float4(0.f, 0.f, 0.f, 0.f), yb4 = nb4;
    auto fetch = [&](int w2) {
        const int4 it = items[w2];
        if (it.w != 0) return;
        const BatchShot sh = shots[it.x];
        const float *X = p.X + sh.off, *V = p.V + sh.off, *vel = p.vel + sh.off;
#pragma unroll
        for (int j = 0; j < NCH; j++) {
            const int e = tid + j * NT;
            const int r = e / CH, q = e % CH;
            const int x = it.z - NOP + r, z = it.y - SH + 4 * q;
            float4 g = make_float4(0.f, 0.f, 0.f, 0.f), v = g;
            if (e < HX * CH && x >= 0 && x < sh.n2 && z >= 0 && z < n1) {  // n1 % 4 == 0
                const long long jj = (long long)x * n1 + z;
                const float4 xv = *reinterpret_cast<const float4 *>(X + jj);
                const float4 vv = *reinterpret_cast<const float4 *>(vel + jj);
                v = *reinterpret_cast<const float4 *>(V + jj);
                const bool xin = x >= NOP && x < sh.n2 - NOP;
                g.x = (xin && z >= NOP && z < n1 - NOP) ? vv.x * xv.x : 0.f;
                g.y = (xin && z + 1 >= NOP && z + 1 < n1 - NOP) ? vv.y * xv.y : 0.f;
                g.z = (xin && z + 2 >= NOP && z + 2 < n1 - NOP) ? vv.z * xv.z : 0.f;
                g.w = (xin && z + 3 >= NOP && z + 3 < n1 - NOP) ? vv.w * xv.w : 0.f;
            }
            gb[j] = g;
            vb[j] = v;
        }
        const int x = it.z + xi, zb = it.y + 4 * zq;
        if (x < sh.n2 && zb < n1) {
            const long long gi = sh.off + (long long)x * n1 + zb;
            nb4 = *reinterpret_cast<const float4 *>(p.X + gi);
            yb4 = *reinterpret_cast<const float4 *>(p.Y + gi);
        }
    };
    if (blockIdx.x < nitems) fetch(blockIdx.x);
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const int4 it = items[w];
        if (it.w != 0) continue;  // receiver items belong to the forward
        const BatchShot sh = shots[it.x];
        const int n2 = sh.n2, z0 = it.y, x0 = it.z;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < NCH; j++) {
            const int e = tid + j * NT;
            if (e < HX * CH) {
                *reinterpret_cast<float4 *>(&gt[e / CH][4 * (e % CH)]) = gb[j];
                *reinterpret_cast<float4 *>(&vt[e / CH][4 * (e % CH)]) = vb[j];
            }
        }
        const float4 nv4 = nb4, yv4 = yb4;
        __syncthreads();
        if (w + (int)gridDim.x < nitems) fetch(w + gridDim.x);
        const int x = x0 + xi, zb = z0 + 4 * zq;
        if (x >= n2 || zb >= n1) continue;
        const long long gi = sh.off + (long long)x * n1 + zb;
        // the gradient accumulators of this strip, loaded before the stencils
        // so the load latency overlaps them
        float2 *G = p.G + gi;
        const float4 G01 = __ldcs(reinterpret_cast<const float4 *>(G));
        const float4 G23 = __ldcs(reinterpret_cast<const float4 *>(G + 2));
        const float nu[4] = {nv4.x, nv4.y, nv4.z, nv4.w}, yv[4] = {yv4.x, yv4.y, yv4.z, yv4.w};
        const float wx = p.sponge ? p.wx[sh.wx_off + x] : 1.f;
        const bool xin = x >= NOP && x < n2 - NOP;
        float mu[4], wc[4];
        float2 ga[4] = {make_float2(G01.x, G01.y), make_float2(G01.z, G01.w), make_float2(G23.x, G23.y),
                        make_float2(G23.z, G23.w)};
        // 16-byte shared loads of both stencils' z windows and x neighbours, packed FP32x2
        const int tz0 = SH + 4 * zq;
        constexpr int NZW = 4 + 2 * SH;
        float gz[NZW], vz[NZW];
#pragma unroll
        for (int j = 0; j < NZW / 4; j++) {
            const float4 a = *reinterpret_cast<const float4 *>(&gt[xi + NOP][tz0 - SH + 4 * j]);
            const float4 b = *reinterpret_cast<const float4 *>(&vt[xi + NOP][tz0 - SH + 4 * j]);
            gz[4 * j] = a.x, gz[4 * j + 1] = a.y, gz[4 * j + 2] = a.z, gz[4 * j + 3] = a.w;
            vz[4 * j] = b.x, vz[4 * j + 1] = b.y, vz[4 * j + 2] = b.z, vz[4 * j + 3] = b.w;
        }
        const float2 c0 = make_float2(p.c0, p.c0);
        float2 g01 = __fmul2_rn(make_float2(gz[SH], gz[SH + 1]), c0), g23 = __fmul2_rn(make_float2(gz[SH + 2], gz[SH + 3]), c0);
        float2 v01 = __fmul2_rn(make_float2(vz[SH], vz[SH + 1]), c0), v23 = __fmul2_rn(make_float2(vz[SH + 2], vz[SH + 3]), c0);
#pragma unroll
        for (int k = 1; k <= NOP; k++) {
            const float2 cz = make_float2(p.cz[k], p.cz[k]), cx = make_float2(p.cx[k], p.cx[k]);
            const float4 gm = *reinterpret_cast<const float4 *>(&gt[xi + NOP - k][tz0]);
            const float4 gp = *reinterpret_cast<const float4 *>(&gt[xi + NOP + k][tz0]);
            const float4 vm = *reinterpret_cast<const float4 *>(&vt[xi + NOP - k][tz0]);
            const float4 vp = *reinterpret_cast<const float4 *>(&vt[xi + NOP + k][tz0]);
            g01 = __ffma2_rn(make_float2(gz[SH - k] + gz[SH + k], gz[SH + 1 - k] + gz[SH + 1 + k]), cz, g01);
            g23 = __ffma2_rn(make_float2(gz[SH + 2 - k] + gz[SH + 2 + k], gz[SH + 3 - k] + gz[SH + 3 + k]), cz, g23);
            g01 = __ffma2_rn(__fadd2_rn(make_float2(gm.x, gm.y), make_float2(gp.x, gp.y)), cx, g01);
            g23 = __ffma2_rn(__fadd2_rn(make_float2(gm.z, gm.w), make_float2(gp.z, gp.w)), cx, g23);
            v01 = __ffma2_rn(make_float2(vz[SH - k] + vz[SH + k], vz[SH + 1 - k] + vz[SH + 1 + k]), cz, v01);
            v23 = __ffma2_rn(make_float2(vz[SH + 2 - k] + vz[SH + 2 + k], vz[SH + 3 - k] + vz[SH + 3 + k]), cz, v23);
            v01 = __ffma2_rn(__fadd2_rn(make_float2(vm.x, vm.y), make_float2(vp.x, vp.y)), cx, v01);
            v23 = __ffma2_rn(__fadd2_rn(make_float2(vm.z, vm.w), make_float2(vp.z, vp.w)), cx, v23);
        }
        const float lt4[4] = {g01.x, g01.y, g23.x, g23.y}, lv4[4] = {v01.x, v01.y, v23.x, v23.y};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int z = zb + i;
            const bool in = xin && z >= NOP && z < n1 - NOP;
            wc[i] = p.sponge ? p.wz[z] * wx : 1.f;
            const float lam = (in ? 2.f * nu[i] : 0.f) + lt4[i] + (in ? -wc[i] : wc[i]) * yv[i];
            mu[i] = wc[i] * lam;
            if (in) ga[i] = gsum_add(ga[i], __fmul_rn(nu[i], lv4[i]));  // FP32 product, compensated sum
        }
        const long long cell0 = (long long)x * n1 + zb;
        // source term of the gradient (corners lie within n1 + 1 of the base index)
        if (sh.ns > 0) {
            const float dd = p.wav[p.it];
            for (int s = 0; s < sh.ns; s++) {
                const long long b0 = p.src[sh.src0 + s].base - cell0;
                if (b0 < -(long long)n1 - 1 || b0 > 3) continue;
                const GeoPoint gp = p.src[sh.src0 + s];
#pragma unroll
                for (int cc = 0; cc < 4; cc++) {
                    const long long d = gp.base + (cc & 1) + (cc >> 1) * (long long)n1 - cell0;
#pragma unroll
                    for (int i = 0; i < 4; i++)
                        if (d == i) ga[i] = gsum_add_prod(ga[i], nu[i], dd * gp.w[cc]);
                }
            }
        }
        *reinterpret_cast<float4 *>(p.Y + gi) = make_float4(mu[0], mu[1], mu[2], mu[3]);
        __stcs(reinterpret_cast<float4 *>(G), make_float4(ga[0].x, ga[0].y, ga[1].x, ga[1].y));
        __stcs(reinterpret_cast<float4 *>(G + 2), make_float4(ga[2].x, ga[2].y, ga[3].x, ga[3].y));
    }
}

template <int NOP, int TZ, int TX>
static void launch_adj_t(const BatchShot *shots, const int4 *items, int nitems, int grid, const BatchAdj &p,
                         cudaStream_t s) {
    k_batch2d_adj<NOP, TZ, TX><<<grid, TZ / 4 * TX, 0, s>>>(shots, items, nitems, p);
}

void launch_batch2d_adj(int nop, int tile, const BatchShot *shots, const int4 *items, int nitems, int grid,
                        const BatchAdj &p, cudaStream_t s) {
#define TILES(N)                                                                     \
    case N:                                                                          \
        if (tile == 0) launch_adj_t<N, 64, 16>(shots, items, nitems, grid, p, s);      \
        else if (tile == 1) launch_adj_t<N, 128, 8>(shots, items, nitems, grid, p, s); \
        else if (tile == 2) launch_adj_t<N, 32, 32>(shots, items, nitems, grid, p, s); \
        else launch_adj_t<N, 64, 8>(shots, items, nitems, grid, p, s);                \
        break;
    switch (nop) {
        TILES(1) TILES(2) TILES(3) TILES(4) TILES(5) TILES(6) TILES(7) TILES(8)
        default: break;
    }
#undef TILES
}

// ---------------------------------------------------------------------------
// Checkpoints of the batch: one block per shot, one FP32 scale per shot and
// level (the shot's max |v|), 16-bit values (BF16 or FP16) or FP32 copies.
template <typename Q>
__device__ __forceinline__ void q_store(Q *q, long long i, float v);
template <>
__device__ __forceinline__ void q_store<__nv_bfloat16>(__nv_bfloat16 *q, long long i, float v) {
    q[i] = __float2bfloat16_rn(v);
}
template <>
__device__ __forceinline__ void q_store<__half>(__half *q, long long i, float v) {
    q[i] = __float2half_rn(v);
}
__device__ __forceinline__ float q_load(const __nv_bfloat16 *q, long long i) { return __bfloat162float(q[i]); }
__device__ __forceinline__ float q_load(const __half *q, long long i) { return __half2float(q[i]); }

template <typename Q>
__global__ void k_batch_ckpt_store(const BatchShot *__restrict__ shots, const float *__restrict__ u, Q *q,
                                   float *scales, int n1) {
    const BatchShot sh = shots[blockIdx.x];
    const long long n = (long long)sh.n2 * n1;
    const float *a = u + sh.off;
    __shared__ float red[32];
    float m = 0.f;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, fabsf(a[i]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x + 31) / 32 ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) red[0] = m;
    }
    __syncthreads();
    const float scale = red[0] > 0.f ? red[0] : 1.f, inv = 1.f / scale;
    if (threadIdx.x == 0) scales[blockIdx.x] = scale;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) q_store<Q>(q, sh.off + i, a[i] * inv);
}

template <typename Q>
__global__ void k_batch_ckpt_load(const BatchShot *__restrict__ shots, const Q *__restrict__ q,
                                  const float *__restrict__ scales, float *u, int n1) {
    const BatchShot sh = shots[blockIdx.x];
    const long long n = (long long)sh.n2 * n1;
    const float sc = scales[blockIdx.x];
    for (long long i = threadIdx.x; i < n; i += blockDim.x) u[sh.off + i] = q_load(q, sh.off + i) * sc;
}

void launch_batch_ckpt(bool store, int fmt, const BatchShot *shots, int nshots, float *u, void *q, float *scales,
                       int n1, long long cells, cudaStream_t s) {
    if (fmt == AWE_CKPT_FP32) {
        if (store) cudaMemcpyAsync(q, u, (size_t)cells * sizeof(float), cudaMemcpyDeviceToDevice, s);
        else cudaMemcpyAsync(u, q, (size_t)cells * sizeof(float), cudaMemcpyDeviceToDevice, s);
        return;
    }
    if (fmt == AWE_CKPT_BFP16) {  // blocks of 64 cells over the concatenated fields, scales per block
        const int grid = (int)((cells + 255) / 256 < 4096 ? (cells + 255) / 256 : 4096);
        if (store) launch_ckpt_store_bfp(u, cells, (short *)q, scales, grid, s);
        else launch_ckpt_load_bfp((const short *)q, scales, cells, u, grid, s);
        return;
    }
    if (fmt == AWE_CKPT_FP16) {
        if (store) k_batch_ckpt_store<__half><<<nshots, 512, 0, s>>>(shots, u, (__half *)q, scales, n1);
        else k_batch_ckpt_load<__half><<<nshots, 512, 0, s>>>(shots, (const __half *)q, scales, u, n1);
    } else {
        if (store) k_batch_ckpt_store<__nv_bfloat16><<<nshots, 512, 0, s>>>(shots, u, (__nv_bfloat16 *)q, scales, n1);
        else k_batch_ckpt_load<__nv_bfloat16><<<nshots, 512, 0, s>>>(shots, (const __nv_bfloat16 *)q, scales, u, n1);
    }
}

// residuals r = d - dobs over the concatenated traces; FP64 partial sums of
// r^2 per block of 1024 samples (summed in order on the host)
__global__ void k_residual_flat(const float *__restrict__ d, const float *__restrict__ dobs, float *__restrict__ r,
                                long long n, double *__restrict__ part) {
    __shared__ double red[256];
    const long long b0 = (long long)blockIdx.x * 1024;
    double acc = 0;
    for (int j = threadIdx.x; j < 1024; j += 256) {
        const long long i = b0 + j;
        if (i < n) {
            const float v = d[i] - dobs[i];
            r[i] = v;
            acc += (double)v * (double)v;
        }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

void launch_residual_flat(const float *d, const float *dobs, float *r, long long n, double *part, cudaStream_t s) {
    const int blocks = (int)((n + 1023) / 1024);
    if (blocks > 0) k_residual_flat<<<blocks, 256, 0, s>>>(d, dobs, r, n, part);
}

// receiver residuals of the adjoint step on mu = W lambda (W R^T r, then the
// W of mu): mu += W (W (w r)) per corner, in (receiver, corner) order
__global__ void k_batch_rec_adj(const BatchRecCell *__restrict__ cells, int ncells, const BatchRecW *__restrict__ ws,
                                const BatchShot *__restrict__ shots, const BatchAdj p) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncells) return;
    const BatchRecCell c = cells[t];
    const BatchShot sh = shots[c.shot];
    const float wc = p.sponge ? p.wz[c.z] * p.wx[sh.wx_off + c.x] : 1.f;
    const float *res = p.res + sh.dat_off + (long long)p.row * sh.nr;
    float mu = p.Y[c.gi];
    for (int e = c.e0; e < c.e1; e++) mu = __fmaf_rn(wc, __fmul_rn(wc, __fmul_rn(ws[e].w, res[ws[e].r])), mu);
    p.Y[c.gi] = mu;
}

void launch_batch_rec_adj(const BatchRecCell *cells, int ncells, const BatchRecW *ws, const BatchShot *shots,
                          const BatchAdj &p, cudaStream_t s) {
    if (ncells > 0 && p.row >= 0) k_batch_rec_adj<<<(ncells + 127) / 128, 128, 0, s>>>(cells, ncells, ws, shots, p);
}

// model gradient: dJ/dvel2 * (-vel2^2 / dt^2), each shot's padded cells summed
// onto the model cells they replicate (window columns x0 .. x0 + nx - 1)
__global__ void k_batch_grad_fold(const BatchShot *__restrict__ shots, const int2 *__restrict__ win, int nshots,
                                  const float2 *__restrict__ G, const float *__restrict__ vel2, double inv_dt2,
                                  int n1, int nb, int nz, int nxm, double *__restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nz * nxm) return;
    const int z = (int)(t % nz), xm = (int)(t / nz);
    const int za = z == 0 ? 0 : z + nb, zbnd = z == nz - 1 ? n1 - 1 : z + nb;
    double acc = 0;
    for (int s = 0; s < nshots; s++) {
        const int x0 = win[s].x, nx = win[s].y;
        const int j = xm - x0;
        if (j < 0 || j >= nx) continue;
        const BatchShot sh = shots[s];
        const int xa = j == 0 ? 0 : j + nb, xb = j == nx - 1 ? sh.n2 - 1 : j + nb;
        for (int ix = xa; ix <= xb; ix++)
            for (int iz = za; iz <= zbnd; iz++) {
                const long long i = sh.off + (long long)ix * n1 + iz;
                const double v2 = vel2[i];
                acc += gsum_value(G[i]) * (-v2 * v2 * inv_dt2);
            }
    }
    out[t] = acc;
}

void launch_batch_grad_fold(const BatchShot *shots, const int2 *win, int nshots, const float2 *G, const float *vel2,
                            float dt, int n1, int nb, int nz, int nxm, double *out, cudaStream_t s) {
    const long long n = (long long)nz * nxm;
    k_batch_grad_fold<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(shots, win, nshots, G, vel2,
                                                                  1.0 / ((double)dt * (double)dt), n1, nb, nz, nxm,
                                                                  out);
}

}  // namespace awe
