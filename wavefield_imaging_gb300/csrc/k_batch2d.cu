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
#include <cuda_runtime.h>

#include "awe_internal.h"

namespace awe {

template <int NOP, int TZ, int TX>
__global__ void __launch_bounds__(TZ / 4 * TX) k_batch2d(const BatchShot *__restrict__ shots,
                                                         const int4 *__restrict__ items, int nitems,
                                                         const BatchStep p) {
    constexpr int NT = TZ / 4 * TX;
    constexpr int SH = (NOP + 3) / 4 * 4;  // halo width along axis 1, rounded to 16 bytes
    constexpr int HX = TX + 2 * NOP;
    constexpr int HZP = TZ + 2 * SH;  // row pitch (floats), keeps rows 16-byte aligned
    __shared__ __align__(16) float tile[HX][HZP];
    const int tid = threadIdx.x;
    const int zq = tid % (TZ / 4), xi = tid / (TZ / 4);
    const float *cur = p.cur, *vel = p.vel;
    float *nxt = p.nxt;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const int4 it = items[w];
        const BatchShot sh = shots[it.x];
        const int n1 = p.n1, n2 = sh.n2;
        if (it.w == 0) {
            // ---- tile item: it.y = z0, it.z = x0
            const int z0 = it.y, x0 = it.z;
            const float *c = cur + sh.off;
            __syncthreads();  // the previous item's readers are done with `tile`
            // halo tile rows x0-NOP .. x0+TX+NOP-1, columns z0-NOP .. (16-byte chunks)
            constexpr int CH = HZP / 4;
            for (int e = tid; e < HX * CH; e += NT) {
                const int r = e / CH, q = e % CH;
                const int x = x0 - NOP + r, z = z0 - SH + 4 * q;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (x >= 0 && x < n2 && z >= 0 && z + 3 < n1)
                    v = *reinterpret_cast<const float4 *>(c + (long long)x * n1 + z);
                else if (x >= 0 && x < n2) {
                    float *pv = &v.x;
                    for (int j = 0; j < 4; j++)
                        if (z + j >= 0 && z + j < n1) pv[j] = c[(long long)x * n1 + z + j];
                }
                *reinterpret_cast<float4 *>(&tile[r][4 * q]) = v;
            }
            __syncthreads();
            const int x = x0 + xi, zb = z0 + 4 * zq;
            if (x >= n2 || zb >= n1) continue;
            const float *row = &tile[xi + NOP][0];  // column SH holds z0
            const long long gi = sh.off + (long long)x * n1 + zb;
            float4 pv = *reinterpret_cast<const float4 *>(nxt + gi);  // previous level (in place)
            const float4 vv = *reinterpret_cast<const float4 *>(vel + gi);
            const float wx = p.wx[sh.wx_off + x];
            float o[4];
            const float pr4[4] = {pv.x, pv.y, pv.z, pv.w}, v4[4] = {vv.x, vv.y, vv.z, vv.w};
            const bool xin = x >= NOP && x < n2 - NOP;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int z = zb + i, tz = SH + 4 * zq + i;
                const float wz = p.wz[z];
                float pr = pr4[i];
                if (p.sponge) pr = (pr * wz) * wx;
                float out = pr;
                if (xin && z >= NOP && z < n1 - NOP) {
                    const float u = row[tz];
                    float lap = u * p.c0;
#pragma unroll
                    for (int k = 1; k <= NOP; k++) {
                        lap = fmaf(row[tz - k] + row[tz + k], p.cz[k], lap);
                        lap = fmaf(tile[xi + NOP - k][tz] + tile[xi + NOP + k][tz], p.cx[k], lap);
                    }
                    out = fmaf(v4[i], lap, 2.f * u - pr);
                }
                o[i] = out;
            }
            // source corners of this shot that fall in this 4-cell strip
            if (sh.ns > 0) {
                const float dd = p.wav[p.it];
                for (int s = 0; s < sh.ns; s++) {
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
            *reinterpret_cast<float4 *>(nxt + gi) = make_float4(o[0], o[1], o[2], o[3]);
        } else if (p.row >= 0) {
            // ---- receiver item: it.y = first receiver of the block
            const int r = it.y + tid;
            if (tid >= kBatchRecBlock || r >= sh.nr) continue;
            const GeoPoint gp = p.rec[sh.rec0 + r];
            const float *c = cur + sh.off;
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

}  // namespace awe
