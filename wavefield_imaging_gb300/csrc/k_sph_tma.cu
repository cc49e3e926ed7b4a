// Spherical-shell step of the GPU-program scheme (AWE_FAST), TMA-staged.
//
// The update is that of spher_kernels.cu:455-526 (solve_3D with the metric
// terms A = 2/r, C = 1/r^2, B = cos/(r^2 sin), D = 1/(r^2 sin^2), precomputed
// per (r) and (r, theta)) followed by the sponge of both time levels
// (spongeKernel_3D, spher_kernels.cu:825) and the free-surface mask, with the
// engine's two-buffer leapfrog: the new level overwrites the previous one and
// the previous level's sponge is applied on read.
//
// A CTA owns a 64 (r) x 16 (theta) tile of one shot and marches along phi over
// a chunk of planes.  Per plane one TMA copy (cp.async.bulk.tensor, mbarrier
// completion) brings the current level's 72 x 18 box - r widened by 4 on each
// side so the box starts on a 16-byte boundary, theta by 1 - into a 6-deep
// shared-memory ring, and for the plane being updated the previous level's
// and the velocity's 64 x 16 boxes, up to five planes ahead of the compute.
// phi-neighbours come from a 3-plane register queue (each thread owns 4
// consecutive radii of one theta row), r- and theta-neighbours from the halo
// box; the 4-cell result is written with one 16-byte store.  Work items
// (tile, phi chunk, shot) are handed out by a global atomic counter, so the
// persistent grid (2 CTAs per SM) stays balanced.  Every wait is bounded; a
// wait that gives up raises the plan's error flag and the CTA drains its
// copies in flight before it leaves.
//
// The arithmetic per cell is that of k_stepA_sph_march2 (packed FP32x2,
// the same operation order), so both kernels give the same AWE_FAST results.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>

#include "awe_internal.h"
#include "gsum.cuh"
#include "tma.cuh"

namespace awe {

namespace sp3 {
constexpr int TR = 64, TT = 16, HR = 4, HT = 1;
constexpr int WR = TR + 2 * HR, WT = TT + 2 * HT;  // 72 x 18 halo box
constexpr int RING = 6, NTHREADS = 256;
constexpr uint32_t BYTES_HALO = WR * WT * 4, BYTES_TILE = TR * TT * 4;
constexpr long long SPIN_LIMIT = 1ll << 22;
constexpr int FTAB_MAX = 256;  // sponge factors held in shared memory (nb < FTAB_MAX)

// every box destination starts on a 128-byte boundary
struct __align__(128) Stage {
    float cur[WT][WR];
    float pad[(128 - (WT * WR * 4) % 128) % 128 / 4];
    float prv[TT][TR];
    float vel[TT][TR];
};
static_assert(sizeof(Stage) % 128 == 0, "stage size");
static_assert(offsetof(Stage, prv) % 128 == 0 && offsetof(Stage, vel) % 128 == 0, "box alignment");
static_assert((WR * 4) % 16 == 0 && (TR * 4) % 16 == 0, "box rows are whole 16-byte units");
}  // namespace sp3

struct SphTmaParams {
    StepAParams a;  // grid, sponge tables, mask, metric tables, reciprocals, dt^2
    int L, ntr, ntt, nchunks, nshot;
    int cur_f0, prv_f0;  // plane offsets of the current and previous levels in their maps
    unsigned long long *counter;
    unsigned long long base;
    int *err;
    float *nxt;
    long long spin;  // polls of a compute-side wait before it gives up (the drain keeps SPIN_LIMIT)
};

// sponge factor of index i (AWE_FAST: the float table, copied to shared memory)
__device__ __forceinline__ float sph_damp(float v, int i, const float *ftab) { return i == 0 ? v : v * ftab[i]; }

// sponge index over the kernel axes in their priority order (r, phi, theta)
// = memory axes (1, 3, 2): the first low face in that order, else the first
// high face (spongeKernel_3D; StepAParams::pri of the spherical grid)
__device__ __forceinline__ int sph_sponge_index(int r, int ph, int th, int nr, int nph, int nth, int nb) {
    if (r < nb) return nb - r;
    if (ph < nb) return nb - ph;
    if (th < nb) return nb - th;
    if (r > nr - nb) return r - (nr - nb);
    if (ph > nph - nb) return ph - (nph - nb);
    if (th > nth - nb) return th - (nth - nb);
    return 0;
}

__global__ void __launch_bounds__(sp3::NTHREADS, 2)
    k_stepA_sph_tma(const __grid_constant__ CUtensorMap tm_cur, const __grid_constant__ CUtensorMap tm_prv,
                    const __grid_constant__ CUtensorMap tm_vel, const SphTmaParams p) {
    using namespace sp3;
    extern __shared__ unsigned char smem_raw[];
    Stage *st = reinterpret_cast<Stage *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    __shared__ __align__(8) uint64_t full[RING];
    __shared__ int s_item;
    __shared__ float s_ftab[FTAB_MAX];

    const int tid = threadIdx.x;
    const int rq = tid & 15, ti = tid >> 4;
    for (int i = tid; i <= p.a.nb && i < FTAB_MAX; i += NTHREADS) s_ftab[i] = p.a.ftab[i];
    if (tid == 0) {
        for (int r = 0; r < RING; r++) mbar_init(&full[r], 1);
        fence_mbar_init();
        prefetch_tmap(&tm_cur);
        prefetch_tmap(&tm_prv);
        prefetch_tmap(&tm_vel);
    }
    // an earlier launch that gave up on a wait leaves the flag set: do nothing
    if (__syncthreads_or(tid == 0 && *(volatile int *)p.err != 0)) return;

    const int n1 = p.a.g.n1, n2 = p.a.g.n2, n3 = p.a.g.n3, nb = p.a.nb;
    const int per_chunk = p.ntr * p.ntt;
    const int nitems = per_chunk * p.nchunks * p.nshot;
    const long long plane = (long long)n1 * n2;
    const float2 r0v = make_float2(p.a.rd[0], p.a.rd[0]), r1v = make_float2(p.a.rd[1], p.a.rd[1]);
    const float2 r2v = make_float2(p.a.rd[2], p.a.rd[2]), r3v = make_float2(p.a.rd[3], p.a.rd[3]);
    const float2 r4v = make_float2(p.a.rd[4], p.a.rd[4]), dt2v = make_float2(p.a.dt2, p.a.dt2);
    const float2 m1 = make_float2(-1.f, -1.f), m2 = make_float2(-2.f, -2.f);
    const bool mask3 = p.a.mask == 3;

    // ring position of the current item's first plane: slot and mbarrier parity
    int slot0 = 0;
    uint32_t ph0 = 0;
    for (;;) {
        if (tid == 0) s_item = (int)(atomicAdd(p.counter, 1ull) - p.base);
        __syncthreads();
        const int item = s_item;
        if (item >= nitems || item < 0) break;
        const int tile = item % per_chunk, rest = item / per_chunk;
        const int chunk = rest % p.nchunks, shot = rest / p.nchunks;
        const int r0 = (tile % p.ntr) * TR, t0 = (tile / p.ntr) * TT;
        const int y0 = chunk * p.L, y1 = min(y0 + p.L, n3);
        const int S = (y1 - y0) + 2;  // current-level planes y0-1 .. y1
        const int fo = shot * n3;     // the shot's first plane in the stacked fields

        // stage s: current-level plane y0-1+s; from s = 2 on also the previous
        // level and the velocity of plane y0+s-2, the plane updated at stage s
        auto issue = [&](int s) {
            const int slot = (slot0 + s) % RING;
            const bool out = s >= 2;
            mbar_expect_tx(&full[slot], BYTES_HALO + (out ? 2 * BYTES_TILE : 0));
            tma_load_3d(&st[slot].cur[0][0], &tm_cur, &full[slot], r0 - HR, t0 - HT, p.cur_f0 + fo + y0 - 1 + s);
            if (out) {
                const int y = y0 + s - 2;
                tma_load_3d(&st[slot].prv[0][0], &tm_prv, &full[slot], r0, t0, p.prv_f0 + fo + y);
                tma_load_3d(&st[slot].vel[0][0], &tm_vel, &full[slot], r0, t0, y);
            }
        };
        if (tid == 0)
            for (int s = 0; s < RING && s < S; s++) issue(s);

        // per-thread constants: 4 radii r .. r+3 of theta row t
        const int r = r0 + 4 * rq, t = t0 + ti;
        const bool col_ok = r < n1 && t < n2;  // n1 % 4 == 0: the 4 cells exist together
        const bool th_in = t >= 4 && t < n2 - 4;
        bool rin[4];
        bool any_r = false;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            rin[j] = r + j >= 4 && r + j < n1 - 4;
            any_r = any_r || rin[j];
        }
        float4 A2 = make_float4(0.f, 0.f, 0.f, 0.f), Cr = A2, B = A2, D = A2;
        if (col_ok) {
            const long long tt = (long long)t * n1 + r;
            A2 = __ldg(reinterpret_cast<const float4 *>(p.a.tr0 + r));
            Cr = __ldg(reinterpret_cast<const float4 *>(p.a.tr1 + r));
            B = __ldg(reinterpret_cast<const float4 *>(p.a.tt0 + tt));
            D = __ldg(reinterpret_cast<const float4 *>(p.a.tt1 + tt));
        }
        // every (r, theta) cell of the tile is outside the r and theta sponge bands
        const bool tile_undamped = r0 >= nb && r0 + TR - 1 <= n1 - nb && t0 >= nb && t0 + TT - 1 <= n2 - nb;
        float *dst = p.nxt + ((long long)(fo + y0) * n2 + t) * n1 + r;

        int slot = slot0;  // ring slot and parity of stage s
        uint32_t ph = ph0;
        float q[3][4];  // phi queue: the centre values of stage s live in q[s % 3]
#pragma unroll 1
        for (int blk = 0; blk < S; blk += 3) {
#pragma unroll
            for (int u = 0; u < 3; u++) {
                const int s = blk + u;
                if (s < S) {
                    const bool bad = !mbar_wait(&full[slot], ph, p.spin);
                    if (bad) atomicExch(p.err, 1);
                    const float4 cq = *reinterpret_cast<const float4 *>(&st[slot].cur[ti + HT][4 * rq + HR]);
                    q[u][0] = cq.x;
                    q[u][1] = cq.y;
                    q[u][2] = cq.z;
                    q[u][3] = cq.w;
                    if (s >= 2) {
                        const int y = y0 + s - 2;
                        const int hs = slot == 0 ? RING - 1 : slot - 1;  // stage s-1: plane y and its halo
                        const float(*H)[WR] = st[hs].cur;
                        const float *um = q[(u + 1) % 3], *uc = q[(u + 2) % 3], *up = q[u];
                        const float4 pv = *reinterpret_cast<const float4 *>(&st[slot].prv[ti][4 * rq]);
                        const float4 vv = *reinterpret_cast<const float4 *>(&st[slot].vel[ti][4 * rq]);
                        float2 lap01 = make_float2(0.f, 0.f), lap23 = lap01;
                        const bool ph_in = y >= 4 && y < n3 - 4;
                        if (th_in && ph_in && any_r) {
                            const float rm = H[ti + HT][4 * rq + HR - 1], rp = H[ti + HT][4 * rq + HR + 4];
                            const float4 tm = *reinterpret_cast<const float4 *>(&H[ti][4 * rq + HR]);
                            const float4 tp = *reinterpret_cast<const float4 *>(&H[ti + 2 * HT][4 * rq + HR]);
                            // pair (0, 1) and pair (2, 3): r - 1 and r + 1 of both cells
                            const float2 c01 = make_float2(uc[0], uc[1]), c23 = make_float2(uc[2], uc[3]);
                            const float2 mi01 = make_float2(rm, uc[0]), pl01 = make_float2(uc[1], uc[2]);
                            const float2 mi23 = make_float2(uc[1], uc[2]), pl23 = make_float2(uc[3], rp);
                            auto lap2 = [&](float2 c, float2 mi, float2 pl, float2 tmv, float2 tpv, float2 umv,
                                            float2 upv, float2 a2, float2 cr, float2 b, float2 dd) {
                                const float2 pra = __fmul2_rn(__ffma2_rn(mi, m1, pl), r0v);
                                const float2 ppra = __fmul2_rn(__fadd2_rn(__ffma2_rn(c, m2, pl), mi), r1v);
                                const float2 pth = __fmul2_rn(__ffma2_rn(tmv, m1, tpv), r2v);
                                const float2 ppth = __fmul2_rn(__fadd2_rn(__ffma2_rn(c, m2, tpv), tmv), r3v);
                                const float2 ppph = __fmul2_rn(__fadd2_rn(__ffma2_rn(c, m2, upv), umv), r4v);
                                float2 l = __ffma2_rn(a2, pra, ppra);
                                l = __ffma2_rn(b, pth, l);
                                l = __ffma2_rn(cr, ppth, l);
                                return __ffma2_rn(dd, ppph, l);
                            };
                            lap01 = lap2(c01, mi01, pl01, make_float2(tm.x, tm.y), make_float2(tp.x, tp.y),
                                         make_float2(um[0], um[1]), make_float2(up[0], up[1]),
                                         make_float2(A2.x, A2.y), make_float2(Cr.x, Cr.y), make_float2(B.x, B.y),
                                         make_float2(D.x, D.y));
                            lap23 = lap2(c23, mi23, pl23, make_float2(tm.z, tm.w), make_float2(tp.z, tp.w),
                                         make_float2(um[2], um[3]), make_float2(up[2], up[3]),
                                         make_float2(A2.z, A2.w), make_float2(Cr.z, Cr.w), make_float2(B.z, B.w),
                                         make_float2(D.z, D.w));
                            if (!rin[0]) lap01.x = 0.f;
                            if (!rin[1]) lap01.y = 0.f;
                            if (!rin[2]) lap23.x = 0.f;
                            if (!rin[3]) lap23.y = 0.f;
                        }
                        const float2 a01 = __fmul2_rn(dt2v, __fmul2_rn(make_float2(vv.x, vv.y), make_float2(vv.x, vv.y)));
                        const float2 a23 = __fmul2_rn(dt2v, __fmul2_rn(make_float2(vv.z, vv.w), make_float2(vv.z, vv.w)));
                        const float2 f01 = __ffma2_rn(a01, lap01, __fadd2_rn(make_float2(uc[0], uc[1]),
                                                                              make_float2(uc[0], uc[1])));
                        const float2 f23 = __ffma2_rn(a23, lap23, __fadd2_rn(make_float2(uc[2], uc[3]),
                                                                              make_float2(uc[2], uc[3])));
                        float f[4] = {f01.x, f01.y, f23.x, f23.y};
                        const float pr[4] = {pv.x, pv.y, pv.z, pv.w};
                        const bool undamped = tile_undamped && y >= nb && y <= n3 - nb;
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const int si = undamped ? 0 : sph_sponge_index(r + j, y, t, n1, n3, n2, nb);
                            float v = f[j] - sph_damp(pr[j], si, s_ftab);
                            if (mask3 && (r + j > n1 - nb || (r + j < p.a.spill && (t >= 1 || y >= 1)))) v = 0.f;
                            f[j] = sph_damp(v, si, s_ftab);
                        }
                        if (col_ok) *reinterpret_cast<float4 *>(dst) = make_float4(f[0], f[1], f[2], f[3]);
                        dst += plane;
                    }
                    if (__syncthreads_or(bad)) {
                        // drain: wait (bounded) for every copy still in flight, then leave
                        if (tid == 0) {
                            const int issued = min(S, max(RING, s - 1 + RING));
                            for (int k = s; k < issued; k++) {
                                const int x = slot0 + k;
                                mbar_wait(&full[x % RING], ph0 ^ (uint32_t)((x / RING) & 1), SPIN_LIMIT);
                            }
                        }
                        __syncthreads();
                        return;
                    }
                    // stage s-1's slot is free (its centre values are in the queue)
                    if (tid == 0 && s >= 1 && s - 1 + RING < S) issue(s - 1 + RING);
                    if (++slot == RING) {
                        slot = 0;
                        ph ^= 1u;
                    }
                }
            }
        }
        const int x = slot0 + S;
        ph0 ^= (uint32_t)((x / RING) & 1);
        slot0 = x % RING;
    }
}

bool sphA_tma_eligible(const Grid &g, int nb) {
    return g.n1 % 4 == 0 && g.n1 >= 16 && g.n2 >= 16 && g.n3 >= 3 && nb < sp3::FTAB_MAX;
}

// tensor maps: [0] u[0] halo box, [1] u[1] halo box, [2] u[0] tile, [3] u[1]
// tile (the level fields of all shots stacked along phi), [4] vel tile
bool sphA_tma_maps(CUtensorMap *maps, float *const u[2], const float *vel, const Grid &g, int nshot) {
    using namespace sp3;
    const int n3s = g.n3 * (nshot > 0 ? nshot : 1);
    return make_tmap_3d(&maps[0], u[0], g.n1, g.n2, n3s, WR, WT) &&
           make_tmap_3d(&maps[1], u[1], g.n1, g.n2, n3s, WR, WT) &&
           make_tmap_3d(&maps[2], u[0], g.n1, g.n2, n3s, TR, TT) &&
           make_tmap_3d(&maps[3], u[1], g.n1, g.n2, n3s, TR, TT) &&
           make_tmap_3d(&maps[4], vel, g.n1, g.n2, g.n3, TR, TT);
}

Step3Launch sphA_tma_shape(const Grid &g, int nshot, int num_sms, int L) {
    using namespace sp3;
    Step3Launch s{};
    s.L = L > 0 ? L : 64;
    s.ntz = (g.n1 + TR - 1) / TR;
    s.ntx = (g.n2 + TT - 1) / TT;
    s.nchunks = (g.n3 + s.L - 1) / s.L;
    s.items = s.ntz * s.ntx * s.nchunks * (nshot > 0 ? nshot : 1);
    s.grid = std::min(s.items, 2 * num_sms);
    s.smem = RING * sizeof(Stage) + 128;
    return s;
}

cudaError_t launch_stepA_sph_tma(const CUtensorMap &cur, const CUtensorMap &prv, const CUtensorMap &vel, float *nxt,
                                 const StepAParams &pa, const Step3Launch &sh, unsigned long long *counter,
                                 unsigned long long base, int *err, long long spin, cudaStream_t s, int cur_f0,
                                 int prv_f0) {
    SphTmaParams p{};
    p.a = pa;
    p.cur_f0 = cur_f0;
    p.prv_f0 = prv_f0;
    p.L = sh.L;
    p.ntr = sh.ntz;
    p.ntt = sh.ntx;
    p.nchunks = sh.nchunks;
    p.nshot = pa.nshot > 0 ? pa.nshot : 1;
    p.counter = counter;
    p.base = base;
    p.err = err;
    p.nxt = nxt;
    p.spin = spin >= 0 ? spin : sp3::SPIN_LIMIT;
    cudaFuncSetAttribute(k_stepA_sph_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem);
    k_stepA_sph_tma<<<sh.grid, sp3::NTHREADS, sh.smem, s>>>(cur, prv, vel, p);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Adjoint step of the spherical scheme (the update of k_adjA_sph2, TMA-staged):
//   z_j = W M (L^T(I c z_{j+1}) + 2 z_{j+1} - W z_{j+2}),  c = dt^2 v^2,
//   G += z_{j+1} L(A_j)  (or z_{j+1} A_j for the cross-correlation image),
// on interior cells (at least 4 from every face).  L^T gathers this cell's
// weight in each neighbour's stencil times the neighbour's I c z.  Per plane
// the ring holds the 72 x 18 boxes of z_{j+1}, v and A_j, and for the plane
// being updated the 64 x 16 boxes of z_{j+2} and of G (float pairs, a
// 128 x 16 float box); the phi neighbours of I c z and of A come from 3-plane
// register queues.  z_j and G are written back with plain 16-byte stores.

namespace sa3 {
using sp3::HR;
using sp3::HT;
using sp3::TR;
using sp3::TT;
using sp3::WR;
using sp3::WT;
constexpr int RING = 4, NTHREADS = 256;
constexpr uint32_t BYTES_HALOS = 3 * WR * WT * 4, BYTES_OUT = TR * TT * 4 + 2 * TR * TT * 4;
constexpr int PAD = (128 - (WT * WR * 4) % 128) % 128 / 4;

struct __align__(128) Stage {
    float x[WT][WR];
    float px[PAD];
    float v[WT][WR];
    float pv[PAD];
    float a[WT][WR];
    float pa[PAD];
    float y[TT][TR];
    float g[TT][2 * TR];
};
static_assert(sizeof(Stage) % 128 == 0, "stage size");
static_assert(offsetof(Stage, v) % 128 == 0 && offsetof(Stage, a) % 128 == 0 && offsetof(Stage, y) % 128 == 0 &&
                  offsetof(Stage, g) % 128 == 0,
              "box alignment");
}  // namespace sa3

struct SphAdjParams {
    StepAParams a;
    int L, ntr, ntt, nchunks;
    int a_f0;  // plane offset of A_j in its map
    unsigned long long *counter;
    unsigned long long base;
    int *err;
    float *Y;
    float2 *G;
    int xcorr;
    long long spin;
};

__global__ void __launch_bounds__(sa3::NTHREADS, 2)
    k_adjA_sph_tma(const __grid_constant__ CUtensorMap tm_x, const __grid_constant__ CUtensorMap tm_v,
                   const __grid_constant__ CUtensorMap tm_a, const __grid_constant__ CUtensorMap tm_y,
                   const __grid_constant__ CUtensorMap tm_g, const SphAdjParams p) {
    using namespace sa3;
    extern __shared__ unsigned char smem_raw[];
    Stage *st = reinterpret_cast<Stage *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    __shared__ __align__(8) uint64_t full[RING];
    __shared__ int s_item;
    __shared__ float s_ftab[sp3::FTAB_MAX];

    const int tid = threadIdx.x;
    const int rq = tid & 15, ti = tid >> 4;
    for (int i = tid; i <= p.a.nb && i < sp3::FTAB_MAX; i += NTHREADS) s_ftab[i] = p.a.ftab[i];
    if (tid == 0) {
        for (int r = 0; r < RING; r++) mbar_init(&full[r], 1);
        fence_mbar_init();
        prefetch_tmap(&tm_x);
        prefetch_tmap(&tm_v);
        prefetch_tmap(&tm_a);
        prefetch_tmap(&tm_y);
        prefetch_tmap(&tm_g);
    }
    if (__syncthreads_or(tid == 0 && *(volatile int *)p.err != 0)) return;

    const int n1 = p.a.g.n1, n2 = p.a.g.n2, n3 = p.a.g.n3, nb = p.a.nb;
    const int per_chunk = p.ntr * p.ntt;
    const int nitems = per_chunk * p.nchunks;
    const long long plane = (long long)n1 * n2;
    const float rd0 = p.a.rd[0], rd1 = p.a.rd[1], rd2 = p.a.rd[2], rd3 = p.a.rd[3], rd4 = p.a.rd[4];
    const float2 r0v = make_float2(rd0, rd0), r1v = make_float2(rd1, rd1), r2v = make_float2(rd2, rd2);
    const float2 r3v = make_float2(rd3, rd3), r4v = make_float2(rd4, rd4);
    const float2 m1 = make_float2(-1.f, -1.f), m2 = make_float2(-2.f, -2.f), two = make_float2(2.f, 2.f);
    const float dt2 = p.a.dt2;
    const float2 dt22 = make_float2(dt2, dt2);
    const bool mask3 = p.a.mask == 3;
    auto rin = [&](int r) { return r >= 4 && r < n1 - 4; };
    auto tin = [&](int t) { return t >= 4 && t < n2 - 4; };
    auto pin = [&](int f) { return f >= 4 && f < n3 - 4; };
    auto cx2 = [&](float2 v, float2 x) { return __fmul2_rn(__fmul2_rn(dt22, __fmul2_rn(v, v)), x); };  // c X
    auto cx1 = [&](float v, float x) { return (dt2 * (v * v)) * x; };
    // the forward Laplacian of a pair of cells (k_stepA_sph_march2's expressions)
    auto lap2 = [&](float2 c, float2 mi, float2 pl, float2 tmv, float2 tpv, float2 umv, float2 upv, float2 a2,
                    float2 cr, float2 b, float2 dd) {
        const float2 pra = __fmul2_rn(__ffma2_rn(mi, m1, pl), r0v);
        const float2 ppra = __fmul2_rn(__fadd2_rn(__ffma2_rn(c, m2, pl), mi), r1v);
        const float2 pth = __fmul2_rn(__ffma2_rn(tmv, m1, tpv), r2v);
        const float2 ppth = __fmul2_rn(__fadd2_rn(__ffma2_rn(c, m2, tpv), tmv), r3v);
        const float2 ppph = __fmul2_rn(__fadd2_rn(__ffma2_rn(c, m2, upv), umv), r4v);
        float2 l = __ffma2_rn(a2, pra, ppra);
        l = __ffma2_rn(b, pth, l);
        l = __ffma2_rn(cr, ppth, l);
        return __ffma2_rn(dd, ppph, l);
    };

    int slot0 = 0;
    uint32_t ph0 = 0;
    for (;;) {
        if (tid == 0) s_item = (int)(atomicAdd(p.counter, 1ull) - p.base);
        __syncthreads();
        const int item = s_item;
        if (item >= nitems || item < 0) break;
        const int tile = item % per_chunk, chunk = item / per_chunk;
        const int r0 = (tile % p.ntr) * TR, t0 = (tile / p.ntr) * TT;
        const int y0 = chunk * p.L, y1 = min(y0 + p.L, n3);
        const int S = (y1 - y0) + 2;

        // stage s: plane y0-1+s of z_{j+1}, v and A_j; from s = 2 on also
        // z_{j+2} and G of plane y0+s-2, the plane updated at stage s
        auto issue = [&](int s) {
            const int slot = (slot0 + s) % RING;
            const int f = y0 - 1 + s;
            const bool out = s >= 2;
            mbar_expect_tx(&full[slot], BYTES_HALOS + (out ? BYTES_OUT : 0));
            tma_load_3d(&st[slot].x[0][0], &tm_x, &full[slot], r0 - HR, t0 - HT, f);
            tma_load_3d(&st[slot].v[0][0], &tm_v, &full[slot], r0 - HR, t0 - HT, f);
            tma_load_3d(&st[slot].a[0][0], &tm_a, &full[slot], r0 - HR, t0 - HT, p.a_f0 + f);
            if (out) {
                tma_load_3d(&st[slot].y[0][0], &tm_y, &full[slot], r0, t0, f - 1);
                tma_load_3d(&st[slot].g[0][0], &tm_g, &full[slot], 2 * r0, t0, f - 1);
            }
        };
        if (tid == 0)
            for (int s = 0; s < RING && s < S; s++) issue(s);

        // per-thread constants: radii r .. r+3 of theta row t
        const int r = r0 + 4 * rq, t = t0 + ti;
        const bool col_ok = r < n1 && t < n2;
        const bool t_in = tin(t), tm_ok = tin(t - 1), tp_ok = tin(t + 1);
        bool c[4];
        bool any_c = false;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            c[j] = rin(r + j) && t_in;
            any_c = any_c || c[j];
        }
        float A2[4] = {0.f, 0.f, 0.f, 0.f}, Cr[4] = {0.f, 0.f, 0.f, 0.f}, B[4] = {0.f, 0.f, 0.f, 0.f},
              D[4] = {0.f, 0.f, 0.f, 0.f}, Bm[4] = {0.f, 0.f, 0.f, 0.f}, Bp[4] = {0.f, 0.f, 0.f, 0.f};
        float trm = 0.f, trp = 0.f;
        if (col_ok) {
            const long long tt = (long long)t * n1 + r;
            const float4 a4 = __ldg(reinterpret_cast<const float4 *>(p.a.tr0 + r));
            const float4 c4 = __ldg(reinterpret_cast<const float4 *>(p.a.tr1 + r));
            const float4 b4 = __ldg(reinterpret_cast<const float4 *>(p.a.tt0 + tt));
            const float4 d4 = __ldg(reinterpret_cast<const float4 *>(p.a.tt1 + tt));
            A2[0] = a4.x, A2[1] = a4.y, A2[2] = a4.z, A2[3] = a4.w;
            Cr[0] = c4.x, Cr[1] = c4.y, Cr[2] = c4.z, Cr[3] = c4.w;
            B[0] = b4.x, B[1] = b4.y, B[2] = b4.z, B[3] = b4.w;
            D[0] = d4.x, D[1] = d4.y, D[2] = d4.z, D[3] = d4.w;
            if (tm_ok) {
                const float4 m4 = __ldg(reinterpret_cast<const float4 *>(p.a.tt0 + tt - n1));
                Bm[0] = m4.x, Bm[1] = m4.y, Bm[2] = m4.z, Bm[3] = m4.w;
            }
            if (tp_ok) {
                const float4 q4 = __ldg(reinterpret_cast<const float4 *>(p.a.tt0 + tt + n1));
                Bp[0] = q4.x, Bp[1] = q4.y, Bp[2] = q4.z, Bp[3] = q4.w;
            }
            if (r >= 1) trm = __ldg(p.a.tr0 + r - 1);
            if (r + 4 < n1) trp = __ldg(p.a.tr0 + r + 4);
        }
        // this cell's weight in each neighbour's stencil (0 where the neighbour has none)
        float wrm[4], wrp[4], wtm[4], wtp[4], wc[4], wph[4];
        wrm[0] = (rin(r - 1) && t_in) ? fmaf(trm, rd0, rd1) : 0.f;
        wrp[3] = (rin(r + 4) && t_in) ? fmaf(-trp, rd0, rd1) : 0.f;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (j >= 1) wrm[j] = c[j - 1] ? fmaf(A2[j - 1], rd0, rd1) : 0.f;
            if (j <= 2) wrp[j] = c[j + 1] ? fmaf(-A2[j + 1], rd0, rd1) : 0.f;
            wtm[j] = (tm_ok && rin(r + j)) ? fmaf(Bm[j], rd2, Cr[j] * rd3) : 0.f;
            wtp[j] = (tp_ok && rin(r + j)) ? fmaf(-Bp[j], rd2, Cr[j] * rd3) : 0.f;
            wc[j] = -2.f * (rd1 + Cr[j] * rd3 + D[j] * rd4);
            wph[j] = D[j] * rd4;
        }
        const bool tile_undamped = r0 >= nb && r0 + TR - 1 <= n1 - nb && t0 >= nb && t0 + TT - 1 <= n2 - nb;
        const long long col = (long long)t * n1 + r;

        int slot = slot0;
        uint32_t ph = ph0;
        float q[3][4];   // I c z_{j+1} of the own cells (0 off the interior), stage s in q[s % 3]
        float qa[3][4];  // A_j of the own cells
#pragma unroll 1
        for (int blk = 0; blk < S; blk += 3) {
#pragma unroll
            for (int u = 0; u < 3; u++) {
                const int s = blk + u;
                if (s < S) {
                    const int y = y0 + s - 2;
                    const bool upd = s >= 2;
                    const bool phy = upd && pin(y);
                    const bool gok = col_ok && phy && any_c;
                    const long long idx = (long long)y * plane + col;
                    const bool bad = !mbar_wait(&full[slot], ph, p.spin);
                    if (bad) atomicExch(p.err, 1);
                    {
                        const float4 xs = *reinterpret_cast<const float4 *>(&st[slot].x[ti + HT][4 * rq + HR]);
                        const float4 vs = *reinterpret_cast<const float4 *>(&st[slot].v[ti + HT][4 * rq + HR]);
                        const float4 as = *reinterpret_cast<const float4 *>(&st[slot].a[ti + HT][4 * rq + HR]);
                        const float2 p01 = cx2(make_float2(vs.x, vs.y), make_float2(xs.x, xs.y));
                        const float2 p23 = cx2(make_float2(vs.z, vs.w), make_float2(xs.z, xs.w));
                        const bool pf = pin(y0 - 1 + s);
                        q[u][0] = c[0] && pf ? p01.x : 0.f;
                        q[u][1] = c[1] && pf ? p01.y : 0.f;
                        q[u][2] = c[2] && pf ? p23.x : 0.f;
                        q[u][3] = c[3] && pf ? p23.y : 0.f;
                        qa[u][0] = as.x;
                        qa[u][1] = as.y;
                        qa[u][2] = as.z;
                        qa[u][3] = as.w;
                    }
                    if (upd) {
                        const int hs = slot == 0 ? RING - 1 : slot - 1;  // stage s-1: plane y and its halo
                        const Stage &H = st[hs];
                        const float *ym = q[(u + 1) % 3], *yc = q[(u + 2) % 3], *yp = q[u];
                        const float *am = qa[(u + 1) % 3], *ac = qa[(u + 2) % 3], *ap = qa[u];
                        const float4 xc4 = *reinterpret_cast<const float4 *>(&H.x[ti + HT][4 * rq + HR]);
                        const float xc[4] = {xc4.x, xc4.y, xc4.z, xc4.w};
                        float2 lt01 = __fmul2_rn(make_float2(wph[0], wph[1]),
                                                 __fadd2_rn(make_float2(ym[0], ym[1]), make_float2(yp[0], yp[1])));
                        float2 lt23 = __fmul2_rn(make_float2(wph[2], wph[3]),
                                                 __fadd2_rn(make_float2(ym[2], ym[3]), make_float2(yp[2], yp[3])));
                        if (phy) {
                            lt01 = __ffma2_rn(make_float2(wc[0], wc[1]), make_float2(yc[0], yc[1]), lt01);
                            lt23 = __ffma2_rn(make_float2(wc[2], wc[3]), make_float2(yc[2], yc[3]), lt23);
                            const float yrm = wrm[0] != 0.f ? cx1(H.v[ti + HT][4 * rq + HR - 1],
                                                                  H.x[ti + HT][4 * rq + HR - 1]) : 0.f;
                            const float yrp = wrp[3] != 0.f ? cx1(H.v[ti + HT][4 * rq + HR + 4],
                                                                  H.x[ti + HT][4 * rq + HR + 4]) : 0.f;
                            lt01 = __ffma2_rn(make_float2(wrm[0], wrm[1]), make_float2(yrm, yc[0]), lt01);
                            lt01 = __ffma2_rn(make_float2(wrp[0], wrp[1]), make_float2(yc[1], yc[2]), lt01);
                            lt23 = __ffma2_rn(make_float2(wrm[2], wrm[3]), make_float2(yc[1], yc[2]), lt23);
                            lt23 = __ffma2_rn(make_float2(wrp[2], wrp[3]), make_float2(yc[3], yrp), lt23);
                            if (tm_ok) {
                                const float4 xm = *reinterpret_cast<const float4 *>(&H.x[ti][4 * rq + HR]);
                                const float4 vm = *reinterpret_cast<const float4 *>(&H.v[ti][4 * rq + HR]);
                                lt01 = __ffma2_rn(make_float2(wtm[0], wtm[1]),
                                                  cx2(make_float2(vm.x, vm.y), make_float2(xm.x, xm.y)), lt01);
                                lt23 = __ffma2_rn(make_float2(wtm[2], wtm[3]),
                                                  cx2(make_float2(vm.z, vm.w), make_float2(xm.z, xm.w)), lt23);
                            }
                            if (tp_ok) {
                                const float4 xp = *reinterpret_cast<const float4 *>(&H.x[ti + 2 * HT][4 * rq + HR]);
                                const float4 vp = *reinterpret_cast<const float4 *>(&H.v[ti + 2 * HT][4 * rq + HR]);
                                lt01 = __ffma2_rn(make_float2(wtp[0], wtp[1]),
                                                  cx2(make_float2(vp.x, vp.y), make_float2(xp.x, xp.y)), lt01);
                                lt23 = __ffma2_rn(make_float2(wtp[2], wtp[3]),
                                                  cx2(make_float2(vp.z, vp.w), make_float2(xp.z, xp.w)), lt23);
                            }
                        }
                        const float2 mu01 = __ffma2_rn(two, make_float2(xc[0], xc[1]), lt01);
                        const float2 mu23 = __ffma2_rn(two, make_float2(xc[2], xc[3]), lt23);
                        float out[4] = {mu01.x, mu01.y, mu23.x, mu23.y};
                        const float4 yv = *reinterpret_cast<const float4 *>(&st[slot].y[ti][4 * rq]);
                        const float yy[4] = {yv.x, yv.y, yv.z, yv.w};
                        const bool undamped = tile_undamped && y >= nb && y <= n3 - nb;
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const int si = undamped ? 0 : sph_sponge_index(r + j, y, t, n1, n3, n2, nb);
                            float m = fmaf(-sph_damp(1.f, si, s_ftab), yy[j], out[j]);
                            if (mask3 && (r + j > n1 - nb || (r + j < p.a.spill && (t >= 1 || y >= 1)))) m = 0.f;
                            out[j] = sph_damp(m, si, s_ftab);
                        }
                        if (col_ok) __stcs(reinterpret_cast<float4 *>(p.Y + idx), make_float4(out[0], out[1], out[2], out[3]));
                        if (gok) {
                            const float4 g0 = *reinterpret_cast<const float4 *>(&st[slot].g[ti][8 * rq]);
                            const float4 g1 = *reinterpret_cast<const float4 *>(&st[slot].g[ti][8 * rq + 4]);
                            float2 ga[4] = {make_float2(g0.x, g0.y), make_float2(g0.z, g0.w), make_float2(g1.x, g1.y),
                                            make_float2(g1.z, g1.w)};
                            float term[4];
                            if (p.xcorr) {
#pragma unroll
                                for (int j = 0; j < 4; j++) term[j] = __fmul_rn(xc[j], ac[j]);
                            } else {
                                const float rm = H.a[ti + HT][4 * rq + HR - 1], rp = H.a[ti + HT][4 * rq + HR + 4];
                                const float4 tm = *reinterpret_cast<const float4 *>(&H.a[ti][4 * rq + HR]);
                                const float4 tp = *reinterpret_cast<const float4 *>(&H.a[ti + 2 * HT][4 * rq + HR]);
                                const float2 l01 = lap2(make_float2(ac[0], ac[1]), make_float2(rm, ac[0]),
                                                        make_float2(ac[1], ac[2]), make_float2(tm.x, tm.y),
                                                        make_float2(tp.x, tp.y), make_float2(am[0], am[1]),
                                                        make_float2(ap[0], ap[1]), make_float2(A2[0], A2[1]),
                                                        make_float2(Cr[0], Cr[1]), make_float2(B[0], B[1]),
                                                        make_float2(D[0], D[1]));
                                const float2 l23 = lap2(make_float2(ac[2], ac[3]), make_float2(ac[1], ac[2]),
                                                        make_float2(ac[3], rp), make_float2(tm.z, tm.w),
                                                        make_float2(tp.z, tp.w), make_float2(am[2], am[3]),
                                                        make_float2(ap[2], ap[3]), make_float2(A2[2], A2[3]),
                                                        make_float2(Cr[2], Cr[3]), make_float2(B[2], B[3]),
                                                        make_float2(D[2], D[3]));
                                const float lp[4] = {l01.x, l01.y, l23.x, l23.y};
#pragma unroll
                                for (int j = 0; j < 4; j++) term[j] = __fmul_rn(xc[j], lp[j]);
                            }
#pragma unroll
                            for (int j = 0; j < 4; j++)
                                if (c[j]) ga[j] = gsum_add(ga[j], term[j]);
                            __stcs(reinterpret_cast<float4 *>(p.G + idx), make_float4(ga[0].x, ga[0].y, ga[1].x, ga[1].y));
                            __stcs(reinterpret_cast<float4 *>(p.G + idx + 2),
                                   make_float4(ga[2].x, ga[2].y, ga[3].x, ga[3].y));
                        }
                    }
                    if (__syncthreads_or(bad)) {
                        if (tid == 0) {
                            const int issued = min(S, max(RING, s - 1 + RING));
                            for (int k = s; k < issued; k++) {
                                const int x = slot0 + k;
                                mbar_wait(&full[x % RING], ph0 ^ (uint32_t)((x / RING) & 1), sp3::SPIN_LIMIT);
                            }
                        }
                        __syncthreads();
                        return;
                    }
                    if (tid == 0 && s >= 1 && s - 1 + RING < S) issue(s - 1 + RING);
                    if (++slot == RING) {
                        slot = 0;
                        ph ^= 1u;
                    }
                }
            }
        }
        const int x = slot0 + S;
        ph0 ^= (uint32_t)((x / RING) & 1);
        slot0 = x % RING;
    }
}

bool sphA_tma_level_maps(CUtensorMap *halo, CUtensorMap *tile, const float *base, const Grid &g, int nlevels) {
    const int n3s = g.n3 * (nlevels > 0 ? nlevels : 1);
    return (!halo || make_tmap_3d(halo, base, g.n1, g.n2, n3s, sp3::WR, sp3::WT)) &&
           (!tile || make_tmap_3d(tile, base, g.n1, g.n2, n3s, sp3::TR, sp3::TT));
}

// the accumulator pairs as a float field of 2 n1 floats per line, 128 x 16 boxes
bool sphA_tma_pair_map(CUtensorMap *m, const float2 *base, const Grid &g) {
    return make_tmap_3d(m, reinterpret_cast<const float *>(base), 2 * g.n1, g.n2, g.n3, 2 * sp3::TR, sp3::TT);
}

cudaError_t launch_adjA_sph_tma(const CUtensorMap &x_halo, const CUtensorMap &v_halo, const CUtensorMap &a_halo,
                                int a_f0, const CUtensorMap &y_tile, const CUtensorMap &g_tile, float *Y, float2 *G,
                                const StepAParams &pa, const Step3Launch &sh, unsigned long long *counter,
                                unsigned long long base, int *err, long long spin, bool xcorr, cudaStream_t s) {
    SphAdjParams p{};
    p.a = pa;
    p.L = sh.L;
    p.ntr = sh.ntz;
    p.ntt = sh.ntx;
    p.nchunks = sh.nchunks;
    p.a_f0 = a_f0;
    p.counter = counter;
    p.base = base;
    p.err = err;
    p.Y = Y;
    p.G = G;
    p.xcorr = xcorr ? 1 : 0;
    p.spin = spin >= 0 ? spin : sp3::SPIN_LIMIT;
    const int smem = (int)(sa3::RING * sizeof(sa3::Stage) + 128);
    cudaFuncSetAttribute(k_adjA_sph_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_adjA_sph_tma<<<sh.grid, sa3::NTHREADS, smem, s>>>(x_halo, v_halo, a_halo, y_tile, g_tile, p);
    return cudaGetLastError();
}

}  // namespace awe
