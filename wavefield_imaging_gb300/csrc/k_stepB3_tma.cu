// 3D 8th-order step of the CPU-program scheme, TMA-staged 2.5D blocking.
//
// A CTA owns a 64 (z) x 16 (x) tile and marches along y over a chunk of
// planes.  For every plane it TMA-loads (cp.async.bulk.tensor, mbarrier
// completion) the current level's 72 x 24 halo tile into a 9-deep ring (the
// halo of plane y is read when plane y+4 arrives, so five slots are in use)
// and, for the plane being updated, the previous level and v^2 dt^2 64 x 16
// tiles into a 5-deep ring, five planes ahead of the compute.  y-neighbours come from a 9-plane register queue
// (each thread owns a 4-cell z strip of one x column), z- and x-neighbours
// from the halo tile in shared memory; the leapfrog update, the sponge of
// the previous level (applied on read) and of the new level (outside the ABC
// shell) are fused, and the 4-cell result is written with one 16-byte store.
// Work items (tile, y-chunk) are handed out by a global atomic counter, so
// the persistent grid (2 CTAs per SM) stays balanced.
//
// Operation order per cell is that of ts_kernel.c:286-307
// (lap = u*c0 + sum_k [(z pair)*cz + (x pair)*cx + (y pair)*cy]), so the
// EXACT instantiation is bit-identical to k_stepB.
#include <cuda.h>
#include <cuda_runtime.h>

#include "awe_internal.h"
#include "gsum.cuh"
#include "fp_exact.cuh"
#include "tma.cuh"

#include <algorithm>

namespace awe {

namespace s3 {
constexpr int TZ = 64, TX = 16, HALO = 4, RING = 9, TRING = 5, NOPQ = 4;
constexpr int HZ = TZ + 2 * HALO, HX = TX + 2 * HALO;
constexpr int NTHREADS = 256;
constexpr uint32_t BYTES_HALO = HZ * HX * 4, BYTES_TILE = TZ * TX * 4;
constexpr long long SPIN_LIMIT = 1ll << 22;

struct __align__(128) Stage {  // halo ring entry
    float cur[HX][HZ];
};
struct __align__(128) Tile {  // tile ring entry
    float prv[TX][TZ];
    float vel[TX][TZ];
};
static_assert(sizeof(Stage) % 128 == 0 && sizeof(Tile) % 128 == 0, "stage size");
// the tile of output plane o is refilled (for o + TRING) only after plane o
// is computed: the refill is issued after stage o + 2 NOPQ + TRING - RING + NOPQ
static_assert(TRING >= RING - NOPQ, "tile ring depth");
}  // namespace s3

struct Step3Params {
    int n1, n2, n3;
    float c0, cz[5], cx[5], cy[5];
    const float *w1, *w2, *w3;
    int damp_prev, sponge_new, shell;
    int ilo[3], ihi[3];  // undamped interior per axis
    int L, ntz, ntx, nchunks;
    unsigned long long *counter;
    unsigned long long base;
    int *err;
    float *nxt;
    // MODE 1: L(cur) of interior cells (0 elsewhere) stored here, laid out as the field
    float *lap_out;
    // MODE 2 (adjoint step): cur = I vel2 nu, prv = nu_{k+1} (overwritten by
    // mu = W lambda), vel = nu_k; lap_v = L(V_k); grad += I nu L(V_k) (FP64)
    const float *lap_v;
    float2 *grad;  // gradient accumulators (compensated pairs)
    long long spin;  // polls of a compute-side wait before it gives up (the drain keeps SPIN_LIMIT)
};

template <bool EXACT>
__device__ __forceinline__ float damp3(float v, float a, float b, float c) {
    return fmul<EXACT>(fmul<EXACT>(fmul<EXACT>(v, a), b), c);
}

// MODE 0: forward step; 1: forward step that also stores L(cur); 2: adjoint
// step of the misfit gradient (the tile loads are the same, the epilogue differs)
template <bool EXACT, int MODE>
__global__ void __launch_bounds__(s3::NTHREADS, 2)
    k_stepB3_o8(const __grid_constant__ CUtensorMap tm_cur, const __grid_constant__ CUtensorMap tm_prv,
                const __grid_constant__ CUtensorMap tm_vel, const Step3Params p) {
    using namespace s3;
    extern __shared__ unsigned char smem_raw[];
    Stage *st = reinterpret_cast<Stage *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    Tile *tl = reinterpret_cast<Tile *>(st + RING);
    float *s_w3 = reinterpret_cast<float *>(tl + TRING);  // y sponge factors (1 without a sponge)
    __shared__ __align__(8) uint64_t full[RING];
    __shared__ int s_item;

    const int tid = threadIdx.x;
    const int zq = tid & 15, xi = tid >> 4;
    for (int i = tid; i < p.n3; i += NTHREADS) s_w3[i] = p.w3 ? p.w3[i] : 1.f;
    if (tid == 0) {
        for (int r = 0; r < RING; r++) mbar_init(&full[r], 1);
        fence_mbar_init();
        prefetch_tmap(&tm_cur);
        prefetch_tmap(&tm_prv);
        prefetch_tmap(&tm_vel);
    }
    // an earlier launch that gave up on a wait leaves the flag set: do nothing
    if (__syncthreads_or(tid == 0 && *(volatile int *)p.err != 0)) return;

    const int nitems = p.ntz * p.ntx * p.nchunks;
    const long long plane = (long long)p.n1 * p.n2;
    // ring position of the current item's first plane: slot and mbarrier
    // parity; tile ring slot of its first output plane
    int slot0 = 0, tile0 = 0;
    uint32_t ph0 = 0;
    for (;;) {
        if (tid == 0) s_item = (int)(atomicAdd(p.counter, 1ull) - p.base);
        __syncthreads();
        const int item = s_item;
        if (item >= nitems || item < 0) break;
        const int tile = item % (p.ntz * p.ntx), chunk = item / (p.ntz * p.ntx);
        const int z0 = (tile % p.ntz) * TZ, x0 = (tile / p.ntz) * TX;
        const int y0 = chunk * p.L, y1 = min(y0 + p.L, p.n3);
        const int S = (y1 - y0) + 2 * NOPQ;

        auto issue = [&](int s) {
            const int slot = (slot0 + s) % RING;
            const bool out = s >= 2 * NOPQ;
            mbar_expect_tx(&full[slot], BYTES_HALO + (out ? 2 * BYTES_TILE : 0));
            tma_load_3d(&st[slot].cur[0][0], &tm_cur, &full[slot], z0 - HALO, x0 - HALO, y0 - NOPQ + s);
            if (out) {
                const int pl = y0 + s - 2 * NOPQ;
                Tile &t = tl[(tile0 + s - 2 * NOPQ) % TRING];
                tma_load_3d(&t.prv[0][0], &tm_prv, &full[slot], z0, x0, pl);
                tma_load_3d(&t.vel[0][0], &tm_vel, &full[slot], z0, x0, pl);
            }
        };
        if (tid == 0)
            for (int s = 0; s < RING && s < S; s++) issue(s);

        // per-thread constants
        const int zg = z0 + 4 * zq, x = x0 + xi;
        const bool col_ok = x < p.n2 && zg < p.n1;
        float wz[4], wx = 1.f;
        bool zin[4], zshell[4];
        const bool xin = x >= NOPQ && x < p.n2 - NOPQ;
        const bool xshell = x < p.shell || x >= p.n2 - p.shell;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int z = zg + i;
            wz[i] = (p.w1 && z < p.n1) ? __ldg(p.w1 + z) : 1.f;
            zin[i] = z >= NOPQ && z < p.n1 - NOPQ;
            zshell[i] = z < p.shell || z >= p.n1 - p.shell;
        }
        if (p.w2 && x < p.n2) wx = __ldg(p.w2 + x);
        // the whole tile lies where the z and x sponge factors are exactly 1
        const bool tile_undamped = z0 >= p.ilo[0] && z0 + TZ <= p.ihi[0] && x0 >= p.ilo[1] && x0 + TX <= p.ihi[1];
        // every column of the tile is at least NOPQ from the z and x faces
        const bool tile_inner = z0 >= NOPQ && z0 + TZ <= p.n1 - NOPQ && x0 >= NOPQ && x0 + TX <= p.n2 - NOPQ;
        float *dst = p.nxt + ((long long)y0 * p.n2 + x) * p.n1 + zg;

        int slot = slot0;  // ring slot and parity of plane s
        uint32_t ph = ph0;
        float q[9][4];  // y queue: plane y0-4+s lives in q[s % 9]
#pragma unroll 1
        for (int blk = 0; blk < S; blk += 9) {
#pragma unroll
            for (int u = 0; u < 9; u++) {
                const int s = blk + u;
                if (s < S) {
                    // adjoint: the plane's L(V) and gradient loads go out before the
                    // ring wait and the stencil, so their latency overlaps both
                    float4 lvp = make_float4(0.f, 0.f, 0.f, 0.f);
                    float4 gp0 = make_float4(0.f, 0.f, 0.f, 0.f), gp1 = gp0;
                    bool gok = false;
                    long long gip = 0;
                    if constexpr (MODE == 2) {
                        if (s >= 2 * NOPQ) {
                            const int yp = y0 + s - 2 * NOPQ;
                            gok = col_ok && xin && yp >= NOPQ && yp < p.n3 - NOPQ;
                            gip = ((long long)yp * p.n2 + x) * p.n1 + zg;
                            if (gok) {
                                lvp = __ldcs(reinterpret_cast<const float4 *>(p.lap_v + gip));
                                gp0 = __ldcs(reinterpret_cast<const float4 *>(p.grad + gip));
                                gp1 = __ldcs(reinterpret_cast<const float4 *>(p.grad + gip + 2));
                            }
                        }
                    }
                    const bool bad = !mbar_wait(&full[slot], ph, p.spin);
                    if (bad) atomicExch(p.err, 1);
                    const float4 cq = *reinterpret_cast<const float4 *>(&st[slot].cur[xi + HALO][4 * zq + HALO]);
                    q[u][0] = cq.x;
                    q[u][1] = cq.y;
                    q[u][2] = cq.z;
                    q[u][3] = cq.w;
                    if (s >= 2 * NOPQ) {
                        const int y = y0 + s - 2 * NOPQ;
                        const int hs = slot >= NOPQ ? slot - NOPQ : slot + RING - NOPQ;  // halo tile of plane y
                        const float(*H)[HZ] = st[hs].cur;
                        float zw[12];
#pragma unroll
                        for (int v = 0; v < 3; v++) {
                            const float4 t = *reinterpret_cast<const float4 *>(&H[xi + HALO][4 * zq + 4 * v]);
                            zw[4 * v] = t.x;
                            zw[4 * v + 1] = t.y;
                            zw[4 * v + 2] = t.z;
                            zw[4 * v + 3] = t.w;
                        }
                        const int jc = (u + 1 + 4) % 9;  // queue slot of plane y: ((s - 8) + 4) % 9
                        float lap[4];
                        if constexpr (EXACT) {
#pragma unroll
                            for (int i = 0; i < 4; i++) lap[i] = fmul<true>(zw[4 + i], p.c0);
#pragma unroll
                            for (int k = 1; k <= NOPQ; k++) {
                                const float4 xm = *reinterpret_cast<const float4 *>(&H[xi + HALO - k][4 * zq + HALO]);
                                const float4 xp = *reinterpret_cast<const float4 *>(&H[xi + HALO + k][4 * zq + HALO]);
                                const float xmv[4] = {xm.x, xm.y, xm.z, xm.w}, xpv[4] = {xp.x, xp.y, xp.z, xp.w};
#pragma unroll
                                for (int i = 0; i < 4; i++) {
                                    const float zp = fadd<true>(zw[4 + i - k], zw[4 + i + k]);
                                    const float xpair = fadd<true>(xmv[i], xpv[i]);
                                    const float ypair = fadd<true>(q[(jc + 9 - k) % 9][i], q[(jc + k) % 9][i]);
                                    // ts_kernel.c:292-300 order: (z*cz + x*cx) + y*cy, then into lap
                                    float t = fadd<true>(fmul<true>(zp, p.cz[k]), fmul<true>(xpair, p.cx[k]));
                                    t = fadd<true>(t, fmul<true>(ypair, p.cy[k]));
                                    lap[i] = fadd<true>(lap[i], t);
                                }
                            }
                        } else {
                            // packed FP32x2 (add.f32x2 / fma.rn.f32x2): two cells per instruction
                            float2 l01 = __fmul2_rn(make_float2(zw[4], zw[5]), make_float2(p.c0, p.c0));
                            float2 l23 = __fmul2_rn(make_float2(zw[6], zw[7]), make_float2(p.c0, p.c0));
#pragma unroll
                            for (int k = 1; k <= NOPQ; k++) {
                                const float4 xm = *reinterpret_cast<const float4 *>(&H[xi + HALO - k][4 * zq + HALO]);
                                const float4 xp = *reinterpret_cast<const float4 *>(&H[xi + HALO + k][4 * zq + HALO]);
                                float2 z01, z23;
                                if (k % 2 == 0) {  // pairs aligned with the 16-byte loads
                                    z01 = __fadd2_rn(make_float2(zw[4 - k], zw[5 - k]), make_float2(zw[4 + k], zw[5 + k]));
                                    z23 = __fadd2_rn(make_float2(zw[6 - k], zw[7 - k]), make_float2(zw[6 + k], zw[7 + k]));
                                } else {
                                    z01 = make_float2(zw[4 - k] + zw[4 + k], zw[5 - k] + zw[5 + k]);
                                    z23 = make_float2(zw[6 - k] + zw[6 + k], zw[7 - k] + zw[7 + k]);
                                }
                                const float2 x01 = __fadd2_rn(make_float2(xm.x, xm.y), make_float2(xp.x, xp.y));
                                const float2 x23 = __fadd2_rn(make_float2(xm.z, xm.w), make_float2(xp.z, xp.w));
                                const float *qa = q[(jc + 9 - k) % 9], *qb = q[(jc + k) % 9];
                                const float2 y01 = __fadd2_rn(make_float2(qa[0], qa[1]), make_float2(qb[0], qb[1]));
                                const float2 y23 = __fadd2_rn(make_float2(qa[2], qa[3]), make_float2(qb[2], qb[3]));
                                const float2 cz = make_float2(p.cz[k], p.cz[k]), cx = make_float2(p.cx[k], p.cx[k]);
                                const float2 cy = make_float2(p.cy[k], p.cy[k]);
                                l01 = __ffma2_rn(z01, cz, l01);
                                l23 = __ffma2_rn(z23, cz, l23);
                                l01 = __ffma2_rn(x01, cx, l01);
                                l23 = __ffma2_rn(x23, cx, l23);
                                l01 = __ffma2_rn(y01, cy, l01);
                                l23 = __ffma2_rn(y23, cy, l23);
                            }
                            lap[0] = l01.x;
                            lap[1] = l01.y;
                            lap[2] = l23.x;
                            lap[3] = l23.y;
                        }
                        const Tile &tp = tl[(tile0 + s - 2 * NOPQ) % TRING];
                        const float4 pv = *reinterpret_cast<const float4 *>(&tp.prv[xi][4 * zq]);
                        const float4 vv = *reinterpret_cast<const float4 *>(&tp.vel[xi][4 * zq]);
                        const float prv4[4] = {pv.x, pv.y, pv.z, pv.w}, vel4[4] = {vv.x, vv.y, vv.z, vv.w};
                        const bool yin = y >= NOPQ && y < p.n3 - NOPQ;
                        // every sponge factor of this plane of the tile is 1: the
                        // multiplies are identities and are skipped (CTA-uniform)
                        const bool undamped = tile_undamped && y >= p.ilo[2] && y < p.ihi[2];
                        float out[4];
                        if constexpr (MODE == 2) {
                            // lambda = 2 I nu + L(I vel2 nu) + W (1 - 2 I) nu_{k+1}; out = W lambda
                            const float wy = undamped ? 1.f : s_w3[y];
                            const float lv4[4] = {lvp.x, lvp.y, lvp.z, lvp.w};
                            float2 ga[4] = {make_float2(gp0.x, gp0.y), make_float2(gp0.z, gp0.w),
                                            make_float2(gp1.x, gp1.y), make_float2(gp1.z, gp1.w)};
#pragma unroll
                            for (int i = 0; i < 4; i++) {
                                const bool in = zin[i] && xin && yin;
                                const float w = undamped ? 1.f : (wz[i] * wx) * wy;
                                const float nu = vel4[i];
                                const float lam = (in ? 2.f * nu : 0.f) + lap[i] + (in ? -w : w) * prv4[i];
                                out[i] = w * lam;
                                // product in FP32 (the fields are FP32), compensated FP32 sum
                                if (in) ga[i] = gsum_add(ga[i], __fmul_rn(nu, lv4[i]));
                            }
                            if (gok) {
                                float2 *G = p.grad + gip;
                                __stcs(reinterpret_cast<float4 *>(G), make_float4(ga[0].x, ga[0].y, ga[1].x, ga[1].y));
                                __stcs(reinterpret_cast<float4 *>(G + 2), make_float4(ga[2].x, ga[2].y, ga[3].x, ga[3].y));
                            }
                        } else if (!EXACT && undamped && tile_inner && yin) {
                            // every cell of the strip is interior and undamped: packed update
                            const float2 two = make_float2(2.f, 2.f);
                            const float2 t01 = __ffma2_rn(two, make_float2(zw[4], zw[5]), make_float2(-pv.x, -pv.y));
                            const float2 t23 = __ffma2_rn(two, make_float2(zw[6], zw[7]), make_float2(-pv.z, -pv.w));
                            const float2 o01 = __ffma2_rn(make_float2(vv.x, vv.y), make_float2(lap[0], lap[1]), t01);
                            const float2 o23 = __ffma2_rn(make_float2(vv.z, vv.w), make_float2(lap[2], lap[3]), t23);
                            out[0] = o01.x;
                            out[1] = o01.y;
                            out[2] = o23.x;
                            out[3] = o23.y;
                        } else if (undamped) {
#pragma unroll
                            for (int i = 0; i < 4; i++) {
                                const float pr = prv4[i], u0 = zw[4 + i];
                                float o = pr;
                                if (zin[i] && xin && yin) {
                                    if constexpr (EXACT)
                                        o = sum3_rn(__fmul_rn(vel4[i], lap[i]), __fadd_rn(u0, u0), -pr);
                                    else
                                        o = fmaf(vel4[i], lap[i], 2.f * u0 - pr);
                                }
                                out[i] = o;
                            }
                        } else {
                            const float wy = s_w3[y];
                            const bool yshell = y < p.shell || y >= p.n3 - p.shell;
#pragma unroll
                            for (int i = 0; i < 4; i++) {
                                float pr = prv4[i];
                                if (p.damp_prev) pr = damp3<EXACT>(pr, wz[i], wx, wy);
                                float o = pr;
                                if (zin[i] && xin && yin) {
                                    const float u0 = zw[4 + i];
                                    if constexpr (EXACT)
                                        o = sum3_rn(__fmul_rn(vel4[i], lap[i]), __fadd_rn(u0, u0), -pr);
                                    else
                                        o = fmaf(vel4[i], lap[i], 2.f * u0 - pr);
                                }
                                if (p.sponge_new && !(zshell[i] || xshell || yshell))
                                    o = damp3<EXACT>(o, wz[i], wx, wy);
                                out[i] = o;
                            }
                        }
                        if (col_ok) *reinterpret_cast<float4 *>(dst) = make_float4(out[0], out[1], out[2], out[3]);
                        if constexpr (MODE == 1) {
                            if (col_ok) {
                                float lo[4];
#pragma unroll
                                for (int i = 0; i < 4; i++) lo[i] = (zin[i] && xin && yin) ? lap[i] : 0.f;
                                *reinterpret_cast<float4 *>(p.lap_out + (dst - p.nxt)) =
                                    make_float4(lo[0], lo[1], lo[2], lo[3]);
                            }
                        }
                        dst += plane;
                    }
                    if (__syncthreads_or(bad)) {
                        // drain: wait (bounded) for every copy still in flight, then leave
                        if (tid == 0) {
                            const int issued = min(S, max(RING, s - NOPQ + RING));
                            for (int t = s; t < issued; t++) {
                                const int tt = slot0 + t;
                                mbar_wait(&full[tt % RING], ph0 ^ (uint32_t)((tt / RING) & 1), SPIN_LIMIT);
                            }
                        }
                        __syncthreads();
                        return;
                    }
                    if (tid == 0 && s >= NOPQ && s - NOPQ + RING < S) issue(s - NOPQ + RING);
                    if (++slot == RING) {
                        slot = 0;
                        ph ^= 1u;
                    }
                }
            }
        }
        const int t = slot0 + S;
        ph0 ^= (uint32_t)((t / RING) & 1);
        slot0 = t % RING;
        tile0 = (tile0 + (S - 2 * NOPQ)) % TRING;
    }
}
// cuTensorMapEncodeTiled, fetched from the driver at run time (no link-time libcuda dependency)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn g_encode = nullptr;

static bool encode_fn() {
    if (g_encode) return true;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    // the function as introduced in CUDA 12.0 (its ABI version)
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
        return false;
    g_encode = reinterpret_cast<EncodeTiledFn>(fn);
    return true;
}

bool make_tmap_3d(CUtensorMap *m, const float *base, int n1, int n2, int n3, int b1, int b2) {
    if (!encode_fn()) return false;
    cuuint64_t dims[3] = {(cuuint64_t)n1, (cuuint64_t)n2, (cuuint64_t)n3};
    cuuint64_t strides[2] = {(cuuint64_t)n1 * 4, (cuuint64_t)n1 * n2 * 4};
    cuuint32_t box[3] = {(cuuint32_t)b1, (cuuint32_t)b2, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

void stepB3_tma_boxes(int *halo1, int *halo2, int *tile1, int *tile2) {
    *halo1 = s3::HZ;
    *halo2 = s3::HX;
    *tile1 = s3::TZ;
    *tile2 = s3::TX;
}

bool stepB3_tma_eligible(int ndim, int nop, bool rho, const Grid &g) {
    // n3 <= 16384: the y sponge factors fit beside the rings in shared memory
    return ndim == 3 && nop == 4 && !rho && g.n1 % 4 == 0 && g.n1 >= 16 && g.n2 >= 16 && g.n3 >= 9 && g.n3 <= 16384;
}

// tensor maps: [0] u[0] halo box, [1] u[1] halo box, [2] u[0] tile, [3] u[1] tile, [4] vel tile
bool stepB3_tma_maps(CUtensorMap *maps, float *const u[2], const float *vel, const Grid &g) {
    using namespace s3;
    return make_tmap_3d(&maps[0], u[0], g.n1, g.n2, g.n3, HZ, HX) &&
           make_tmap_3d(&maps[1], u[1], g.n1, g.n2, g.n3, HZ, HX) &&
           make_tmap_3d(&maps[2], u[0], g.n1, g.n2, g.n3, TZ, TX) &&
           make_tmap_3d(&maps[3], u[1], g.n1, g.n2, g.n3, TZ, TX) &&
           make_tmap_3d(&maps[4], vel, g.n1, g.n2, g.n3, TZ, TX);
}

Step3Launch stepB3_tma_shape(const Grid &g, int num_sms, int L) {
    using namespace s3;
    Step3Launch s{};
    s.L = L > 0 ? L : 64;
    s.ntz = (g.n1 + TZ - 1) / TZ;
    s.ntx = (g.n2 + TX - 1) / TX;
    s.nchunks = (g.n3 + s.L - 1) / s.L;
    s.items = s.ntz * s.ntx * s.nchunks;
    s.grid = std::min(s.items, 2 * num_sms);
    s.smem = RING * sizeof(Stage) + TRING * sizeof(Tile) + (size_t)g.n3 * sizeof(float) + 128;
    return s;
}

// launch one step: cur = u[icur], nxt = u[1-icur]
cudaError_t launch_stepB3_tma(bool exact, const CUtensorMap *maps, int icur, float *nxt, const StepBParams &sp,
                              const Step3Launch &sh, unsigned long long *counter, unsigned long long base, int *err,
                              cudaStream_t s) {
    return launch_stepB3_tma_with(exact, maps[icur], maps[2 + (1 - icur)], maps[4], nxt, sp, sh, counter, base, err,
                                  s, nullptr);
}

static Step3Params step3_params(const StepBParams &sp, const Step3Launch &sh, unsigned long long *counter,
                                unsigned long long base, int *err, float *nxt) {
    Step3Params p{};
    p.n1 = sp.g.n1;
    p.n2 = sp.g.n2;
    p.n3 = sp.g.n3;
    p.c0 = sp.k.c0;
    for (int k = 0; k <= 4; k++) {
        p.cz[k] = sp.k.c[0][k];
        p.cx[k] = sp.k.c[1][k];
        p.cy[k] = sp.k.c[2][k];
    }
    p.w1 = sp.w1;
    p.w2 = sp.w2;
    p.w3 = sp.w3;
    p.damp_prev = sp.damp_prev;
    p.sponge_new = sp.sponge_new;
    p.shell = sp.shell;
    for (int a = 0; a < 3; a++) {
        p.ilo[a] = sp.ilo[a];
        p.ihi[a] = sp.ihi[a];
    }
    p.L = sh.L;
    p.ntz = sh.ntz;
    p.ntx = sh.ntx;
    p.nchunks = sh.nchunks;
    p.counter = counter;
    p.base = base;
    p.err = err;
    p.nxt = nxt;
    p.spin = sp.spin >= 0 ? sp.spin : s3::SPIN_LIMIT;
    return p;
}

// adjoint step (AWE_FAST): g_halo = halo-box map of I vel2 nu_k, y_tile = tile
// map of nu_{k+1} (Y, overwritten by mu_k), x_tile = tile map of nu_k
cudaError_t launch_stepB3_adj(const CUtensorMap &g_halo, const CUtensorMap &y_tile, const CUtensorMap &x_tile,
                              float *Y, const float *lap_v, float2 *grad, const StepBParams &sp,
                              const Step3Launch &sh, unsigned long long *counter, unsigned long long base, int *err,
                              cudaStream_t s) {
    Step3Params p = step3_params(sp, sh, counter, base, err, Y);
    p.lap_v = lap_v;
    p.grad = grad;
    cudaFuncSetAttribute(k_stepB3_o8<false, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem);
    k_stepB3_o8<false, 2><<<sh.grid, s3::NTHREADS, sh.smem, s>>>(g_halo, y_tile, x_tile, p);
    return cudaGetLastError();
}

// one step with explicit maps: cur halo-box map, prv tile-box map (the buffer
// the new level replaces, or another one when stepping out of place), vel
cudaError_t launch_stepB3_tma_with(bool exact, const CUtensorMap &cur, const CUtensorMap &prv, const CUtensorMap &vel,
                                   float *nxt, const StepBParams &sp, const Step3Launch &sh,
                                   unsigned long long *counter, unsigned long long base, int *err, cudaStream_t s,
                                   float *lap_out) {
    Step3Params p{};
    p.n1 = sp.g.n1;
    p.n2 = sp.g.n2;
    p.n3 = sp.g.n3;
    p.c0 = sp.k.c0;
    for (int k = 0; k <= 4; k++) {
        p.cz[k] = sp.k.c[0][k];
        p.cx[k] = sp.k.c[1][k];
        p.cy[k] = sp.k.c[2][k];
    }
    p.w1 = sp.w1;
    p.w2 = sp.w2;
    p.w3 = sp.w3;
    p.damp_prev = sp.damp_prev;
    p.sponge_new = sp.sponge_new;
    p.shell = sp.shell;
    for (int a = 0; a < 3; a++) {
        p.ilo[a] = sp.ilo[a];
        p.ihi[a] = sp.ihi[a];
    }
    p.L = sh.L;
    p.ntz = sh.ntz;
    p.ntx = sh.ntx;
    p.nchunks = sh.nchunks;
    p.counter = counter;
    p.base = base;
    p.err = err;
    p.nxt = nxt;
    p.lap_out = lap_out;
    p.spin = sp.spin >= 0 ? sp.spin : s3::SPIN_LIMIT;
    if (exact) {
        cudaFuncSetAttribute(k_stepB3_o8<true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem);
        k_stepB3_o8<true, 0><<<sh.grid, s3::NTHREADS, sh.smem, s>>>(cur, prv, vel, p);
    } else if (lap_out) {
        cudaFuncSetAttribute(k_stepB3_o8<false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem);
        k_stepB3_o8<false, 1><<<sh.grid, s3::NTHREADS, sh.smem, s>>>(cur, prv, vel, p);
    } else {
        cudaFuncSetAttribute(k_stepB3_o8<false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem);
        k_stepB3_o8<false, 0><<<sh.grid, s3::NTHREADS, sh.smem, s>>>(cur, prv, vel, p);
    }
    return cudaGetLastError();
}

}  // namespace awe
