// Batched 2D forward, column march (8th order): the same step as k_batch2d
// (V_{k+1} = W (N + S) of the CPU-program scheme on every shot's window),
// laid out for HBM streaming.
//
// A work item is one shot and a chunk of L consecutive columns (x).  A CTA
// of n1/4 threads (four z cells each) marches along x: for every column it
// needs, one thread issues 1D bulk copies (cp.async.bulk, mbarrier
// completion) of the current level's column and, for output columns, of the
// previous level's and v^2 dt^2's columns into a ring of CRING shared-memory
// slots, CRING - 4 columns ahead of the one being computed.  The x
// neighbours of a cell come from a 9-column register queue, the z
// neighbours from the centre column in shared memory (zero-padded ends).
// Each plane is copied once per item (the chunk's 8 halo columns are read
// twice), so DRAM traffic is about (1 + 8/L) x 4 + 12 bytes per cell.
// Receiver items gather from the current level as in k_batch2d.
//
// Every mbarrier wait is bounded; a CTA that gives up sets *err, waits
// (bounded) for its copies in flight and returns.
#include <cuda_runtime.h>

#include "awe_internal.h"
#include "gsum.cuh"
#include "tma.cuh"

namespace awe {
namespace {

constexpr int CNOP = 4, QL = 2 * CNOP + 1, CRING = 8;
constexpr long long CSPIN = 1ll << 22;
constexpr int kColMaxN1 = 2048;  // ring of 8 slots of 3 columns: 197 KB of shared memory at 2048

__host__ __device__ inline int col_pitch(int n1) { return n1 + 8; }           // cur column: 4 zeros each end
__host__ __device__ inline int col_slot(int n1) { return col_pitch(n1) + 2 * n1; }  // + prv + vel columns

// Rarely taken parts of the column loops, kept out of line so the nine
// unrolled copies of the loop body stay small.

// forward: the shot's source terms on a 4-cell strip (cells cell0 .. cell0 + 3)
__device__ __noinline__ float4 col_sources_fwd(float4 o, float4 v4, const GeoPoint *src, int ns, float dd, int n1,
                                               long long cell0) {
    float r[4] = {o.x, o.y, o.z, o.w};
    const float v[4] = {v4.x, v4.y, v4.z, v4.w};
    for (int sidx = 0; sidx < ns; sidx++) {
        const GeoPoint gp = src[sidx];
#pragma unroll
        for (int cc = 0; cc < 4; cc++) {
            const long long d = gp.base + (cc & 1) + (cc >> 1) * (long long)n1 - cell0;
#pragma unroll
            for (int i = 0; i < 4; i++)
                if (d == i) r[i] = r[i] + (dd * gp.w[cc]) * v[i];
        }
    }
    return make_float4(r[0], r[1], r[2], r[3]);
}

// adjoint: the shot's source terms of the gradient on a 2-cell strip
__device__ __noinline__ float4 col_sources_adj(float4 ga, float2 nu, const GeoPoint *src, int ns, float dd, int n1,
                                               long long cell0) {
    float2 g[2] = {make_float2(ga.x, ga.y), make_float2(ga.z, ga.w)};
    const float v[2] = {nu.x, nu.y};
    for (int sidx = 0; sidx < ns; sidx++) {
        const GeoPoint gp = src[sidx];
#pragma unroll
        for (int cc = 0; cc < 4; cc++) {
            const long long d = gp.base + (cc & 1) + (cc >> 1) * (long long)n1 - cell0;
#pragma unroll
            for (int i = 0; i < 2; i++)
                if (d == i) g[i] = gsum_add_prod(g[i], v[i], dd * gp.w[cc]);
        }
    }
    return make_float4(g[0].x, g[0].y, g[1].x, g[1].y);
}

// tid 0 after a timed-out wait: waits (bounded) for every copy still in
// flight of the item (columns s .. issued - 1)
__device__ __noinline__ void col_drain(uint64_t *full, int ring, int slot0, uint32_t ph0, int s, int issued) {
    for (int t = s; t < issued; t++) {
        const int tt = slot0 + t;
        mbar_wait(&full[tt % ring], ph0 ^ (uint32_t)((tt / ring) & 1), CSPIN);
    }
}

__global__ void __launch_bounds__(512) k_batch2d_col(const BatchShot *__restrict__ shots,
                                                      const int4 *__restrict__ items, int nitems, const BatchStep p,
                                                      int L, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int n1 = p.n1;
    const int CP = col_pitch(n1), SLOT = col_slot(n1);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw);
    float *ring = reinterpret_cast<float *>(smem_raw + 128);
    const int tid = threadIdx.x;
    const int zb = 4 * tid;
    const bool active = zb < n1;
    if (tid == 0) {
        for (int i = 0; i < CRING; i++) mbar_init(&full[i], 1);
        fence_mbar_init();
    }
    for (int i = tid; i < CRING * 8; i += blockDim.x) {  // zero ends of every cur column
        const int sl = i / 8, k = i % 8;
        ring[sl * SLOT + (k < 4 ? k : CP - 8 + k)] = 0.f;
    }
    __syncthreads();
    const float *prvb = p.prv ? p.prv : p.nxt;
    float wz[4];
    bool zin[4];
    bool zone = true;  // this thread's four z factors are all 1 (the multiplies are identities)
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int z = zb + i;
        wz[i] = (p.sponge && z < n1) ? __ldg(p.wz + z) : 1.f;
        zin[i] = z >= CNOP && z < n1 - CNOP;
        zone = zone && wz[i] == 1.f;
    }
    int slot0 = 0;
    uint32_t ph0 = 0;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const int4 it = items[w];
        const BatchShot sh = shots[it.x];
        if (it.w != 0) {  // receiver item: it.y = first receiver of the block
            if (p.row < 0) continue;
            const float *c = p.cur + sh.off;
            const int rend = min(it.y + kBatchRecBlock, sh.nr);
            for (int r = it.y + tid; r < rend; r += blockDim.x) {
                const GeoPoint gp = p.rec[sh.rec0 + r];
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
            continue;
        }
        // ---- column item: it.z = first output column
        const int x0 = it.z, x1 = min(x0 + L, sh.n2);
        const int S = (x1 - x0) + 2 * CNOP;
        const float *cbase = p.cur + sh.off;
        const uint32_t cb = (uint32_t)n1 * 4u;
        // columns of the shot's first sources (a source's corners lie within
        // two columns of its base index); more than 4 sources: every column is checked
        int scol[4] = {-2, -2, -2, -2};
        const bool few = sh.ns <= 4;
        for (int k = 0; k < sh.ns && k < 4; k++) scol[k] = (int)(p.src[sh.src0 + k].base / n1);
        auto issue = [&](int s) {
            const int sx = (slot0 + s) % CRING;
            float *sl = ring + sx * SLOT;
            const int xc = x0 - CNOP + s;
            const bool cin = xc >= 0 && xc < sh.n2;
            const bool out = s >= 2 * CNOP;
            mbar_expect_tx(&full[sx], (cin ? cb : 0u) + (out ? 2u * cb : 0u));
            if (cin) bulk_load_1d(sl + 4, cbase + (long long)xc * n1, cb, &full[sx]);
            if (out) {
                const long long go = sh.off + (long long)(x0 + s - 2 * CNOP) * n1;
                bulk_load_1d(sl + CP, prvb + go, cb, &full[sx]);
                bulk_load_1d(sl + CP + n1, p.vel + go, cb, &full[sx]);
            }
        };
        if (tid == 0)
            for (int s = 0; s < CRING && s < S; s++) issue(s);

        int slot = slot0;
        uint32_t ph = ph0;
        float q[QL][4];
#pragma unroll 1
        for (int blk = 0; blk < S; blk += QL) {
#pragma unroll
            for (int u = 0; u < QL; u++) {
                const int s = blk + u;
                if (s < S) {
                    const bool bad = !mbar_wait(&full[slot], ph, CSPIN);
                    if (bad) atomicExch(err, 1);
                    const float *sl = ring + slot * SLOT;
                    const int xc = x0 - CNOP + s;
                    if (active) {
                        float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (xc >= 0 && xc < sh.n2) c = *reinterpret_cast<const float4 *>(sl + 4 + zb);
                        q[u][0] = c.x;
                        q[u][1] = c.y;
                        q[u][2] = c.z;
                        q[u][3] = c.w;
                    }
                    if (s >= 2 * CNOP && active) {
                        const int x = x0 + s - 2 * CNOP;
                        const int hs = (slot + CRING - CNOP) % CRING;  // slot of the centre column
                        const float *H = ring + hs * SLOT;             // padded: H[4 + z] = column[z]
                        float zw[12];
#pragma unroll
                        for (int v = 0; v < 3; v++) {
                            const float4 t = *reinterpret_cast<const float4 *>(H + zb + 4 * v);
                            zw[4 * v] = t.x;
                            zw[4 * v + 1] = t.y;
                            zw[4 * v + 2] = t.z;
                            zw[4 * v + 3] = t.w;
                        }
                        const int jc = (u + 1 + CNOP) % QL;  // queue slot of the centre column
                        float2 l01 = __fmul2_rn(make_float2(zw[4], zw[5]), make_float2(p.c0, p.c0));
                        float2 l23 = __fmul2_rn(make_float2(zw[6], zw[7]), make_float2(p.c0, p.c0));
#pragma unroll
                        for (int k = 1; k <= CNOP; k++) {
                            const float2 z01 = make_float2(zw[4 - k] + zw[4 + k], zw[5 - k] + zw[5 + k]);
                            const float2 z23 = make_float2(zw[6 - k] + zw[6 + k], zw[7 - k] + zw[7 + k]);
                            const float *qa = q[(jc + QL - k) % QL], *qb = q[(jc + k) % QL];
                            const float2 x01 = __fadd2_rn(make_float2(qa[0], qa[1]), make_float2(qb[0], qb[1]));
                            const float2 x23 = __fadd2_rn(make_float2(qa[2], qa[3]), make_float2(qb[2], qb[3]));
                            const float2 cz = make_float2(p.cz[k], p.cz[k]), cx = make_float2(p.cx[k], p.cx[k]);
                            l01 = __ffma2_rn(z01, cz, l01);
                            l23 = __ffma2_rn(z23, cz, l23);
                            l01 = __ffma2_rn(x01, cx, l01);
                            l23 = __ffma2_rn(x23, cx, l23);
                        }
                        const float lap[4] = {l01.x, l01.y, l23.x, l23.y};
                        const float4 pv = *reinterpret_cast<const float4 *>(sl + CP + zb);
                        const float4 vv = *reinterpret_cast<const float4 *>(sl + CP + n1 + zb);
                        const float pr4[4] = {pv.x, pv.y, pv.z, pv.w}, v4[4] = {vv.x, vv.y, vv.z, vv.w};
                        const float wx = p.sponge ? __ldg(p.wx + sh.wx_off + x) : 1.f;
                        const bool damp = p.sponge && !(zone && wx == 1.f);  // else multiplies by 1 skipped
                        const bool xin = x >= CNOP && x < sh.n2 - CNOP;
                        float o[4];
#pragma unroll
                        for (int i = 0; i < 4; i++) {
                            float pr = pr4[i];
                            if (damp) pr = (pr * wz[i]) * wx;
                            float out = pr;
                            if (xin && zin[i]) out = fmaf(v4[i], lap[i], 2.f * zw[4 + i] - pr);
                            o[i] = out;
                        }
                        bool near = !few;
#pragma unroll
                        for (int k = 0; k < 4; k++) near = near || (unsigned)(x - scol[k]) <= 2u;
                        if (sh.ns > 0 && near) {  // source corners of this shot in this 4-cell strip
                            const float4 r = col_sources_fwd(make_float4(o[0], o[1], o[2], o[3]), vv,
                                                             p.src + sh.src0, sh.ns, p.wav[p.it], n1,
                                                             (long long)x * n1 + zb);
                            o[0] = r.x, o[1] = r.y, o[2] = r.z, o[3] = r.w;
                        }
                        if (damp) {
#pragma unroll
                            for (int i = 0; i < 4; i++) o[i] = (o[i] * wz[i]) * wx;
                        }
                        *reinterpret_cast<float4 *>(p.nxt + sh.off + (long long)x * n1 + zb) =
                            make_float4(o[0], o[1], o[2], o[3]);
                    }
                    if (__syncthreads_or(bad)) {
                        // drain: wait (bounded) for every copy still in flight, then leave
                        if (tid == 0) col_drain(full, CRING, slot0, ph0, s, min(S, max(CRING, s - CNOP + CRING)));
                        __syncthreads();
                        return;
                    }
                    if (tid == 0 && s >= CNOP && s - CNOP + CRING < S) issue(s - CNOP + CRING);
                    if (++slot == CRING) {
                        slot = 0;
                        ph ^= 1u;
                    }
                }
            }
        }
        const int t = slot0 + S;
        ph0 ^= (uint32_t)((t / CRING) & 1);
        slot0 = t % CRING;
    }
}

// ---------------------------------------------------------------------------
// Adjoint step of the batch as a column march (the arithmetic of
// k_batch2d_adj in the same order).  Two z cells per thread (twice the warps
// of the forward's four-cell layout, half the queue registers).  Per plane
// (column xc): X = nu_k, v^2dt^2 and V_k columns by bulk copy; the thread
// forms g = I vel2 nu for its cells and writes it to the slot's g column
// (zero-padded) for the z window, and keeps g and V in 9-column register
// queues for the x neighbours.  For the output column (the centre) the
// thread's nu_{k+1} (Y) and gradient-accumulator strips are loaded before the ring
// wait; mu_k = W lambda goes back to Y and the gradient strip is updated and
// stored (the receiver term follows in k_batch_rec_adj); sources are tested
// only near their columns.
constexpr int ARING = 8;
constexpr int kAdjMaxN1 = 1024;  // 512 threads of two cells
constexpr int YG_AHEAD = 3;      // output columns whose nu_{k+1} / gradient strips are in flight
constexpr int YG_DEPTH = YG_AHEAD + 1;

__host__ __device__ inline int adj_slot(int n1) { return 2 * n1 + 2 * (n1 + 8); }
// slot layout (floats): X [n1] | vel [n1] | V [4 | n1 | 4] | g [4 | n1 | 4]; after the
// ring, YG_DEPTH slots of the output columns' gradient accumulators [n1] and nu_{k+1} [n1]
__host__ __device__ inline int adj_off_v(int n1) { return 2 * n1; }
__host__ __device__ inline int adj_off_g(int n1) { return 2 * n1 + (n1 + 8); }

__global__ void __maxnreg__(96) k_batch2d_col_adj(const BatchShot *__restrict__ shots,
                                                         const int4 *__restrict__ items, int nitems,
                                                         const BatchAdj p, int L, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int n1 = p.n1;
    const int SLOT = adj_slot(n1), OV = adj_off_v(n1), OG = adj_off_g(n1);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw);
    float *ring = reinterpret_cast<float *>(smem_raw + 128);
    float2 *gring = reinterpret_cast<float2 *>(ring + ARING * SLOT);
    float *yring = reinterpret_cast<float *>(gring + YG_DEPTH * n1);
    const int tid = threadIdx.x;
    const int zb = 2 * tid;
    const bool active = zb < n1;
    if (tid == 0) {
        for (int i = 0; i < ARING; i++) mbar_init(&full[i], 1);
        fence_mbar_init();
    }
    for (int i = tid; i < ARING * 16; i += blockDim.x) {  // zero ends of every V and g column
        const int sl = i / 16, k = i % 16, base = (k < 8) ? OV : OG, kk = k % 8;
        ring[sl * SLOT + base + (kk < 4 ? kk : n1 + kk)] = 0.f;
    }
    __syncthreads();
    bool zin[2];
    float wz[2];
#pragma unroll
    for (int i = 0; i < 2; i++) {
        zin[i] = zb + i >= CNOP && zb + i < n1 - CNOP;
        wz[i] = (p.sponge && zb + i < n1) ? __ldg(p.wz + zb + i) : 1.f;
    }
    int slot0 = 0;
    uint32_t ph0 = 0;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const int4 it = items[w];
        if (it.w != 0) continue;  // receiver items belong to the forward
        const BatchShot sh = shots[it.x];
        const int x0 = it.z, x1 = min(x0 + L, sh.n2);
        const int S = (x1 - x0) + 2 * CNOP;
        const uint32_t cb = (uint32_t)n1 * 4u;
        auto issue = [&](int s) {
            const int sx = (slot0 + s) % ARING;
            float *sl = ring + sx * SLOT;
            const int xc = x0 - CNOP + s;
            const bool cin = xc >= 0 && xc < sh.n2;
            mbar_expect_tx(&full[sx], cin ? 3u * cb : 0u);
            if (cin) {
                const long long gc = sh.off + (long long)xc * n1;
                bulk_load_1d(sl, p.X + gc, cb, &full[sx]);
                bulk_load_1d(sl + n1, p.vel + gc, cb, &full[sx]);
                bulk_load_1d(sl + OV + 4, p.V + gc, cb, &full[sx]);
            }
        };
        if (tid == 0)
            for (int s = 0; s < ARING && s < S; s++) issue(s);
        int scol[4] = {-8, -8, -8, -8};
        const bool few = sh.ns <= 4;
        for (int k = 0; k < sh.ns && k < 4; k++) scol[k] = (int)(p.src[sh.src0 + k].base / n1);
        // this thread's strips of output column t (t >= 2 CNOP), one commit group per column
        auto issue_yg = [&](int t) {
            if (active && t >= 2 * CNOP && t < S) {
                const long long gi = sh.off + (long long)(x0 + t - 2 * CNOP) * n1 + zb;
                const int q = (t % YG_DEPTH) * n1 + zb;
                cp_async_16(gring + q, p.G + gi);
                cp_async_8(yring + q, p.Y + gi);
            }
            cp_async_commit();
        };
        for (int t = 0; t < YG_AHEAD; t++) issue_yg(t);

        int slot = slot0;
        uint32_t ph = ph0;
        float gq[QL][2], vq[QL][2];
#pragma unroll 1
        for (int blk = 0; blk < S; blk += QL) {
#pragma unroll
            for (int u = 0; u < QL; u++) {
                const int s = blk + u;
                if (s < S) {
                    const bool outp = s >= 2 * CNOP && active;
                    const int x = x0 + s - 2 * CNOP;
                    const long long gi = sh.off + (long long)x * n1 + zb;
                    const float wx = (p.sponge && outp) ? __ldg(p.wx + sh.wx_off + x) : 1.f;
                    issue_yg(s + YG_AHEAD);
                    cp_async_wait<YG_AHEAD>();  // column s's strips are in (own copies only)
                    const bool bad = !mbar_wait(&full[slot], ph, CSPIN);
                    if (bad) atomicExch(err, 1);
                    float *sl = ring + slot * SLOT;
                    const int xc = x0 - CNOP + s;
                    if (active) {
                        float2 gv = make_float2(0.f, 0.f), vv = gv;
                        if (xc >= 0 && xc < sh.n2) {
                            const float2 xv = *reinterpret_cast<const float2 *>(sl + zb);
                            const float2 wv = *reinterpret_cast<const float2 *>(sl + n1 + zb);
                            vv = *reinterpret_cast<const float2 *>(sl + OV + 4 + zb);
                            const bool xin = xc >= CNOP && xc < sh.n2 - CNOP;
                            gv.x = (xin && zin[0]) ? wv.x * xv.x : 0.f;
                            gv.y = (xin && zin[1]) ? wv.y * xv.y : 0.f;
                        }
                        // this column's g, for its z window when it is the centre (after barriers)
                        *reinterpret_cast<float2 *>(sl + OG + 4 + zb) = gv;
                        gq[u][0] = gv.x, gq[u][1] = gv.y;
                        vq[u][0] = vv.x, vq[u][1] = vv.y;
                    }
                    if (outp) {
                        const float *H = ring + ((slot + ARING - CNOP) % ARING) * SLOT;  // centre column's slot
                        float gz[10], vz[10];  // z = zb - 4 .. zb + 5
#pragma unroll
                        for (int v = 0; v < 5; v++) {
                            const float2 a = *reinterpret_cast<const float2 *>(H + OG + zb + 2 * v);
                            const float2 c = *reinterpret_cast<const float2 *>(H + OV + zb + 2 * v);
                            gz[2 * v] = a.x, gz[2 * v + 1] = a.y;
                            vz[2 * v] = c.x, vz[2 * v + 1] = c.y;
                        }
                        const int jc = (u + 1 + CNOP) % QL;
                        const float2 c0 = make_float2(p.c0, p.c0);
                        float2 g01 = __fmul2_rn(make_float2(gz[4], gz[5]), c0);
                        float2 v01 = __fmul2_rn(make_float2(vz[4], vz[5]), c0);
#pragma unroll
                        for (int k = 1; k <= CNOP; k++) {
                            const float2 cz = make_float2(p.cz[k], p.cz[k]), cx = make_float2(p.cx[k], p.cx[k]);
                            const float *ga = gq[(jc + QL - k) % QL], *gb = gq[(jc + k) % QL];
                            const float *va = vq[(jc + QL - k) % QL], *vb = vq[(jc + k) % QL];
                            const float2 gs = (k % 2 == 0)
                                                  ? __fadd2_rn(make_float2(gz[4 - k], gz[5 - k]), make_float2(gz[4 + k], gz[5 + k]))
                                                  : make_float2(gz[4 - k] + gz[4 + k], gz[5 - k] + gz[5 + k]);
                            const float2 vs = (k % 2 == 0)
                                                  ? __fadd2_rn(make_float2(vz[4 - k], vz[5 - k]), make_float2(vz[4 + k], vz[5 + k]))
                                                  : make_float2(vz[4 - k] + vz[4 + k], vz[5 - k] + vz[5 + k]);
                            g01 = __ffma2_rn(gs, cz, g01);
                            g01 = __ffma2_rn(__fadd2_rn(make_float2(ga[0], ga[1]), make_float2(gb[0], gb[1])), cx, g01);
                            v01 = __ffma2_rn(vs, cz, v01);
                            v01 = __ffma2_rn(__fadd2_rn(make_float2(va[0], va[1]), make_float2(vb[0], vb[1])), cx, v01);
                        }
                        const float lt[2] = {g01.x, g01.y}, lv[2] = {v01.x, v01.y};
                        const float2 nv2 = *reinterpret_cast<const float2 *>(H + zb);  // nu_k of the centre
                        const int q = (s % YG_DEPTH) * n1 + zb;
                        const float2 yv2 = *reinterpret_cast<const float2 *>(yring + q);
                        const float4 G01 = *reinterpret_cast<const float4 *>(gring + q);
                        const float nu[2] = {nv2.x, nv2.y}, yv[2] = {yv2.x, yv2.y};
                        const bool xin = x >= CNOP && x < sh.n2 - CNOP;
                        float mu[2], wc[2];
                        float2 ga[2] = {make_float2(G01.x, G01.y), make_float2(G01.z, G01.w)};
#pragma unroll
                        for (int i = 0; i < 2; i++) {
                            const bool in = xin && zin[i];
                            wc[i] = p.sponge ? wz[i] * wx : 1.f;
                            const float lam = (in ? 2.f * nu[i] : 0.f) + lt[i] + (in ? -wc[i] : wc[i]) * yv[i];
                            mu[i] = wc[i] * lam;
                            if (in) ga[i] = gsum_add(ga[i], __fmul_rn(nu[i], lv[i]));  // FP32 product, compensated sum
                        }
                        bool near = !few;
#pragma unroll
                        for (int k = 0; k < 4; k++) near = near || (unsigned)(x - scol[k]) <= 2u;
                        if (sh.ns > 0 && near) {  // source term of the gradient
                            const float4 r = col_sources_adj(make_float4(ga[0].x, ga[0].y, ga[1].x, ga[1].y), nv2,
                                                             p.src + sh.src0, sh.ns, p.wav[p.it], n1,
                                                             (long long)x * n1 + zb);
                            ga[0] = make_float2(r.x, r.y);
                            ga[1] = make_float2(r.z, r.w);
                        }
                        *reinterpret_cast<float2 *>(p.Y + gi) = make_float2(mu[0], mu[1]);
                        __stcs(reinterpret_cast<float4 *>(p.G + gi), make_float4(ga[0].x, ga[0].y, ga[1].x, ga[1].y));
                    }
                    if (__syncthreads_or(bad)) {
                        cp_async_wait<0>();
                        if (tid == 0) col_drain(full, ARING, slot0, ph0, s, min(S, max(ARING, s - CNOP + ARING)));
                        __syncthreads();
                        return;
                    }
                    if (tid == 0 && s >= CNOP && s - CNOP + ARING < S) issue(s - CNOP + ARING);
                    if (++slot == ARING) {
                        slot = 0;
                        ph ^= 1u;
                    }
                }
            }
        }
        const int t = slot0 + S;
        ph0 ^= (uint32_t)((t / ARING) & 1);
        slot0 = t % ARING;
    }
}

}  // namespace

size_t batch2d_col_adj_smem(int n1) {
    return 128 + (size_t)ARING * adj_slot(n1) * sizeof(float) + (size_t)YG_DEPTH * n1 * (sizeof(float2) + sizeof(float));
}

static int adj_threads(int n1) { return ((n1 / 2 + 31) / 32) * 32; }

int batch2d_col_adj_ctas_per_sm(int n1) {
    if (!batch2d_col_shape(CNOP, n1, nullptr) || n1 > kAdjMaxN1) return 0;
    const size_t smem = batch2d_col_adj_smem(n1);
    if (cudaFuncSetAttribute(k_batch2d_col_adj, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch2d_col_adj, adj_threads(n1), smem) != cudaSuccess)
        return 0;
    return nb;
}

void launch_batch2d_col_adj(const BatchShot *shots, const int4 *items, int nitems, int grid, int L,
                            const BatchAdj &p, int *err,
                            cudaStream_t s) {
    if (p.n1 > kAdjMaxN1 || grid < 1) return;
    k_batch2d_col_adj<<<grid, adj_threads(p.n1), batch2d_col_adj_smem(p.n1), s>>>(shots, items, nitems, p, L, err);
}

int batch2d_col_shape(int nop, int n1, size_t *smem) {
    if (nop != CNOP || n1 % 4 != 0 || n1 < 16 || n1 > kColMaxN1) return 0;
    if (smem) *smem = 128 + (size_t)CRING * col_slot(n1) * sizeof(float);
    return ((n1 / 4 + 31) / 32) * 32;
}

int batch2d_col_ctas_per_sm(int n1) {
    size_t smem = 0;
    const int threads = batch2d_col_shape(CNOP, n1, &smem);
    if (!threads) return 0;
    if (cudaFuncSetAttribute(k_batch2d_col, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch2d_col, threads, smem) != cudaSuccess) return 0;
    return nb;
}

void launch_batch2d_col(const BatchShot *shots, const int4 *items, int nitems, int grid, int L, const BatchStep &p,
                        int *err, cudaStream_t s) {
    size_t smem = 0;
    const int threads = batch2d_col_shape(CNOP, p.n1, &smem);
    if (!threads || grid < 1) return;
    k_batch2d_col<<<grid, threads, smem, s>>>(shots, items, nitems, p, L, err);
}

}  // namespace awe
