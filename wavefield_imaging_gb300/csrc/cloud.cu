// Point-cloud windowing and merging: the ground-point selection that cuts an
// orbital survey into windows (CODE/Mbycloudwin3d.c) and the fold-normalised
// sum of the windows' data back onto the full cloud (CODE/Mbycloudmerge3d.c
// with the coordinate hash of CODE/hash.c).
//
// Window: one thread per ground point tests the orbit points, staged 256 at a
// time in shared memory, against the point's aperture cone (isInCone,
// Mbycloudwin3d.c:19-35, in the same float operations with IEEE
// round-to-nearest intrinsics so the flags match the C code bit for bit);
// a two-level exclusive scan of the flags gives every kept point its place
// in input order (the reference's gwmap), and two gathers move the points
// and the data columns [nf][ng] -> [nf][nw].
//
// Merge: the hash table of the full cloud is built on the host in the
// reference's insertion order (open addressing from an FNV-1a hash of the
// distance to the centroid), so every lookup probes the same slots as
// htLookup; the lookups of all window points run on the GPU, and the window
// data are added window after window (the reference's summation order per
// output sample), then divided by the fold.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "awe_internal.h"

namespace awe {
namespace {

constexpr int kNco = AWE_CLOUD_NCO;
constexpr int kOrbitTile = 256;
constexpr int kChunk = 1024;  // flags per scan block (256 threads x 4)

__device__ __forceinline__ bool in_cone(float ox, float oy, float oz, float gx, float gy, float gz, float nx,
                                        float ny, float nz, float cosapt) {
    float rx = __fsub_rn(ox, gx), ry = __fsub_rn(oy, gy), rz = __fsub_rn(oz, gz);
    const float r = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(rx, rx), __fmul_rn(ry, ry)), __fmul_rn(rz, rz)));
    rx = __fdiv_rn(rx, r);
    ry = __fdiv_rn(ry, r);
    rz = __fdiv_rn(rz, r);
    const float c = __fadd_rn(__fadd_rn(__fmul_rn(rx, nx), __fmul_rn(ry, ny)), __fmul_rn(rz, nz));
    return fabsf(c) > cosapt;
}

__global__ void __launch_bounds__(256) k_cloud_flag(const float *__restrict__ g, long long ng,
                                                    const float *__restrict__ orb, long long no, float cosapt,
                                                    unsigned char *__restrict__ flag) {
    __shared__ float so[3][kOrbitTile];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float gx = 0.f, gy = 0.f, gz = 0.f, nx = 0.f, ny = 0.f, nz = 0.f;
    if (i < ng) {
        const float *p = g + i * kNco;
        gx = p[0], gy = p[1], gz = p[2], nx = p[3], ny = p[4], nz = p[5];
    }
    bool hit = false;
    for (long long o0 = 0; o0 < no; o0 += kOrbitTile) {
        const long long j = o0 + threadIdx.x;
        if (j < no) {
            so[0][threadIdx.x] = orb[j * kNco];
            so[1][threadIdx.x] = orb[j * kNco + 1];
            so[2][threadIdx.x] = orb[j * kNco + 2];
        }
        __syncthreads();
        const int m = (int)(no - o0 < kOrbitTile ? no - o0 : kOrbitTile);
        if (i < ng && !hit)
            for (int k = 0; k < m; k++)
                if (in_cone(so[0][k], so[1][k], so[2][k], gx, gy, gz, nx, ny, nz, cosapt)) {
                    hit = true;
                    break;
                }
        __syncthreads();
    }
    if (i < ng) flag[i] = hit ? 1 : 0;
}

// flags kept per chunk of kChunk points
__global__ void __launch_bounds__(256) k_chunk_count(const unsigned char *__restrict__ flag, long long n,
                                                     long long *__restrict__ counts) {
    const long long base = (long long)blockIdx.x * kChunk + 4 * threadIdx.x;
    int c = 0;
    for (int k = 0; k < 4; k++)
        if (base + k < n) c += flag[base + k];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __shared__ int part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long s = 0;
        for (int w = 0; w < 8; w++) s += part[w];
        counts[blockIdx.x] = s;
    }
}

// exclusive scan of the chunk counts in place (one block); total at counts[nb]
__global__ void __launch_bounds__(1024) k_scan_counts(long long *counts, long long nb) {
    __shared__ long long buf[1024];
    long long carry = 0;
    for (long long b0 = 0; b0 < nb; b0 += 1024) {
        const long long j = b0 + threadIdx.x;
        const long long v = j < nb ? counts[j] : 0;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {  // Hillis-Steele inclusive scan
            const long long t = threadIdx.x >= (unsigned)off ? buf[threadIdx.x - off] : 0;
            __syncthreads();
            buf[threadIdx.x] += t;
            __syncthreads();
        }
        if (j < nb) counts[j] = carry + buf[threadIdx.x] - v;
        const long long total = buf[1023];
        __syncthreads();
        carry += total;
    }
    if (threadIdx.x == 0) counts[nb] = carry;
}

// positions of the kept points, in input order
__global__ void __launch_bounds__(256) k_chunk_compact(const unsigned char *__restrict__ flag, long long n,
                                                       const long long *__restrict__ offsets,
                                                       long long *__restrict__ index) {
    __shared__ int scan[256];
    const long long base = (long long)blockIdx.x * kChunk + 4 * threadIdx.x;
    unsigned char f[4];
    int c = 0;
    for (int k = 0; k < 4; k++) {
        f[k] = base + k < n ? flag[base + k] : 0;
        c += f[k];
    }
    scan[threadIdx.x] = c;
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {
        const int t = threadIdx.x >= (unsigned)off ? scan[threadIdx.x - off] : 0;
        __syncthreads();
        scan[threadIdx.x] += t;
        __syncthreads();
    }
    long long pos = offsets[blockIdx.x] + scan[threadIdx.x] - c;
    for (int k = 0; k < 4; k++)
        if (f[k]) index[pos++] = base + k;
}

__global__ void k_gather_points(const float *__restrict__ g, const long long *__restrict__ index, long long nw,
                                float *__restrict__ out) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nw * kNco;
         t += (long long)gridDim.x * blockDim.x)
        out[t] = g[index[t / kNco] * kNco + t % kNco];
}

// data [nf][ng] (ncomp floats per sample) -> [nf][nw]
__global__ void k_gather_columns(const float *__restrict__ d, long long ng, const long long *__restrict__ index,
                                 long long nw, long long nf, int ncomp, float *__restrict__ out) {
    const long long row = nw * ncomp;
    for (long long jf = blockIdx.y; jf < nf; jf += gridDim.y)
        for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < row;
             t += (long long)gridDim.x * blockDim.x) {
            const long long iw = t / ncomp;
            out[jf * row + t] = d[(jf * ng + index[iw]) * ncomp + t % ncomp];
        }
}

// ---- merge ----

// distance as hash.c evaluates it: float differences, squares and sum in
// double (pow(x, 2) is the correctly rounded square), sqrtf of the sum
// rounded to float, widened back to double
__host__ __device__ inline double cloud_dist(float ax, float ay, float az, float bx, float by, float bz) {
#ifdef __CUDA_ARCH__  // no contraction, IEEE rounding throughout
    const double dx = (double)__fsub_rn(ax, bx), dy = (double)__fsub_rn(ay, by), dz = (double)__fsub_rn(az, bz);
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return (double)__fsqrt_rn(__double2float_rn(s));
#else
    const double dx = (double)(ax - bx), dy = (double)(ay - by), dz = (double)(az - bz);
    const double s = dx * dx + dy * dy + dz * dz;
    return (double)sqrtf((float)s);
#endif
}

// FNV-1a over the 8 bytes of the distance to the reference point (hashF1a, hash.c:33-53)
__host__ __device__ inline unsigned long long cloud_hash(unsigned long long nhash, float px, float py, float pz,
                                                         float ox, float oy, float oz) {
    const double h = cloud_dist(px, py, pz, ox, oy, oz);
#ifdef __CUDA_ARCH__
    const unsigned long long bits = (unsigned long long)__double_as_longlong(h);
#else
    unsigned long long bits;
    memcpy(&bits, &h, sizeof bits);
#endif
    unsigned long long x = 14695981039346656037ull;
    for (int i = 0; i < 8; i++) {
        x ^= (bits >> (8 * i)) & 0xffull;
        x *= 1099511628211ull;
    }
    x *= 1099511628211ull;
    return x % nhash;
}

__global__ void k_cloud_lookup(const float *__restrict__ all, const long long *__restrict__ table,
                               unsigned long long nhash, float ox, float oy, float oz, double tol,
                               const float *__restrict__ q, long long nq, long long *__restrict__ idx,
                               int *__restrict__ missing) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nq) return;
    const float qx = q[t * kNco], qy = q[t * kNco + 1], qz = q[t * kNco + 2];
    const unsigned long long h = cloud_hash(nhash, qx, qy, qz, ox, oy, oz);
    long long found = -2;
    for (unsigned long long j = 0; j < nhash; j++) {  // htLookup: every occupied slot from h on, wrapping
        const unsigned long long s = (h + j) % nhash;
        const long long a = table[s];
        if (a < 0) continue;
        if (cloud_dist(all[a * kNco], all[a * kNco + 1], all[a * kNco + 2], qx, qy, qz) < tol) {
            found = a;
            break;
        }
    }
    idx[t] = found;
    if (found < 0) atomicExch(missing, 1);
}

// out[jf][idx[jw]] += win[jf][jw], one window (indices distinct within it)
__global__ void k_cloud_add(const float *__restrict__ win, long long nwc, const long long *__restrict__ idx,
                            long long na, long long nf, int ncomp, float *__restrict__ out) {
    const long long row = nwc * ncomp;
    for (long long jf = blockIdx.y; jf < nf; jf += gridDim.y)
        for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < row;
             t += (long long)gridDim.x * blockDim.x) {
            const long long jw = t / ncomp;
            float *o = out + (jf * na + idx[jw]) * ncomp + t % ncomp;
            *o = __fadd_rn(*o, win[jf * row + t]);
        }
}

__global__ void k_cloud_fold(const long long *__restrict__ idx, long long nwc, float *__restrict__ fold) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nwc) fold[idx[t]] = __fadd_rn(fold[idx[t]], 1.f);
}

// out /= max(fold, 1), each component of a complex sample by the real fold
__global__ void k_cloud_norm(float *__restrict__ out, const float *__restrict__ fold, long long na, long long nf,
                             int ncomp) {
    const long long n = na * nf * ncomp;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const float f = fmaxf(fold[(t / ncomp) % na], 1.f);
        out[t] = __fdiv_rn(out[t], f);
    }
}

// device buffers freed on every return path
struct DevBufs {
    std::vector<void *> p;
    ~DevBufs() {
        for (void *q : p) cudaFree(q);
    }
    template <class T>
    cudaError_t get(T **out, size_t bytes) {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, bytes ? bytes : 16);
        if (e == cudaSuccess) p.push_back(q);
        *out = (T *)q;
        return e;
    }
};

inline unsigned grid_for(long long n, int t = 256) {
    const long long b = (n + t - 1) / t;
    return (unsigned)std::max<long long>(1, std::min<long long>(b, 1 << 20));
}

}  // namespace
}  // namespace awe

using namespace awe;

#define CLOUD_TRY(expr, what)                                                       \
    do {                                                                            \
        cudaError_t e_ = (expr);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            set_error("%s: %s failed: %s", fn, what, cudaGetErrorString(e_));     \
            return e_ == cudaErrorMemoryAllocation ? AWE_ERR_NOMEM : AWE_ERR_CUDA; \
        }                                                                           \
    } while (0)

extern "C" {

awe_status awe_cloud_window(int device, const float *ground, long long ng, const float *orbit, long long no,
                            float apt, long long nf, int ncomp, const float *data, long long *nw, long long *index,
                            float *win, float *win_data) {
    const char *fn = "awe_cloud_window";
    if (!ground || !orbit || !nw || !index || ng < 0 || no < 0 || nf < 0 || (nf > 0 && (!data || !win_data)) ||
        (ncomp != 1 && ncomp != 2)) {
        set_error("%s: bad arguments (ground, orbit, nw and index needed; ncomp 1 or 2; data and win_data with nf > 0)",
                  fn);
        return AWE_ERR_INVALID;
    }
    *nw = 0;
    if (ng == 0) return AWE_OK;
    CLOUD_TRY(cudaSetDevice(device), "cudaSetDevice");
    // cos(apt * SF_PI / 180) in double, kept as float (Mbycloudwin3d.c:81)
    const float cosapt = (float)std::cos((double)apt * 3.14159265358979323846264338328 / 180);
    DevBufs B;
    float *d_g, *d_o;
    unsigned char *d_flag;
    long long *d_counts, *d_index;
    const long long nb = (ng + kChunk - 1) / kChunk;
    CLOUD_TRY(B.get(&d_g, (size_t)ng * kNco * sizeof(float)), "cudaMalloc");
    CLOUD_TRY(B.get(&d_o, (size_t)std::max<long long>(no, 1) * kNco * sizeof(float)), "cudaMalloc");
    CLOUD_TRY(B.get(&d_flag, (size_t)ng), "cudaMalloc");
    CLOUD_TRY(B.get(&d_counts, (size_t)(nb + 1) * sizeof(long long)), "cudaMalloc");
    CLOUD_TRY(B.get(&d_index, (size_t)ng * sizeof(long long)), "cudaMalloc");
    CLOUD_TRY(cudaMemcpy(d_g, ground, (size_t)ng * kNco * sizeof(float), cudaMemcpyHostToDevice), "upload");
    if (no > 0) CLOUD_TRY(cudaMemcpy(d_o, orbit, (size_t)no * kNco * sizeof(float), cudaMemcpyHostToDevice), "upload");
    k_cloud_flag<<<grid_for(ng), 256>>>(d_g, ng, d_o, no, cosapt, d_flag);
    k_chunk_count<<<(unsigned)nb, 256>>>(d_flag, ng, d_counts);
    k_scan_counts<<<1, 1024>>>(d_counts, nb);
    k_chunk_compact<<<(unsigned)nb, 256>>>(d_flag, ng, d_counts, d_index);
    CLOUD_TRY(cudaGetLastError(), "kernel launch");
    long long n = 0;
    CLOUD_TRY(cudaMemcpy(&n, d_counts + nb, sizeof n, cudaMemcpyDeviceToHost), "download");
    if (n > 0) {
        CLOUD_TRY(cudaMemcpy(index, d_index, (size_t)n * sizeof(long long), cudaMemcpyDeviceToHost), "download");
        if (win) {
            float *d_w;
            CLOUD_TRY(B.get(&d_w, (size_t)n * kNco * sizeof(float)), "cudaMalloc");
            k_gather_points<<<grid_for(n * kNco), 256>>>(d_g, d_index, n, d_w);
            CLOUD_TRY(cudaMemcpy(win, d_w, (size_t)n * kNco * sizeof(float), cudaMemcpyDeviceToHost), "download");
        }
        if (nf > 0) {
            float *d_d, *d_wd;
            CLOUD_TRY(B.get(&d_d, (size_t)nf * ng * ncomp * sizeof(float)), "cudaMalloc");
            CLOUD_TRY(B.get(&d_wd, (size_t)nf * n * ncomp * sizeof(float)), "cudaMalloc");
            CLOUD_TRY(cudaMemcpy(d_d, data, (size_t)nf * ng * ncomp * sizeof(float), cudaMemcpyHostToDevice),
                      "upload");
            dim3 grid(grid_for(n * ncomp), (unsigned)std::min<long long>(nf, 65535));
            k_gather_columns<<<grid, 256>>>(d_d, ng, d_index, n, nf, ncomp, d_wd);
            CLOUD_TRY(cudaMemcpy(win_data, d_wd, (size_t)nf * n * ncomp * sizeof(float), cudaMemcpyDeviceToHost),
                      "download");
        }
    }
    CLOUD_TRY(cudaDeviceSynchronize(), "synchronize");
    *nw = n;
    return AWE_OK;
}

awe_status awe_cloud_merge(int device, const float *all, long long na, int nwin, const long long *nwp,
                           const float *win_pts, const float *win_data, long long nf, int ncomp, int norm,
                           float hashscale, float *out) {
    const char *fn = "awe_cloud_merge";
    if (!all || !out || na <= 0 || nwin < 0 || (nwin > 0 && (!nwp || !win_pts || !win_data)) || nf < 0 ||
        (ncomp != 1 && ncomp != 2)) {
        set_error("%s: bad arguments (all, out, na > 0; window counts, points and data; ncomp 1 or 2)", fn);
        return AWE_ERR_INVALID;
    }
    long long ntot = 0;
    for (int c = 0; c < nwin; c++) {
        if (nwp[c] < 0) {
            set_error("%s: window %d has a negative size", fn, c);
            return AWE_ERR_INVALID;
        }
        ntot += nwp[c];
    }
    // centroid (float running sums, Mbycloudmerge3d.c:132-142) and the
    // smallest spacing of consecutive points (:146-152)
    float ox = 0.f, oy = 0.f, oz = 0.f;
    for (long long a = 0; a < na; a++) {
        ox += all[a * kNco];
        oy += all[a * kNco + 1];
        oz += all[a * kNco + 2];
    }
    ox /= (float)na;
    oy /= (float)na;
    oz /= (float)na;
    double ddmin = DBL_MAX;
    for (long long a = 1; a < na; a++)
        ddmin = std::min(ddmin, cloud_dist(all[a * kNco], all[a * kNco + 1], all[a * kNco + 2], all[(a - 1) * kNco],
                                           all[(a - 1) * kNco + 1], all[(a - 1) * kNco + 2]));
    const unsigned long long nhash = (unsigned long long)(hashscale * (float)na);
    if (nhash < (unsigned long long)na) {
        set_error("%s: hash table of %llu slots cannot hold %lld points (hashscale %g)", fn, nhash, na, hashscale);
        return AWE_ERR_INVALID;
    }
    // the table in insertion order, as htInsert fills it
    std::vector<long long> table(nhash, -1);
    for (long long a = 0; a < na; a++) {
        const unsigned long long h = cloud_hash(nhash, all[a * kNco], all[a * kNco + 1], all[a * kNco + 2], ox, oy, oz);
        unsigned long long j = 0;
        while (table[(h + j) % nhash] >= 0) j++;
        table[(h + j) % nhash] = a;
    }
    CLOUD_TRY(cudaSetDevice(device), "cudaSetDevice");
    DevBufs B;
    float *d_all, *d_out, *d_fold, *d_wp, *d_wd;
    long long *d_table, *d_idx;
    int *d_missing;
    const size_t out_bytes = (size_t)nf * na * ncomp * sizeof(float);
    long long wd_tot = 0;
    for (int c = 0; c < nwin; c++) wd_tot += nwp[c] * nf * ncomp;
    CLOUD_TRY(B.get(&d_all, (size_t)na * kNco * sizeof(float)), "cudaMalloc");
    CLOUD_TRY(B.get(&d_out, out_bytes), "cudaMalloc");
    CLOUD_TRY(B.get(&d_fold, (size_t)na * sizeof(float)), "cudaMalloc");
    CLOUD_TRY(B.get(&d_table, (size_t)nhash * sizeof(long long)), "cudaMalloc");
    CLOUD_TRY(B.get(&d_wp, (size_t)ntot * kNco * sizeof(float)), "cudaMalloc");
    CLOUD_TRY(B.get(&d_wd, (size_t)wd_tot * sizeof(float)), "cudaMalloc");
    CLOUD_TRY(B.get(&d_idx, (size_t)ntot * sizeof(long long)), "cudaMalloc");
    CLOUD_TRY(B.get(&d_missing, sizeof(int)), "cudaMalloc");
    CLOUD_TRY(cudaMemcpy(d_all, all, (size_t)na * kNco * sizeof(float), cudaMemcpyHostToDevice), "upload");
    CLOUD_TRY(cudaMemcpy(d_table, table.data(), (size_t)nhash * sizeof(long long), cudaMemcpyHostToDevice), "upload");
    if (ntot > 0) {
        CLOUD_TRY(cudaMemcpy(d_wp, win_pts, (size_t)ntot * kNco * sizeof(float), cudaMemcpyHostToDevice), "upload");
        CLOUD_TRY(cudaMemcpy(d_wd, win_data, (size_t)wd_tot * sizeof(float), cudaMemcpyHostToDevice), "upload");
    }
    CLOUD_TRY(cudaMemset(d_out, 0, out_bytes), "cudaMemset");
    CLOUD_TRY(cudaMemset(d_fold, 0, (size_t)na * sizeof(float)), "cudaMemset");
    CLOUD_TRY(cudaMemset(d_missing, 0, sizeof(int)), "cudaMemset");
    if (ntot > 0)
        k_cloud_lookup<<<grid_for(ntot), 256>>>(d_all, d_table, nhash, ox, oy, oz, ddmin / 10, d_wp, ntot, d_idx,
                                                d_missing);
    int missing = 0;
    CLOUD_TRY(cudaMemcpy(&missing, d_missing, sizeof missing, cudaMemcpyDeviceToHost), "download");
    if (missing) {
        set_error("%s: a window point has no full-cloud point within %g (ddMIN/10)", fn, ddmin / 10);
        return AWE_ERR_INVALID;
    }
    long long p0 = 0, d0 = 0;
    for (int c = 0; c < nwin; c++) {  // windows in order: the reference's summation order
        const long long m = nwp[c];
        if (m > 0) {
            dim3 grid(grid_for(m * ncomp), (unsigned)std::max<long long>(1, std::min<long long>(nf, 65535)));
            if (nf > 0) k_cloud_add<<<grid, 256>>>(d_wd + d0, m, d_idx + p0, na, nf, ncomp, d_out);
            if (norm) k_cloud_fold<<<grid_for(m), 256>>>(d_idx + p0, m, d_fold);
        }
        p0 += m;
        d0 += m * nf * ncomp;
    }
    if (norm && nf > 0) k_cloud_norm<<<grid_for(na * nf * ncomp), 256>>>(d_out, d_fold, na, nf, ncomp);
    CLOUD_TRY(cudaGetLastError(), "kernel launch");
    CLOUD_TRY(cudaMemcpy(out, d_out, out_bytes, cudaMemcpyDeviceToHost), "download");
    return AWE_OK;
}

}  // extern "C"
