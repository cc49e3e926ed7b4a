// 2D forward modelling that allocates nothing.
//
// Some callers cannot call cudaMalloc: code that runs inside a framework that
// owns the device memory pool, code that is captured into a larger CUDA
// graph, or plug-ins that must not grow the process's device footprint at run
// time.  They hand over device buffers for the inputs and outputs only; the
// wavefields, the padded v^2 dt^2 model, the sponge tables and the
// interpolation points live in one file-scope __device__ array instead.
//
// The array's size is fixed at build time (kStaticBytes, about 12.2 MiB) and
// every GPU that loads this library holds it until the process exits.  All
// calls share it: each call re-initialises what must start at zero, and two
// calls whose work overlaps on the GPU (different streams, or different host
// threads on the same device) race on it and produce garbage.
//
// The arithmetic is that of awe_forward for the same descriptor: the same
// set-up formulas (evaluated on the device with explicitly rounded float
// operations) and the same step, injection, sponge and gather kernels.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "awe_internal.h"

namespace awe {

// Limits of the static scratch (padded grid, points, sponge width).
constexpr long long kStaticMaxCells = 1ll << 20;  // padded n1 * n2
constexpr int kStaticMaxAxis = 8192;              // padded length of one axis
constexpr int kStaticMaxPoints = 4096;            // sources + receivers
constexpr int kStaticMaxNb = 256;                 // padding / sponge width

constexpr size_t kOffU0 = 0;
constexpr size_t kOffU1 = kOffU0 + kStaticMaxCells * sizeof(float);
constexpr size_t kOffVel = kOffU1 + kStaticMaxCells * sizeof(float);
constexpr size_t kOffW1 = kOffVel + kStaticMaxCells * sizeof(float);
constexpr size_t kOffW2 = kOffW1 + kStaticMaxAxis * sizeof(float);
constexpr size_t kOffW3 = kOffW2 + kStaticMaxAxis * sizeof(float);
constexpr size_t kOffOff = kOffW3 + 256;
constexpr size_t kOffPts = kOffOff + 256;
constexpr size_t kStaticBytes = kOffPts + kStaticMaxPoints * sizeof(GeoPoint);

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

// Host-side address of g_static_scratch per device (the symbol's host name
// is only a stand-in).  It is looked up with the device current on every
// call made outside stream capture, so a context that was torn down and
// rebuilt (cudaDeviceReset), which may load the module at another address,
// is followed; a call made during capture uses the address cached by the
// last call outside capture on that device.
static std::mutex g_static_mu;
static void *g_static_addr[64];

static awe_status static_scratch(int dev, cudaStream_t s, unsigned char **out) {
    if (dev < 0 || dev >= 64) {
        set_error("device index %d beyond the static-scratch table", dev);
        return AWE_ERR_INVALID;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusNone;
    }
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (cap == cudaStreamCaptureStatusNone || !g_static_addr[dev]) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_scratch);
        if (e != cudaSuccess || !ptr) {
            set_error("cudaGetSymbolAddress(static scratch) failed: %s", cudaGetErrorString(e));
            return AWE_ERR_CUDA;
        }
        g_static_addr[dev] = ptr;
    }
    *out = (unsigned char *)g_static_addr[dev];
    return AWE_OK;
}

struct SpongeParam {
    float w[kStaticMaxNb];
};

// per-axis sponge factors and the cartesian 2D corner offsets
__global__ void k_na_tables(float *w1, int n1, float *w2, int n2, float *w3, long long *off, int nb, int sponge,
                            SpongeParam sw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n1) {
        float t = 1.f;
        if (sponge && i < nb) t = sw.w[nb - i - 1];
        if (sponge && i >= n1 - nb) t = sw.w[nb - (n1 - 1 - i) - 1];
        w1[i] = t;
    }
    if (i < n2) {
        float t = 1.f;
        if (sponge && i < nb) t = sw.w[nb - i - 1];
        if (sponge && i >= n2 - nb) t = sw.w[nb - (n2 - 1 - i) - 1];
        w2[i] = t;
    }
    if (i == 0) {
        w3[0] = 1.f;
        off[0] = 0;
        off[1] = 1;
        off[2] = n1;
        off[3] = (long long)n1 + 1;
        for (int c = 4; c < 8; c++) off[c] = 0;
    }
}

// edge-replicating pad (expand2d) and v <- v * (v * dt^2), free surface zeroes
// the first nb+1 samples of every axis-1 line
__global__ void k_na_pad_vel(const float *__restrict__ vel, float *__restrict__ v2, int n1, int n2, int nb,
                             float dt2, int fsrf) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int p1 = n1 + 2 * nb, p2 = n2 + 2 * nb;
    if (t >= (long long)p1 * p2) return;
    const int i1 = (int)(t % p1), i2 = (int)(t / p1);
    const int j1 = min(max(i1 - nb, 0), n1 - 1), j2 = min(max(i2 - nb, 0), n2 - 1);
    const float v = vel[(long long)j2 * n1 + j1];
    float out = __fmul_rn(v, __fmul_rn(v, dt2));
    if (fsrf && i1 < nb + 1) out = 0.f;
    v2[t] = out;
}

// lint2d_make for each point, with explicitly rounded float operations
__global__ void k_na_lint2d(const float *__restrict__ xz, int n, GeoPoint *pts, float oz, float ox, float dz,
                            float dx, int nz, int nx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = xz[2 * i], z = xz[2 * i + 1];
    int jz = 0, jx = 0;
    float f1 = 1.f, f2 = 0.f;
    const bool inside = z >= oz && z < __fadd_rn(oz, __fmul_rn((float)(nz - 1), dz)) && x >= ox &&
                        x < __fadd_rn(ox, __fmul_rn((float)(nx - 1), dx));
    if (inside) {
        const float qz = __fdiv_rn(__fsub_rn(z, oz), dz), qx = __fdiv_rn(__fsub_rn(x, ox), dx);
        jz = __float2int_rz(qz);
        jx = __float2int_rz(qx);
        f1 = __fsub_rn(qz, (float)jz);
        f2 = __fsub_rn(qx, (float)jx);
    }
    GeoPoint g;
    g.base = (long long)jx * nz + jz;
    g.w[0] = __fmul_rn(__fsub_rn(1.f, f1), __fsub_rn(1.f, f2));
    g.w[1] = __fmul_rn(f1, __fsub_rn(1.f, f2));
    g.w[2] = __fmul_rn(__fsub_rn(1.f, f1), f2);
    g.w[3] = __fmul_rn(f1, f2);
    for (int c = 4; c < 8; c++) g.w[c] = 0.f;
    pts[i] = g;
}

}  // namespace awe

using namespace awe;

extern "C" awe_status awe_forward2d_noalloc(const awe_desc *desc, const float *d_vel, const float *d_wav, int ncs,
                                            int ns, const float *d_sou, int nr, const float *d_rec, float *d_dat,
                                            void *stream) {
    if (!desc || !d_vel || !d_wav || !d_dat || ns < 0 || nr < 0 || (ns && !d_sou) || (nr && !d_rec)) {
        set_error("awe_forward2d_noalloc: null or negative argument");
        return AWE_ERR_INVALID;
    }
    // awe_plan_create's checks first, then what this path leaves out
    const awe_status chk = check_desc(desc);
    if (chk != AWE_OK) return chk;
    const awe_desc &d = *desc;
    if (d.ndim != 2 || d.coords != AWE_CART || d.scheme != AWE_SCHEME_CPU) {
        set_error("awe_forward2d_noalloc: only the 2D cartesian CPU-program scheme is available without allocation");
        return AWE_ERR_UNSUPPORTED;
    }
    if (d.hybrid || d.jsnap != 0 || d.bnds || d.refl) {
        set_error("awe_forward2d_noalloc: hybrid ABC, snapshots and reflectivity injection need awe_forward");
        return AWE_ERR_UNSUPPORTED;
    }
    const int fdorder = d.fdorder ? d.fdorder : 4;
    if (ncs != 1 && ncs != ns) {
        set_error("awe_forward2d_noalloc: ncs must be 1 or ns (ncs %d, ns %d)", ncs, ns);
        return AWE_ERR_INVALID;
    }
    const int nop = fdorder / 2;
    const int nb = d.nb < nop ? nop : d.nb;
    const long long p1 = d.n[0] + 2ll * nb, p2 = d.n[1] + 2ll * nb;
    if (nb > kStaticMaxNb || p1 > kStaticMaxAxis || p2 > kStaticMaxAxis || p1 * p2 > kStaticMaxCells ||
        ns + (long long)nr > kStaticMaxPoints) {
        set_error("awe_forward2d_noalloc: size beyond the static scratch (padded %lld x %lld = %lld cells, max %lld; "
                  "axis max %d; nb %d, max %d; %d points, max %d)",
                  p1, p2, p1 * p2, kStaticMaxCells, kStaticMaxAxis, nb, kStaticMaxNb, ns + nr, kStaticMaxPoints);
        return AWE_ERR_INVALID;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        set_error("awe_forward2d_noalloc: no CUDA device");
        return AWE_ERR_NODEVICE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *base = nullptr;
    awe_status st = static_scratch(dev, s, &base);
    if (st != AWE_OK) return st;

    float *u0 = (float *)(base + kOffU0), *u1 = (float *)(base + kOffU1), *vel = (float *)(base + kOffVel);
    float *w1 = (float *)(base + kOffW1), *w2 = (float *)(base + kOffW2), *w3 = (float *)(base + kOffW3);
    long long *off = (long long *)(base + kOffOff);
    GeoPoint *src = (GeoPoint *)(base + kOffPts), *rec = src + ns;

    // set-up on the host: coefficients and sponge profile (sponge_make,
    // fdutil.c:2181-2200), stack storage only
    Coef k;
    const float dd[3] = {d.d[0], d.d[1], 1.f};
    fd_coefficients(nop, 2, dd, d.optfd, k);
    SpongeParam sw;
    {
        float sb = 4.0 * nb;
        for (int ib = 0; ib < nb; ib++) {
            float fb = ib / (std::sqrt(2.0) * sb);
            sw.w[ib] = (float)std::exp((double)(-fb * fb));
        }
    }
    const bool sponge = d.dabc != 0;
    const float oz = d.o[0] - nb * d.d[0], ox = d.o[1] - nb * d.d[1];

    // set-up on the device: tables, padded model, interpolation points, zeroed levels
    const int T = 256;
    const long long maxax = p1 > p2 ? p1 : p2;
    k_na_tables<<<(unsigned)((maxax + T - 1) / T), T, 0, s>>>(w1, (int)p1, w2, (int)p2, w3, off, nb, sponge, sw);
    k_na_pad_vel<<<(unsigned)((p1 * p2 + T - 1) / T), T, 0, s>>>(d_vel, vel, d.n[0], d.n[1], nb, d.dt * d.dt,
                                                                  d.fsrf);
    if (ns) k_na_lint2d<<<(ns + T - 1) / T, T, 0, s>>>(d_sou, ns, src, oz, ox, d.d[0], d.d[1], (int)p1, (int)p2);
    if (nr) k_na_lint2d<<<(nr + T - 1) / T, T, 0, s>>>(d_rec, nr, rec, oz, ox, d.d[0], d.d[1], (int)p1, (int)p2);
    if (cudaMemsetAsync(u0, 0, p1 * p2 * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(u1, 0, p1 * p2 * sizeof(float), s) != cudaSuccess) {
        set_error("awe_forward2d_noalloc: clearing the wavefields failed");
        return AWE_ERR_CUDA;
    }

    // time loop of MAWEFDcart2Dcpu.c:297-383 (the sponge of the new level is
    // applied after the injection, so a source inside the sponge band is
    // handled without a geometry check on the host)
    const Grid g{(int)p1, (int)p2, 1};
    StepBParams sp{};
    sp.g = g;
    sp.k = k;
    sp.w1 = w1;
    sp.w2 = w2;
    sp.w3 = w3;
    sp.damp_prev = sponge;
    sp.sponge_new = 0;
    sp.shell = 0;
    const bool exact = d.precision == AWE_EXACT;
    const int jdata = d.jdata > 0 ? d.jdata : 1;  // 0 = the default, 1
    float *cur = u1, *nxt = u0;
    int row = 0;
    for (int it = 0; it < d.nt; it++) {
        launch_stepB(2, nop, exact, false, cur, nxt, vel, nullptr, sp, s);
        launch_injectB_off(2, exact, nxt, vel, src, ns, d_wav, it, ncs, ncs == 1, off, s);
        if (sponge) launch_band_sponge(2, nb, exact, nxt, w1, w2, w3, g, s);
        float *t = cur;
        cur = nxt;
        nxt = t;
        if (it % jdata == 0) {
            launch_extract_off(2, exact, nxt, rec, nr, d_dat + (size_t)row * nr, sponge ? w1 : nullptr, w2, w3, g,
                               off, s);
            row++;
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("awe_forward2d_noalloc: launch failed: %s", cudaGetErrorString(e));
        return AWE_ERR_CUDA;
    }
    return AWE_OK;
}
