// Host-side set-up math: finite-difference coefficients, sponge and damping
// profiles, bilinear/trilinear interpolation weights and model padding.
// Each function evaluates in the same float/double order as the reference
// (cited per function) so the device path starts from bit-identical tables.
// Built with -ffp-contract=off: no fused multiply-adds on any host.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "awe_internal.h"

namespace awe {

static int factorial(int n) {
    int r = 1;
    for (int i = 1; i <= n; ++i) r *= i;
    return r;
}

// Published least-squares optimal coefficients used by the reference's
// optfd=y (MAWEFDcart2Dcpu.c:502-551): second derivative (Liu 2013) for
// nop 1..10 and first derivative (Zhang & Yao 2013) for nop 1..6.  Entries
// the reference writes as double literals are double literals here too, so
// the float conversion is the same.
static const float kOptC[11][11] = {
    {0},
    {0.f, 1.f},
    {0.f, 1.369074f, -0.09266816},
    {0.f, 1.573661f, -0.1820268f, 0.01728053f},
    {0.f, 1.700010f, -0.2554615f, 0.04445392f, -0.004946851f},
    {0.f, 1.782836f, -0.3124513f, 0.07379487f, -0.01532122f, 0.001954439f},
    {0.f, 1.837023f, -0.3538895f, 0.09978343f, -0.02815486f, 0.006556587f, -0.0009405699f},
    {0.f, 1.874503f, -0.3845794f, 0.1215162f, -0.04121749f, 0.01295522f, -0.003313813f, 0.0005310053f},
    {0.f, 1.901160f, -0.4074304f, 0.1390909f, -0.05318775f, 0.02004823f, -0.006828249f, 0.001895771f,
     -0.0003369052f},
    {0.f, 1.919909f, -0.4240446f, 0.1526043f, -0.06322328f, 0.02676005f, -0.01080739f, 0.003907747f,
     -0.001158024f, 0.0002240247f},
    {0.f, 1.918204f, -0.4225858f, 0.1514992f, -0.06249474f, 0.02637196f, -0.01066631f, 0.003915625f,
     -0.001219872f, 0.0002863976f, -0.00003744830f}};
static const float kOptB[7][7] = {{0},
                                  {0.0f, 0.5f},
                                  {0.0f, 0.67880327, -0.08962729},
                                  {0.0f, 0.77793115, -0.17388691, 0.02338713},
                                  {0.0f, 0.84149635, -0.24532989, 0.06081891, -0.00839807},
                                  {0.0f, 0.88414717, -0.30233648, 0.10275057, -0.02681517, 0.00398089},
                                  {0.0f, 0.91067892, -0.34187892, 0.13833962, -0.04880710, 0.01302148,
                                   -0.00199047}};

// compute_fdcoef + normal_fdcoef (MAWEFDcart3Dcpu.c:404-480): central
// 2N-order weights from the scaled-binomial formula (Chu & Stoffa 2012),
// divided by d^2 (second) or d (first derivative) per axis; centre weight
// -2 * (sum over all axes).  dd[] = spacing per axis in (z, x, y) order.
void fd_coefficients(int nop, int ndim, const float *dd, int optfd, Coef &k) {
    std::memset(&k, 0, sizeof k);
    float cc[kMaxNop + 1] = {0}, bb[kMaxNop + 1] = {0};
    int half = factorial(nop);
    half *= half;
    for (int n = 1; n <= nop; n++) {
        cc[n] = -2.f / (n * n) * std::cos(n * 3.14159265358979323846264338328) * half / factorial(nop + n) /
                factorial(nop - n);
        bb[n] = cc[n] * n / 2.f;
    }
    const float *c2 = optfd ? kOptC[nop] : cc;
    const float *c1 = (optfd && nop <= 6) ? kOptB[nop] : bb;
    float c0 = 0.f;
    for (int idim = 0; idim < ndim; idim++) {
        float dsq = dd[idim] * dd[idim];
        for (int ii = 1; ii <= nop; ii++) {
            k.c[idim][ii] = c2[ii] / dsq;
            c0 += k.c[idim][ii];
        }
    }
    c0 *= -2.0f;
    k.c0 = c0;
    for (int idim = 0; idim < ndim; idim++)
        for (int ii = 1; ii <= nop; ii++) k.b[idim][ii] = c1[ii] / dd[idim];
}

// sponge_make (fdutil.c:2181-2200): w[ib] = exp(-(ib / (sqrt(2) * 4 nb))^2)
void sponge_weights(int nb, std::vector<float> &w) {
    w.assign(nb > 0 ? nb : 0, 1.f);
    float sb = 4.0 * nb;
    for (int ib = 0; ib < nb; ib++) {
        float fb = ib / (std::sqrt(2.0) * sb);
        w[ib] = (float)std::exp((double)(-fb * fb));  // C's double exp, as the reference
    }
}

void undamped_range(const std::vector<float> &w, int &lo, int &hi) {
    const int n = (int)w.size();
    lo = 0;
    hi = n;
    for (int i = 0; i < n / 2; i++)
        if (w[i] != 1.f) lo = i + 1;
    for (int i = n - 1; i >= n / 2; i--)
        if (w[i] != 1.f) hi = i;
    if (hi < lo) hi = lo;
}

// damp_make (MAWEFDcart2Dcpu.c:407-421): the same profile over nbd - nop cells
void hybrid_damp(int ntransit, std::vector<float> &w) { sponge_weights(ntransit, w); }

// lint2d_make / lint3d_make (fdutil.c:1363-1404, :1474-1539): index of the
// lower corner and fractional weights; a point outside the padded grid maps
// to corner (0,0[,0]) with all weight on the +z neighbour.
Lint lint_make(int ndim, float x, float y, float z, const FdmAxes &f) {
    Lint c{};
    float f1, f2, f3 = 0.f;
    bool inside = z >= f.oz && z < f.oz + (f.nz - 1) * f.dz && x >= f.ox && x < f.ox + (f.nx - 1) * f.dx;
    if (ndim == 3) inside = inside && y >= f.oy && y < f.oy + (f.ny - 1) * f.dy;
    if (inside) {
        c.jz = (int)((z - f.oz) / f.dz);
        c.jx = (int)((x - f.ox) / f.dx);
        f1 = (z - f.oz) / f.dz - c.jz;
        f2 = (x - f.ox) / f.dx - c.jx;
        if (ndim == 3) {
            c.jy = (int)((y - f.oy) / f.dy);
            f3 = (y - f.oy) / f.dy - c.jy;
        }
    } else {
        c.jz = c.jx = c.jy = 0;
        f1 = 1;
        f2 = 0;
        f3 = 0;
    }
    if (ndim == 2) {
        c.w[0] = (1 - f1) * (1 - f2);
        c.w[1] = (f1) * (1 - f2);
        c.w[2] = (1 - f1) * (f2);
        c.w[3] = (f1) * (f2);
    } else {
        c.w[0] = (1 - f3) * (1 - f1) * (1 - f2);
        c.w[1] = (1 - f3) * (f1) * (1 - f2);
        c.w[2] = (1 - f3) * (1 - f1) * (f2);
        c.w[3] = (1 - f3) * (f1) * (f2);
        c.w[4] = (f3) * (1 - f1) * (1 - f2);
        c.w[5] = (f3) * (f1) * (1 - f2);
        c.w[6] = (f3) * (1 - f1) * (f2);
        c.w[7] = (f3) * (f1) * (f2);
    }
    return c;
}

// expand2d / expand3d (fdutil.c:435-571): copy into the interior, then
// replicate the edge values outward along axis 1, axis 2, axis 3 in turn.
// a: [n3][n2][n1]; b: padded.
void expand_model(int ndim, const float *a, float *b, int nb, const int *n) {
    const size_t n1 = n[0], n2 = n[1], n3 = ndim == 3 ? n[2] : 1;
    const size_t p1 = n1 + 2 * nb, p2 = n2 + 2 * nb, p3 = ndim == 3 ? n3 + 2 * nb : 1;
    const size_t o3 = ndim == 3 ? nb : 0;
    auto B = [&](size_t i3, size_t i2, size_t i1) -> float & { return b[(i3 * p2 + i2) * p1 + i1]; };
    for (size_t i3 = 0; i3 < n3; i3++)
        for (size_t i2 = 0; i2 < n2; i2++)
            std::memcpy(&B(o3 + i3, nb + i2, nb), a + (i3 * n2 + i2) * n1, n1 * sizeof(float));
    for (size_t i3 = 0; i3 < p3; i3++)
        for (size_t i2 = 0; i2 < p2; i2++)
            for (int i1 = 0; i1 < nb; i1++) {
                B(i3, i2, i1) = B(i3, i2, nb);
                B(i3, i2, p1 - i1 - 1) = B(i3, i2, p1 - nb - 1);
            }
    for (size_t i3 = 0; i3 < p3; i3++)
        for (int i2 = 0; i2 < nb; i2++)
            for (size_t i1 = 0; i1 < p1; i1++) {
                B(i3, i2, i1) = B(i3, nb, i1);
                B(i3, p2 - i2 - 1, i1) = B(i3, p2 - nb - 1, i1);
            }
    if (ndim == 3)
        for (int i3 = 0; i3 < nb; i3++)
            for (size_t i2 = 0; i2 < p2; i2++)
                for (size_t i1 = 0; i1 < p1; i1++) {
                    B(i3, i2, i1) = B(nb, i2, i1);
                    B(p3 - i3 - 1, i2, i1) = B(p3 - nb - 1, i2, i1);
                }
}

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

const char *last_error() { return g_err; }

}  // namespace awe
