/* CPU oracle, part 3: restatement of the reference's point-cloud tools
 * (CODE/Mbycloudwin3d.c, CODE/Mbycloudmerge3d.c, CODE/hash.c).  TEST
 * INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * Window (Mbycloudwin3d.c:108-246, fast=y): a ground point is kept when
 * some orbit point lies in its aperture cone, |unit(orbit - ground) .
 * normal| > cos(apt) (isInCone, :19-35, float arithmetic in the same
 * order); kept points and their data columns are copied in input order.
 *
 * Merge (Mbycloudmerge3d.c:119-300): the full cloud goes into an
 * open-addressing table (FNV-1a of the distance to the centroid, linear
 * probing, hash.c:33-94); each window point takes the first occupied slot
 * from its own hash on whose point lies within ddMIN/10 (hash.c:162-190);
 * the windows' samples are summed in window order and divided by the fold.
 * Built with -ffp-contract=off, so no fused multiply-adds. */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "awe_oracle.h"

#define NCO 9

static int cone(const float *o, const float *g, float cosapt) {
    float rx = o[0] - g[0], ry = o[1] - g[1], rz = o[2] - g[2];
    const float r = sqrtf(rx * rx + ry * ry + rz * rz);
    rx /= r;
    ry /= r;
    rz /= r;
    const float c = rx * g[3] + ry * g[4] + rz * g[5];
    return (c >= 0 ? c : -c) > cosapt;
}

int orc_cloud_window(const float *g, long long ng, const float *o, long long no, float apt, long long nf, int ncomp,
                     const float *data, long long *nw, long long *index, float *win, float *win_data) {
    const float cosapt = (float)cos((double)apt * 3.14159265358979323846264338328 / 180);
    long long n = 0;
    for (long long i = 0; i < ng; i++)
        for (long long j = 0; j < no; j++)
            if (cone(o + j * NCO, g + i * NCO, cosapt)) {
                index[n++] = i;
                break;
            }
    for (long long w = 0; w < n && win; w++) memcpy(win + w * NCO, g + index[w] * NCO, NCO * sizeof(float));
    for (long long f = 0; f < nf; f++)
        for (long long w = 0; w < n; w++)
            for (int c = 0; c < ncomp; c++)
                win_data[(f * n + w) * ncomp + c] = data[(f * ng + index[w]) * ncomp + c];
    *nw = n;
    return 0;
}

/* hash.c's distance: float differences, double squares and sum, sqrtf */
static double dist(const float *a, const float *b) {
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return (double)sqrtf((float)(dx * dx + dy * dy + dz * dz));
}

static unsigned long long fnv(unsigned long long nhash, const float *p, const float *o) {
    const double h = dist(p, o);
    unsigned char b[8];
    memcpy(b, &h, 8);
    unsigned long long x = 14695981039346656037ull;
    for (int i = 0; i < 8; i++) {
        x ^= b[i];
        x *= 1099511628211ull;
    }
    x *= 1099511628211ull;
    return x % nhash;
}

int orc_cloud_merge(const float *all, long long na, int nwin, const long long *nwp, const float *win_pts,
                    const float *win_data, long long nf, int ncomp, int norm, float hashscale, float *out) {
    float o[3] = {0, 0, 0};
    for (long long a = 0; a < na; a++)
        for (int k = 0; k < 3; k++) o[k] += all[a * NCO + k];
    for (int k = 0; k < 3; k++) o[k] /= (float)na;
    double ddmin = DBL_MAX;
    for (long long a = 1; a < na; a++) {
        const double d = dist(all + a * NCO, all + (a - 1) * NCO);
        if (d < ddmin) ddmin = d;
    }
    const unsigned long long nhash = (unsigned long long)(hashscale * (float)na);
    if (nhash < (unsigned long long)na) return 2;
    long long *table = malloc(nhash * sizeof(long long));
    for (unsigned long long s = 0; s < nhash; s++) table[s] = -1;
    for (long long a = 0; a < na; a++) {
        unsigned long long s = fnv(nhash, all + a * NCO, o);
        while (table[s] >= 0) s = (s + 1) % nhash;
        table[s] = a;
    }
    float *fold = calloc((size_t)na, sizeof(float));
    memset(out, 0, (size_t)nf * na * ncomp * sizeof(float));
    long long p0 = 0, d0 = 0;
    int rc = 0;
    for (int c = 0; c < nwin && !rc; c++) {
        for (long long w = 0; w < nwp[c]; w++) {
            const float *q = win_pts + (p0 + w) * NCO;
            const unsigned long long h = fnv(nhash, q, o);
            long long a = -1;
            for (unsigned long long j = 0; j < nhash && a < 0; j++) {
                const long long t = table[(h + j) % nhash];
                if (t >= 0 && dist(all + t * NCO, q) < ddmin / 10) a = t;
            }
            if (a < 0) {
                rc = 3;
                break;
            }
            for (long long f = 0; f < nf; f++)
                for (int k = 0; k < ncomp; k++)
                    out[(f * na + a) * ncomp + k] += win_data[d0 + (f * nwp[c] + w) * ncomp + k];
            fold[a] += 1;
        }
        p0 += nwp[c];
        d0 += nwp[c] * nf * ncomp;
    }
    if (norm && !rc)
        for (long long f = 0; f < nf; f++)
            for (long long a = 0; a < na; a++)
                for (int k = 0; k < ncomp; k++) out[(f * na + a) * ncomp + k] /= (fold[a] > 1 ? fold[a] : 1);
    free(fold);
    free(table);
    return rc;
}
