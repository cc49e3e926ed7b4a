/* CPU oracle for the acoustic wave-propagation hot path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, the smoke check and
 * bench.py's CPU-baseline leg may load this library, and only as the checker.
 * The product path (wavefield_imaging_gb300, libawe) never calls it.
 *
 * It is a plain-C restatement of the reference's algorithms
 * (Nacnud04/wavefield_imaging, CODE/), one entry point per reference program:
 *   orc_cart2d_cpu / orc_cart3d_cpu   - MAWEFDcart{2D,3D}cpu.c (+ ts_kernel.c,
 *                                       fdutil.c): 2N-order Laplacian,
 *                                       Gaussian sponge, one-way ABC,
 *                                       v^2 dt^2-scaled injection.
 * Every float operation is evaluated in the reference's order and precision,
 * so a build with -ffp-contract=off is bit-identical to the reference
 * programs built the same way (pinned by tests/test_oracle_golden.py against
 * fixtures produced by the reference itself, tests/golden/make_golden.py).
 *
 * Compiled twice: liboracle.so (REAL=float, the exact restatement) and
 * liboracle64.so (REAL=double: the same scheme with FP64 wavefields, used to
 * state the FP32 error of each configuration). */
#ifndef AWE_ORACLE_H
#define AWE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int n1, n2, n3;   /* unpadded model size; axis 1 fastest (z, x, y); n3 = 1 in 2D */
    float d1, d2, d3; /* grid spacing per axis */
    float o1, o2, o3; /* origin per axis */
    int nb;           /* requested padding (nb= parameter); < 0 means "not given" */
    int nt;
    float dt;
    int fdorder; /* spatial order 2N (fdorder=) */
    int optfd;   /* least-squares optimal coefficients (optfd=) */
    int dabc;    /* absorbing boundary (dabc=) */
    int fsrf;    /* free surface (free=) */
    int hybrid;  /* hybrid one-way ABC (hybridbc=) */
    int expl;    /* one wavelet for all sources (expl=) */
    int jsnap;   /* snapshot interval; 0 = no snapshots */
    int bnds;    /* snapshots include the padding (bnds=) */
    int nthreads;
} orc_par;

/* Sizes of the padded grid and of one snapshot for parameters p. */
int orc_cart_padded(const orc_par *p, int *nbd, int *n1pad, int *n2pad, int *n3pad);

/* 2D cartesian, scheme of CODE/MAWEFDcart2Dcpu.c.
 * vel, den: [n2][n1] (den may be NULL: constant density).
 * wav: expl ? [nt] : [nt][ns].  sou: [ns][2] (x, z); rec: [nr][2].
 * dat: [nt][nr].  snaps (may be NULL): one frame per it % jsnap == 0. */
int orc_cart2d_cpu(const orc_par *p, const float *vel, const float *den, const float *wav, int ns,
                   const float *sou, int nr, const float *rec, float *dat, float *snaps);

/* 3D cartesian, scheme of CODE/MAWEFDcart3Dcpu.c.  vel, den: [n3][n2][n1];
 * sou/rec: [n][3] (x, y, z). */
int orc_cart3d_cpu(const orc_par *p, const float *vel, const float *den, const float *wav, int ns,
                   const float *sou, int nr, const float *rec, float *dat, float *snaps);

/* Scheme of the GPU programs (awe_oracle_gpu.c).  kind: 0 sfAWEFDcart2Dgpu,
 * 1 sfAWEFDcart3Dgpu (n1 == n2), 2 sfAWEFDspher2Dgpu (polar), 3
 * sfAWEFDspher3Dgpu.  Model [n3][n2][n1] axis 1 fastest (z or r); points in
 * the programs' order: (x,z), (x,y,z), (r,theta), (r,phi,theta).  wav: [nt]
 * (the programs read wav[it]).  dat rows: nt/jdata (spherical 3D: nt). */
typedef struct {
    int n1, n2, n3;
    float d1, d2, d3;
    float o1, o2, o3;
    int nb, nt;
    float dt;
    int jdata, jsnap, bnds, fsrf, expl, refl;
} orc_gpar;

/* The spherical 3D case with FP64 wavefields and arithmetic; dat [nt][nr] double. */
int orc_gpu_spher3d_fp64(const orc_gpar *p, const float *vel, const float *wav, int ns, const float *sou, int nr,
                         const float *rec, double *dat);

/* sfAWEFDspher3Dgpu adj=y (MAWEFDspher3Dgpu.cu:449-566): data [nt][nr]
 * injected, reversed in time, at the receivers; image [nph][nth][nra] is the
 * wavefield's model window after step nt-kt; frames as the program writes
 * them.  Returns the frames written (-1: kt outside [1, nt]). */
int orc_gpu_spher3d_adj(const orc_gpar *p, const float *vel, const float *data, int nr, const float *rec, int kt,
                        float *image, float *snaps);
int orc_gpu_forward(int kind, const orc_gpar *p, const float *vel, const float *rfl, const float *wav, int ns,
                    const float *sou, int nr, const float *rec, float *dat, float *snaps);
/* sfAWEFDcart2Dgpu's scheme on a moving geometry (expl = refl = 0): sou
 * ns*nst points, rec nr*nrt points; move 0 = one row per step (last row
 * held), 1 = MDYNAWEFDcart2Dgpu (entry k*(it+1), free surface only with fsrf) */
int orc_gpu_cart2d_moving(const orc_gpar *p, const float *vel, const float *wav, int ns, int nst, const float *sou,
                          int nr, int nrt, const float *rec, int move, float *dat, float *snaps);

/* Time nsteps of the 3D scheme-B update on a padded grid (for the CPU
 * baseline): returns wall seconds.  Fields are allocated internally. */
double orc_cart3d_cpu_steps(int n1pad, int n2pad, int n3pad, int fdorder, int nsteps, int nthreads);

#ifdef __cplusplus
}
#endif
/* point-cloud tools (oracle/awe_cloud.c): Mbycloudwin3d (fast=y) and
 * Mbycloudmerge3d; ncomp floats per data sample (2 = complex) */
int orc_cloud_window(const float *g, long long ng, const float *o, long long no, float apt, long long nf, int ncomp,
                     const float *data, long long *nw, long long *index, float *win, float *win_data);
int orc_cloud_merge(const float *all, long long na, int nwin, const long long *nwp, const float *win_pts,
                    const float *win_data, long long nf, int ncomp, int norm, float hashscale, float *out);

#endif
