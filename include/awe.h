/* awe.h - C-ABI of the GB300-native acoustic wave-propagation engine.
 *
 * Drop-in boundary for the time-stepping path of the reference programs
 * sfAWEFDcart2Dgpu, sfAWEFDcart3Dgpu, sfAWEFDspher2Dgpu and sfAWEFDspher3Dgpu
 * (Nacnud04/wavefield_imaging, CODE/MAWEFD{cart,spher}{2D,3D}gpu.cu) and of
 * the cartesian CPU programs MAWEFDcart{2D,3D}cpu.c whose 2N-order scheme the
 * GPU programs lack.  Plain C types only: pointers, sizes, scalars.
 *
 * Each entry point replaces one stage of the reference program's main():
 *   awe_plan_create   <- parameter parsing + fdutil_init/fdutil3d_init + the
 *                        cudaMalloc block (MAWEFDcart2Dgpu.cu:74-166, :188-259;
 *                        MAWEFDcart2Dcpu.c:116-235)
 *   awe_set_model     <- sf_floatread(vel/den/rfl) + expand_cpu_2d/3d or
 *                        expand2d/3d + cudaMemcpy (MAWEFDcart2Dgpu.cu:226-246;
 *                        MAWEFDcart3Dcpu.c:257-293)
 *   awe_set_geometry  <- pt2dread1/pt3dread1 + lint2d_make/lint3d_make +
 *                        cudaMemcpy of weights (MAWEFDcart2Dgpu.cu:307-343;
 *                        fdutil.c:1363-1539)
 *   awe_forward       <- the time loop and the trace/snapshot output
 *                        (MAWEFDcart2Dgpu.cu:362-511; MAWEFDcart3Dgpu.cu:380-477;
 *                        MAWEFDspher2Dgpu.cu:341-435; MAWEFDspher3Dgpu.cu:449-566;
 *                        MAWEFDcart2Dcpu.c:297-383; MAWEFDcart3Dcpu.c:295-366)
 *   awe_plan_destroy  <- the cudaFree block (MAWEFDcart2Dgpu.cu:513-527)
 *
 * Conventions: the caller owns every host array; the library owns device
 * state.  Every call returns an awe_status (never exits the process);
 * awe_last_error() describes the last failure on the calling thread.  One
 * plan per host thread at a time.  Arrays are C order with RSF axis 1
 * fastest: a model is [n3][n2][n1] (n3 = 1 in 2D).
 */
#ifndef AWE_H
#define AWE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AWE_ABI_VERSION 1

typedef enum {
    AWE_OK = 0,
    AWE_ERR_INVALID = 1,     /* bad argument or descriptor */
    AWE_ERR_CUDA = 2,        /* CUDA runtime failure */
    AWE_ERR_NOMEM = 3,       /* device or host allocation failed */
    AWE_ERR_UNSUPPORTED = 4, /* combination of options not implemented */
    AWE_ERR_NODEVICE = 5,    /* no usable CUDA device */
    AWE_ERR_STATE = 6        /* call out of order (e.g. forward before set_model) */
} awe_status;

/* Coordinate system of the model axes. */
typedef enum {
    AWE_CART = 0, /* axes (z, x[, y]) - sfAWEFDcart{2D,3D}{gpu,cpu} */
    AWE_SPHER = 1 /* axes (r, theta[, phi]) - sfAWEFDspher2Dgpu (polar), sfAWEFDspher3Dgpu */
} awe_coords;

/* Which reference program's scheme to follow. */
typedef enum {
    /* The GPU programs: 2nd-order Laplacian (cartesian, polar or spherical
     * with metric terms), unscaled bilinear/trilinear injection into the
     * current field before the update, quadratic-alpha sponge on both time
     * levels, the one-way boundary and free-surface masks as those programs
     * apply them. */
    AWE_SCHEME_GPU = 0,
    /* The cartesian CPU programs: 2N-order Laplacian (fdorder 2..20, optional
     * least-squares coefficients, optional variable density), injection into
     * the new field scaled by v^2 dt^2, Gaussian sponge + Clayton-Engquist
     * one-way ABC (dabc=y) or the hybrid ABC (hybridbc=y). */
    AWE_SCHEME_CPU = 1
} awe_scheme;

typedef enum {
    AWE_FAST = 0, /* FP32 with fused multiply-adds */
    AWE_EXACT = 1 /* FP32 in the reference CPU program's operation order and
                     rounding (no contraction; its FP64 leapfrog sum emulated
                     exactly in FP32 arithmetic) */
} awe_precision;

typedef struct {
    int coords;    /* awe_coords */
    int scheme;    /* awe_scheme */
    int ndim;      /* 2 or 3 */
    int n[3];      /* model size per axis (axis 1 fastest); n[2] = 1 in 2D */
    float d[3];    /* spacing */
    float o[3];    /* origin */
    int nb;        /* padding / sponge width (nb=); < 0: the program default */
    int nt;        /* time steps */
    float dt;      /* time step */
    int fdorder;   /* AWE_SCHEME_CPU: spatial order 2N (default 4); GPU: 2 */
    int optfd;     /* AWE_SCHEME_CPU: least-squares optimal coefficients */
    int dabc;      /* AWE_SCHEME_CPU: absorbing boundary */
    int hybrid;    /* AWE_SCHEME_CPU: hybrid one-way ABC */
    int fsrf;      /* free surface (free=) */
    int expl;      /* CPU: one wavelet for all sources; GPU: reflectivity-scaled injection */
    int refl;      /* AWE_SCHEME_GPU, cartesian 2D: injection scaled by an rfl image */
    int jdata;     /* receiver sampling interval (jdata=), default 1 */
    int jsnap;     /* snapshot interval; 0 = no snapshots */
    int bnds;      /* snapshots include the padding (bnds=) */
    int precision; /* awe_precision */
} awe_desc;

/* Derived sizes of a plan. */
typedef struct {
    int npad[3];       /* padded grid per axis (axis 1 fastest) */
    int nbpad;         /* padding actually used */
    int nsmp;          /* trace samples written by awe_forward */
    int nsnap;         /* snapshots written by awe_forward */
    size_t snap_elems; /* floats per snapshot */
    size_t device_bytes; /* device memory held by the plan */
    int step_kernel;     /* 0: register kernels; 1: TMA-staged 3D 8th-order kernel; 2: TMA-staged spherical kernel */
} awe_info;

typedef struct awe_plan awe_plan;

/* Optional per-snapshot callback: frame is a host pointer valid during the call. */
typedef void (*awe_snap_fn)(void *user, int isnap, int it, const float *frame, size_t nelem);

const char *awe_version(void);
const char *awe_last_error(void);
const char *awe_status_string(awe_status s);

awe_status awe_plan_create(const awe_desc *desc, int device, awe_plan **out);
awe_status awe_plan_destroy(awe_plan *plan);
awe_status awe_plan_info(const awe_plan *plan, awe_info *info);

/* vel, den, rfl: host [n3][n2][n1] unpadded; den and rfl may be NULL. */
awe_status awe_set_model(awe_plan *plan, const float *vel, const float *den, const float *rfl);

/* Source and receiver coordinates, host, ndim floats per point in the
 * reference's order: 2D (x, z) [polar: (r, theta)], 3D (x, y, z)
 * [spherical: (r, phi, theta)]. */
awe_status awe_set_geometry(awe_plan *plan, int ns, const float *sou, int nr, const float *rec);

/* Several shots on the plan's grid and model, advanced together (one launch
 * of the step kernel covers every shot's field): the 16-shot track of the
 * spherical-shell survey.  Shot s has ns[s] sources and nr[s] receivers;
 * sou and rec hold all shots' points one shot after the other, in
 * awe_set_geometry's order.  The traces of awe_forward become [nsmp][sum nr]
 * (receivers of shot 0, then of shot 1, ...), every source injecting the same
 * wavelet into its own shot.  Spherical 3D, AWE_SCHEME_GPU, AWE_FAST, no
 * snapshots (nshots = 1 is awe_set_geometry).  Replaces running
 * sfAWEFDspher3Dgpu once per source position. */
awe_status awe_set_shots(awe_plan *plan, int nshots, const int *ns, const float *sou, const int *nr, const float *rec);

/* How a moving geometry's table entry is chosen for point k at step it. */
typedef enum {
    /* entry min(it, rows-1)*n + k: one row of positions per time step (the
     * last row holds after the table ends) - an orbit sampled every step */
    AWE_MOVE_PER_STEP = 0,
    /* entry k*(it+1), as sfDYNAWEFDcart2Dgpu indexes its tables
     * (dyn_cart_kernels.cu:133 inject_sources_2D_dyn, :326 extract_2D_dyn);
     * that program also applies the free surface only with free=y
     * (MDYNAWEFDcart2Dgpu.cu:393-396), which this mode follows.  Cartesian
     * 2D, AWE_SCHEME_GPU only. */
    AWE_MOVE_DYN = 1
} awe_move_mode;

/* Sources and receivers that move during the run (replaces
 * MDYNAWEFDcart2Dgpu.cu:296-344): sou holds ns*nst points and rec nr*nrt
 * points (awe_set_geometry's coordinate order, entry e at e*ndim); at each
 * step ns sources inject and nr receivers record, each from the entry that
 * `mode` selects.  Every entry a run can select must exist (AWE_MOVE_DYN:
 * (n-1)*nt < n*rows).  AWE_SCHEME_GPU plans need expl = 0 (unscaled
 * injection); the misfit gradient is not available on a moving geometry.
 * awe_set_geometry / awe_set_shots return the plan to fixed points. */
awe_status awe_set_moving_geometry(awe_plan *plan, int ns, int nst, const float *sou, int nr, int nrt,
                                   const float *rec, int mode);

/* Host-buffer forward modelling: wav [nt][ncs] (ncs = 1 or ns); dat
 * [nsmp][nr]; wfl (may be NULL) [nsnap][snap_elems].  Snapshots also go to
 * the callback when one is set. */
awe_status awe_forward(awe_plan *plan, const float *wav, int ncs, float *dat, float *wfl);

/* Device-resident variant: d_wav, d_dat (and optional d_wfl) are device
 * pointers; stream is a cudaStream_t (NULL = the plan's own stream).  The
 * call is asynchronous with respect to the host when no snapshot callback is
 * set. */
awe_status awe_forward_device(awe_plan *plan, const float *d_wav, int ncs, float *d_dat, float *d_wfl,
                              void *stream);

awe_status awe_set_snapshot_callback(awe_plan *plan, awe_snap_fn fn, void *user);

/* Waits for the plan's stream. */
awe_status awe_synchronize(awe_plan *plan);

/* Number of kernel launches issued by the last awe_forward / awe_forward_device. */
long long awe_last_launch_count(const awe_plan *plan);

/* Kernel timing: when enabled, the next runs bracket every launch of the
 * stencil (step) kernel - forward steps, and the gradient's recompute steps -
 * and of the adjoint step kernel of a gradient with CUDA events on their
 * stream; awe_profile_read returns the step kernels' summed duration (ms) and
 * launch count after the runs have completed, awe_profile_read_kinds both
 * kinds (arrays of AWE_PROF_KINDS, indexed by AWE_PROF_STEP and
 * AWE_PROF_ADJOINT).  Reading resets the record.  Off by default. */
#define AWE_PROF_STEP 0
#define AWE_PROF_ADJOINT 1
#define AWE_PROF_KINDS 2
awe_status awe_profile_enable(awe_plan *plan, int on);
awe_status awe_profile_read(awe_plan *plan, double *step_kernel_ms, long long *step_launches);
awe_status awe_profile_read_kinds(awe_plan *plan, double *kernel_ms, long long *launches);

/* ---- Misfit gradient (no counterpart in the reference: its adj=y mode
 * back-injects data for an image, MAWEFDcart2Dgpu.cu:386-396) ---- */
/* Checkpoint storage: BF16 or FP16 with one FP32 scale (the level's max |v|)
 * per stored level, FP32 copies, or block floating point (BFP16: 16-bit
 * integers with one FP32 scale per 64 consecutive cells, 2.06 bytes per
 * cell, error at most 1/65534 of the block's largest value; the default when
 * no options are given).  The recomputed levels inherit the rounding:
 * measured gradient error against an FP64 adjoint on the test cases ~1e-2
 * (BF16), ~1e-3 (FP16), ~1e-4 (BFP16), ~1e-7 (FP32). */
typedef enum { AWE_CKPT_BF16 = 0, AWE_CKPT_FP32 = 1, AWE_CKPT_FP16 = 2, AWE_CKPT_BFP16 = 3 } awe_ckpt_format;

typedef struct {
    int ckpt_every;  /* forward steps between checkpoints; <= 0: ceil(sqrt(nt)) */
    int ckpt_format; /* awe_ckpt_format */
} awe_grad_opts;

/* Gradient of J = 0.5 * sum over data rows of ||d - dobs||^2 with respect to
 * m = 1/v^2 on the model grid, for the plan's model and geometry.  Scheme
 * AWE_SCHEME_CPU (2D or 3D, any order, sponge and one-way ABC, free surface),
 * no density, no hybrid ABC; or the spherical 3D AWE_SCHEME_GPU scheme of
 * sfAWEFDspher3Dgpu (sponge, free surface; expl=n, fixed points; the shots
 * of awe_set_shots run one after the other on one set of checkpoint
 * buffers, dobs holding every shot's receivers as awe_forward writes them,
 * gradients and misfits summed).
 * The forward runs in AWE_FAST arithmetic.  The
 * boundary coefficients (one-way ABC, sponge) are held at the plan's model.
 * The forward pass stores both time levels every ckpt_every steps (in
 * opts->ckpt_format); the adjoint sweep recomputes each segment once from
 * its checkpoint.  The gradient is summed over time steps per padded cell as
 * a compensated (Kahan) FP32 pair and folded onto the model in FP64; the
 * misfit sum is FP64.
 * wav as awe_forward; dobs [nsmp][nr]; grad [n3][n2][n1]; misfit: J;
 * dsyn (may be NULL): the synthetic data [nsmp][nr].  opts NULL = defaults
 * (BFP16, ceil(sqrt(nt))). */
awe_status awe_gradient(awe_plan *plan, const float *wav, int ncs, const float *dobs, const awe_grad_opts *opts,
                        double *grad, double *misfit, float *dsyn);

/* The same on device buffers (d_grad double [n3][n2][n1]); misfit is a host
 * pointer, written when the call returns (the call synchronizes `stream`). */
awe_status awe_gradient_device(awe_plan *plan, const float *d_wav, int ncs, const float *d_dobs,
                               const awe_grad_opts *opts, double *d_grad, double *misfit, float *d_dsyn, void *stream);

/* ---- Reverse-time migration on the exact adjoint (replaces the reference
 * recipes that image by correlating a source wavefield with a receiver
 * wavefield, cicmig / awertm2d in byrne_awe.py:428-476, :628-652, and the
 * programs' adj=y back-injection image, MAWEFDcart2Dcpu.c:353-369).  The
 * receiver wavefield is the discrete adjoint of the plan's forward driven by
 * the recorded data; the source wavefield is recomputed from checkpoints as
 * in awe_gradient, so no wavefield is ever written out. */
typedef enum {
    /* image(x) = sum over steps k of nu_k(x) V_k(x): zero-lag cross-correlation
     * of the adjoint (receiver) and forward (source) wavefields, model cells */
    AWE_IMAGE_XCORR = 0,
    /* the Born adjoint of the data: awe_gradient's formula with the residual
     * replaced by the data (dJ/dm for zero synthetics, sign flipped) */
    AWE_IMAGE_BORN = 1
} awe_image_condition;

/* Same plans, options and arguments as awe_gradient; data [nsmp][nr] are
 * the recorded traces; image [n3][n2][n1] in FP64. */
awe_status awe_rtm(awe_plan *plan, const float *wav, int ncs, const float *data, const awe_grad_opts *opts,
                   int condition, double *image);
awe_status awe_rtm_device(awe_plan *plan, const float *d_wav, int ncs, const float *d_data, const awe_grad_opts *opts,
                          int condition, double *d_image, void *stream);

/* ---- Point-cloud windowing and merging (CODE/Mbycloudwin3d.c,
 * CODE/Mbycloudmerge3d.c with CODE/hash.c): the selection of the ground
 * points an orbit stretch illuminates, which cuts a survey into the windows
 * that are modelled, and the fold-normalised sum of the windows' data back
 * onto the full cloud.  A cloud point is AWE_CLOUD_NCO floats: x, y, z, the
 * surface normal, and three more carried along.  Host buffers; device
 * memory is allocated for the call. ---- */
#define AWE_CLOUD_NCO 9

/* Keeps, in input order, the ground points [ng][9] whose aperture cone
 * (half-angle apt degrees about the normal, both sides) contains at least
 * one orbit point (x, y, z of orbit [no][9]); the test is the reference's
 * isInCone in the same float operations.  Writes *nw and index [nw] (input
 * positions; capacity ng), win [nw][9] when win is not NULL (capacity
 * ng*9), and for nf > 0 the data columns: data [nf][ng] -> win_data
 * [nf][nw], ncomp floats per sample (2: complex, as the reference's data;
 * 1: real).  Replaces Mbycloudwin3d.c:108-246 (fast=y). */
awe_status awe_cloud_window(int device, const float *ground, long long ng, const float *orbit, long long no,
                            float apt, long long nf, int ncomp, const float *data, long long *nw, long long *index,
                            float *win, float *win_data);

/* Sums windows' data onto the full cloud all [na][9]: window c holds
 * nwp[c] points (win_pts: the windows' [nwp[c]][9] one after the other) and
 * the data [nf][nwp[c]] (win_data: the windows' blocks one after the other,
 * ncomp floats per sample).  Each window point goes to the full-cloud point
 * that the reference's hash lookup finds (within ddMIN/10, ddMIN the
 * smallest spacing of consecutive full-cloud points; table of
 * hashscale*na slots, default 2), windows added in order; with norm, each
 * full-cloud sample is divided by the number of windows that held the point
 * (at least 1).  out [nf][na] (ncomp floats per sample).  A window point
 * without a match is an error (the reference indexes out of its array).
 * Replaces Mbycloudmerge3d.c:119-300. */
awe_status awe_cloud_merge(int device, const float *all, long long na, int nwin, const long long *nwp,
                           const float *win_pts, const float *win_data, long long nf, int ncomp, int norm,
                           float hashscale, float *out);

/* ---- Batched 2D forward: many shots along a track, each on its own window
 * of one model.  Replaces a loop of sfAWEFDcart2Dcpu runs over cropped
 * windows (the per-shot recipes of byrne_awe.py); the scheme is the CPU
 * programs' (AWE_SCHEME_CPU, AWE_FAST, no hybrid ABC, no snapshots).  All
 * shots advance together: one launch per time step covers every shot's
 * tiles and receivers, and the nt launches run as one captured CUDA graph.
 * Traces are exactly what per-shot awe_forward runs on the same windows
 * return, within FP32 rounding of the fused update. ---- */
typedef struct {
    int x0, nx;       /* window: model columns [x0, x0 + nx) of axis 2 */
    int ns, nr;       /* points of this shot */
    const float *sou; /* [ns][2] (x, z) in model coordinates */
    const float *rec; /* [nr][2] */
} awe_shot;

typedef struct awe_batch awe_batch;

typedef struct {
    int nshots, nsmp;
    long long total_samples; /* sum over shots of nsmp * nr */
    long long cells;         /* padded cells of all shots */
    int tile_z, tile_x, grid; /* forward kernel: tile, or (n1, columns per item) of the column march */
    int work_items;           /* (shot, tile or column chunk) + (shot, receiver block) items per launch */
    int launches_per_forward; /* = nt */
} awe_batch_info_t;

/* desc: the whole model (n[0] = nz, n[1] = model columns), nb, fdorder,
 * dabc, fsrf, jdata, nt, dt; nz + 2 nb must be a multiple of 4. */
awe_status awe_batch_create(const awe_desc *desc, int nshots, const awe_shot *shots, int device, awe_batch **out);
awe_status awe_batch_destroy(awe_batch *batch);
/* vel: host [n2][n1], the whole model; each shot takes its window. */
awe_status awe_batch_set_model(awe_batch *batch, const float *vel);
/* wav: [nt], one wavelet for every source.  dat: the shots' traces one
 * after the other, shot s as [nsmp][nr_s]. */
awe_status awe_batch_forward(awe_batch *batch, const float *wav, float *dat);
awe_status awe_batch_forward_device(awe_batch *batch, const float *d_wav, float *d_dat, void *stream);
/* Autotuner: times `steps` time steps of every tile shape and grid size,
 * and of the column-march kernel (8th order: whole columns streamed by bulk
 * copies, chunks of 16/32/64 columns) on the current model and keeps the
 * fastest for the forward (the next forward recaptures); the gradient keeps
 * the fastest tile shape.  tile_out: the tile index, or 4 for the column
 * march; grid_out: the forward's grid. */
awe_status awe_batch_tune(awe_batch *batch, int steps, int *tile_out, int *grid_out);
awe_status awe_batch_info(const awe_batch *batch, awe_batch_info_t *info);
/* Picks the forward kernel without timing: kernel 0-3 = the tile shapes,
 * 4 = the column march with `chunk` columns per item (8th order only);
 * grid <= 0 = the default (4 CTAs per SM for tiles, every resident CTA for
 * the column march). */
awe_status awe_batch_select(awe_batch *batch, int kernel, int chunk, int grid);
/* Misfit gradient of the whole batch: J = 0.5 sum over shots and samples of
 * (d - dobs)^2, dJ/dm (m = 1/v^2) on the whole model [n2][n1] (each shot's
 * window contributes), with the checkpointing of awe_gradient per shot (one
 * FP32 scale per shot and stored level).  dobs laid out as awe_batch_forward's
 * traces. */
awe_status awe_batch_gradient(awe_batch *batch, const float *wav, const float *dobs, const awe_grad_opts *opts,
                              double *grad, double *misfit);

/* 2D forward modelling without any device allocation.  No counterpart in
 * the reference (its programs cudaMalloc everything in main()).  For callers
 * that cannot call cudaMalloc - code inside a framework that owns the device
 * memory pool, code captured into a larger CUDA graph, plug-ins that must not
 * grow the device footprint at run time.  The caller passes device buffers
 * for the inputs and output only: d_vel [n2][n1] (unpadded), d_wav [nt][ncs],
 * d_sou [ns][2] and d_rec [nr][2] as (x, z) pairs, d_dat [nsmp][nr].  The
 * wavefields, padded model, sponge tables and interpolation points live in
 * one static device array of about 12.2 MiB that every GPU loading the
 * library holds until exit.  Limits: padded n1*n2 <= 1048576, each padded
 * axis <= 8192, nb <= 256, ns + nr <= 4096; larger requests return
 * AWE_ERR_INVALID with the limit in awe_last_error().  Scheme
 * AWE_SCHEME_CPU, cartesian, no hybrid ABC, no density, no snapshots; the
 * result equals awe_forward's for the same descriptor.  The work is queued on
 * `stream` (a cudaStream_t; NULL = legacy default stream) and is complete when
 * the stream is.  A call outside stream capture looks up the array's device
 * address (cudaGetSymbolAddress) with the device current, so a device reset
 * in between is followed; a call during capture reuses the address of the
 * last call outside capture on that device, so make one call before the
 * first capture and after any device reset.  All calls share the array: each call clears
 * what must start at zero, and calls whose work overlaps on the GPU race. */
awe_status awe_forward2d_noalloc(const awe_desc *desc, const float *d_vel, const float *d_wav, int ncs, int ns,
                                 const float *d_sou, int nr, const float *d_rec, float *d_dat, void *stream);

#ifdef __cplusplus
}
#endif
#endif
