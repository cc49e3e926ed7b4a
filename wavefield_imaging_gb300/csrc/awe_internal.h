// Internal declarations shared by the engine's translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "awe.h"

namespace awe {

constexpr int kMaxNop = 10;  // fdorder <= 20, as the reference's optfd tables

// Stencil coefficients, passed by value (kernel parameter space = constant bank).
struct Coef {
    float c0;                   // centre weight  (-2 * sum of all c)
    float c[3][kMaxNop + 1];    // second-derivative weights / d^2 per axis (1..nop)
    float b[3][kMaxNop + 1];    // first-derivative weights / d per axis (variable density)
};

// One interpolation point (source or receiver): flat index of the lowest
// corner and the 4 (2D) or 8 (3D) weights in the reference's corner order.
struct GeoPoint {
    long long base;
    float w[8];
};

// Padded grid, axis 1 fastest.
struct Grid {
    int n1, n2, n3;  // n3 = 1 in 2D
    long long s2() const { return n1; }
    long long s3() const { return (long long)n1 * n2; }
    long long cells() const { return (long long)n1 * n2 * n3; }
};

// ---- scheme of the reference CPU programs (MAWEFDcart{2D,3D}cpu.c) ----
struct StepBParams {
    Grid g;
    Coef k;
    const float *w1, *w2, *w3;  // per-axis sponge factor (1 where undamped); null = no sponge
    int damp_prev;              // prev level carries the sponge of the previous step
    int sponge_new;             // apply the sponge to the new level in the step kernel
    int shell;                  // cells within `shell` of a face are stored raw (boundary pass follows)
    int ilo[3], ihi[3];         // per axis, every sponge factor in [ilo, ihi) is exactly 1
    const float *prv;           // previous level when stepping out of place (null: read nxt in place)
    // 2D only, fused point work: sources added to the new level after its
    // update (k_injectB's arithmetic and order) ...
    const GeoPoint *inj;
    int inj_n, inj_stride, inj_ncs, inj_one, inj_it;
    const float *inj_wav;
    // ... and receivers gathered from `cur` (the level this launch reads,
    // pending sponge applied) by extra blocks after the cell blocks
    const GeoPoint *ext;
    int ext_n, ext_stride;
    float *ext_row;
    // polls allowed to a pipelined kernel's waits for its own copies before it
    // reports a timeout (< 0: the kernel's default); the drain after a timeout
    // always keeps the default
    long long spin;
};

// [lo, hi): the indices of a sponge factor table whose entries are exactly 1
// and that no entry != 1 lies between (the undamped interior of that axis)
void undamped_range(const std::vector<float> &w, int &lo, int &hi);

void launch_stepB(int ndim, int nop, bool exact, bool rho, const float *cur, float *nxt, const float *vel,
                  const float *den, const StepBParams &p, cudaStream_t s);

struct AbcB {
    const float *zl, *zh;  // [n3][n2]
    const float *xl, *xh;  // [n3][n1]
    const float *yl, *yh;  // [n2][n1]
};
// w1 != null (3D): lines at least `band` from the axis-2/3 faces also get the
// sponge of their axis-1 ends in the axis-1 pass (when abc_zfused says the
// fused form applies); launch_band_sponge(..., zfused = 1) then skips them
void launch_abconeB(int ndim, int nop, bool exact, int fsrf, float *uo, const float *um, const AbcB &a,
                    const Grid &g, cudaStream_t s, const float *w1 = nullptr, const float *w2 = nullptr,
                    const float *w3 = nullptr, int band = 0);
bool abc_zfused(int nop, const Grid &g, int band);
void launch_hybridB(int ndim, int nop, int nbd, bool exact, int fsrf, float *uo, const float *um, const AbcB &a,
                    const float *damp, const Grid &g, cudaStream_t s);
void launch_band_sponge(int ndim, int width, bool exact, float *u, const float *w1, const float *w2,
                        const float *w3, const Grid &g, cudaStream_t s, int zfused = 0);

// Model preparation of the CPU-program scheme on the device (k_model.cu):
// padded v^2 dt^2 (free-surface rows zeroed) or a plain padded copy, and the
// one-way ABC coefficient tables, from the model as passed ([n3][n2][n1]).
struct ModelPrep {
    Grid g;                 // padded grid
    int n1, n2, n3, nb, nd;  // model size, padding, dimensions
    float dt, dt2, d1, d2, d3;
    int zero1;              // axis-1 samples set to 0 on every line (free surface), 0: none
};
void launch_model_pad(const float *raw, float *out, const ModelPrep &m, bool vel2, cudaStream_t s);
void launch_model_abc(const float *raw, const ModelPrep &m, float *const abc[6], cudaStream_t s);

// The boundary work of a 3D step in one launch (k_boundary3.cu): one-way ABC
// of the six faces, sponge of the shell the step kernel left unsponged
// (cells within nop + 2 of a face), the receiver gather of the level the step
// read, and the injection (ns > 0; only when no source corner lies in that
// shell, whose cells the ABC reads).  nop = 4.
struct Bnd3Params {
    Grid g;
    float *uo;        // the new level
    const float *um;  // the level the step read
    const float *vel; // v^2 dt^2 (injection)
    const float *zl, *zh, *xl, *xh, *yl, *yh;  // one-way coefficients
    const float *w1, *w2, *w3;                 // sponge factors (null: no sponge)
    int top;                                   // axis-1 low face (0 with a free surface)
    const GeoPoint *rec;
    int nr, rec_stride;
    float *rec_row;  // null: no gather this step
    const GeoPoint *src;
    int ns, src_stride;
    const float *wav;
    int it, ncs, one_wavelet;
    int n_int, nxr, nzr, rec_blocks;  // set by launch_bnd3
    // compact copies of the line ends ([n3][n2][16]: axis-1 cells 0..7, then
    // n1-8..n1-1) of um (em: written by the previous step's launch; null:
    // read um itself) and of the new level once final (eo; null: none)
    const float *em;
    float *eo;
};
bool bnd3_eligible(int nop, const Grid &g);
void launch_bnd3(bool exact, Bnd3Params p, cudaStream_t s);

// The boundary work before one adjoint step of the 3D gradient in one launch
// (k_boundary3.cu): mu += W kappa on the shell (kappa = 0), the transposed
// one-way ABC of the six faces (mu and kappa updated), and g = I vel2 mu on
// every cell.  nop = 4, bnd3_eligible.
struct Bnd3AdjParams {
    Grid g;
    float *mu, *kap, *gout;
    const float *vel2;
    const float *zl, *zh, *xl, *xh, *yl, *yh;
    const float *w1, *w2, *w3;  // sponge factors of the fold (null: weight 1)
    int top;                    // axis-1 low face (0 with a free surface)
    int n_int, nxr, nzr;        // set by launch_bnd3_adj
};
void launch_bnd3_adj(Bnd3AdjParams p, cudaStream_t s);

// injection into the new level scaled by vel (v^2 dt^2): u += (dd*w)*vel.
// off[c] = flat offset of corner c from the point's base index.
// stride: distance between consecutive points in pts (moving geometries)
void launch_injectB_off(int ndim, bool exact, float *u, const float *vel, const GeoPoint *pts, int ns,
                        const float *wav, int it, int ncs, bool one_wavelet, const long long *off, cudaStream_t s,
                        int stride = 1);

// receiver gather; when w1 != null the sponge factors are applied to each node
// value first (the field carries a pending sponge)
void launch_extract_off(int ndim, bool exact, const float *u, const GeoPoint *pts, int nr, float *dat_row,
                        const float *w1, const float *w2, const float *w3, const Grid &g, const long long *off,
                        cudaStream_t s, int stride = 1);

// copy a window (or the whole padded grid) of u into dst, applying pending sponge
void launch_snapshot(int ndim, const float *u, float *dst, const Grid &g, int f1, int f2, int f3, int m1, int m2,
                     int m3, const float *w1, const float *w2, const float *w3, cudaStream_t s);

// ---- scheme of the reference GPU programs (MAWEFD{cart,spher}{2D,3D}gpu.cu) ----
struct StepAParams {
    Grid g;
    int geom;        // 0 cart 2D, 1 cart 3D, 2 polar 2D, 3 spherical 3D
    int nd;          // 2 or 3
    int nb;          // sponge width
    int pri[3];      // sponge priority over memory axes (the kernel's x, y, z)
    int mask;        // 0 none, 1 cart 2D x band, 2 cart 3D z < nb, 3 r band (polar/spherical)
    int spill;       // samples of the next line zeroed by the free-surface grid rounding
    int shell, shell_axes;  // boundary shell width and the axes it spans (bit a = axis a+1)
    float dt2;
    float dd1, dd2, dd3, dd4, dd5;  // divisors of the Laplacian terms
    float rd[5];                    // their reciprocals (AWE_FAST)
    float a0;                       // polar centre weight -2/dra^2
    const float *tr0, *tr1, *tr2, *tr3;  // per-radius tables
    const float *tt0, *tt1;              // per-(theta, r) tables (spherical)
    const double *dtab;                  // sponge factor by index (FP64, as the reference)
    const float *ftab;                   // the same rounded to float (FAST mode)
    float b2lo, b2hi;                    // 2D one-way coefficients at the last sample
    const float *tb[6];                  // cart 3D one-way coefficient tables
    int nshot;                           // shots advanced together (spherical 3D, AWE_FAST), fields back to back
    long long shot_cells;                // cells of one shot's field
};
// out of place (the spherical AWE_FAST march kernels): prv the previous level, out the new one
bool stepA_out_of_place(int geom, bool exact);
void launch_stepA_oop(int geom, bool exact, const float *cur, const float *prv, float *out, const float *vel,
                      const StepAParams &p, cudaStream_t s);
void launch_stepA(int geom, bool exact, const float *cur, float *nxt, const float *vel, const StepAParams &p,
                  cudaStream_t s);
void launch_bcA(bool exact, const float *um, float *uo, float *aux, const StepAParams &p, cudaStream_t s);
// adjoint of the spherical step (AWE_FAST): Y <- W M (L^T(I c X) + 2 X - W Y),
// G += X L(A) on the interior (xcorr: G += X A; A null: none); receivers z += W M (w r)
void launch_adjA_sph(const float *X, float *Y, const float *A, const float *vel, float2 *G, const StepAParams &p,
                     cudaStream_t s, bool xcorr = false);
void launch_rec_adjA(float *z, const GeoPoint *pts, int nr, const float *r, const StepAParams &p, const long long *off,
                     cudaStream_t s);
// wav [nt][ncs]: ncs = 1 (one wavelet for every source) or ns
void launch_injectA(bool exact, int ndim, float *u, const GeoPoint *pts, const float *scale, int ns, const float *wav,
                    int it, bool scaled, const long long *off, cudaStream_t s, int stride = 1, int ncs = 1);
void launch_snapshot_transpose2(const float *u, float *dst, const Grid &g, int f1, int f2, int m1, int m2,
                                cudaStream_t s);

// ---- adjoint of the CPU-program scheme (k_adjoint.cu) ----
struct AdjParams {
    Grid g;
    Coef k;
    int nd, nop;
    const float *w1, *w2, *w3;  // sponge axis factors; null = no sponge
    int xcorr;                  // imaging condition: G += I nu V (cross-correlation) instead of I nu L(V)
    // point terms fused into the step (null: none), per padded cell i the
    // entries [start[i], start[i + 1]) as (point index, weight bits):
    // receivers mu += W (W (w r[point])) with r = rrow; sources G += nu (wav w)
    const int *rc_start, *sc_start;
    const int2 *rc_ent, *sc_ent;
    const float *rrow;     // this step's residual row (null: no receiver term this step)
    const float *wav;      // wavelet (null: no source term)
    int it, ncs, one_wavelet;
};
void launch_adjB(const float *X, float *Y, const float *V, const float *vel, float2 *G, const AdjParams &p,
                 cudaStream_t s);
void launch_abc_adjB(int nop, int fsrf, float *mu, float *kap, const AbcB &a, const Grid &g, cudaStream_t s);
void launch_kap_fold(float *mu, float *kap, const AdjParams &p, cudaStream_t s);
void launch_rec_adj(float *mu, const GeoPoint *pts, int nr, const float *r, const AdjParams &p, const long long *off,
                    cudaStream_t s);
void launch_src_grad(float2 *G, const float *nu, const GeoPoint *pts, int ns, const float *wav, int it, int ncs,
                     bool one_wavelet, int nd, const long long *off, cudaStream_t s);
void launch_residual(const float *d, const float *dobs, float *r, int nrows, int nr, double *row_sum, cudaStream_t s);
void launch_ckpt_store16(bool fp16, const float *u, long long n, unsigned int *amax, void *q, float *scale, int grid,
                         cudaStream_t s);
void launch_ckpt_load16(bool fp16, const void *q, long long n, const float *scale, float *u, int grid,
                        cudaStream_t s);
// block floating point checkpoints: kBfpBlock consecutive cells share one FP32 scale
constexpr int kBfpBlock = 64;
constexpr float kBfpTiny = 1e-30f;  // blocks with max |v| <= this are stored as zero
void launch_ckpt_store_bfp(const float *u, long long n, short *q, float *scale, int grid, cudaStream_t s);
void launch_ckpt_load_bfp(const short *q, const float *scale, long long n, float *u, int grid, cudaStream_t s);
// image on the model grid: the padded grid's model window of G
void launch_add_f64(double *dst, const double *src, long long n, cudaStream_t s);
void launch_image_cut(const float2 *G, const Grid &g, int nb, const int *n, int nd, double *out, cudaStream_t s);
// vel2: v^2 dt^2 per padded cell, or the velocity itself (raw_v: c = dt^2 v^2)
void launch_grad_fold(const float2 *G, const float *vel2, float dt, const Grid &g, int nb, const int *n, int nd,
                      double *out, cudaStream_t s, bool raw_v = false);

// ---- batched 2D forward (k_batch2d.cu) ----
struct BatchShot {
    long long off;      // first cell of the shot's padded grid in the concatenated fields
    int n2;             // padded columns
    int wx_off;         // first entry of its axis-2 sponge table
    int ns, src0;       // sources: count, first index in the point table
    int nr, rec0;       // receivers
    long long dat_off;  // first sample of its traces [nsmp][nr]
};
struct BatchStep {
    const float *cur;
    float *nxt;
    const float *vel;
    const float *wz, *wx;  // sponge tables (axis 1 common, axis 2 per shot)
    int sponge;
    int n1;  // padded rows (axis 1), common
    float c0, cz[kMaxNop + 1], cx[kMaxNop + 1];
    const GeoPoint *src, *rec;
    const float *wav;  // one wavelet, [nt]
    int it;
    float *dat;
    int row;            // trace row written by this step, -1: none
    const float *prv;   // previous level when stepping out of place (null: in place in nxt)
};
// a padded cell that receivers inject adjoint residuals into, with its
// receiver corners [e0, e1) in (receiver, corner) order
struct BatchRecCell {
    long long gi;  // cell of the concatenated padded grids
    int shot, x, z, e0, e1, pad;
};
struct BatchRecW {
    int r;    // receiver index within the shot
    float w;  // interpolation weight
};
struct BatchAdj {
    const float *X;  // nu_k
    float *Y;        // nu_{k+1} in, mu_k out
    const float *V;  // forward level V_k
    const float *vel;
    float2 *G;  // dJ/dvel2 accumulators (compensated pairs), per shot, padded grids
    const float *wz, *wx;
    int sponge, n1;
    float c0, cz[kMaxNop + 1], cx[kMaxNop + 1];
    const GeoPoint *src;
    const float *wav;
    int it;
    const float *res;  // residuals, laid out as the traces
    int row;           // residual row of this step, -1: none
};
void launch_batch2d_adj(int nop, int tile, const BatchShot *shots, const int4 *items, int nitems, int grid,
                        const BatchAdj &p, cudaStream_t s);
void launch_batch_ckpt(bool store, int fmt, const BatchShot *shots, int nshots, float *u, void *q, float *scales,
                       int n1, long long cells, cudaStream_t s);
void launch_residual_flat(const float *d, const float *dobs, float *r, long long n, double *part, cudaStream_t s);
void launch_batch_grad_fold(const BatchShot *shots, const int2 *win, int nshots, const float2 *G, const float *vel2,
                            float dt, int n1, int nb, int nz, int nxm, double *out, cudaStream_t s);
// column-march forward (k_batch2d_col.cu): 8th order, n1 % 4 == 0, n1 <= 2048;
// returns the threads per CTA (0 if the shape is not covered) and the dynamic shared memory
int batch2d_col_shape(int nop, int n1, size_t *smem);
int batch2d_col_ctas_per_sm(int n1);
void launch_batch2d_col(const BatchShot *shots, const int4 *items, int nitems, int grid, int L, const BatchStep &p,
                        int *err, cudaStream_t s);
// adjoint step as a column march (same arithmetic as k_batch2d_adj)
int batch2d_col_adj_ctas_per_sm(int n1);
void launch_batch2d_col_adj(const BatchShot *shots, const int4 *items, int nitems, int grid, int L,
                            const BatchAdj &p, int *err, cudaStream_t s);
// the adjoint step's receiver term W R^T r on mu (p.Y), after either adjoint
// kernel: one thread per receiver cell, its corners in order
void launch_batch_rec_adj(const BatchRecCell *cells, int ncells, const BatchRecW *ws, const BatchShot *shots,
                          const BatchAdj &p, cudaStream_t s);
constexpr int kBatchNumTiles = 4;
constexpr int kBatchRecBlock = 128;  // receivers per receiver item (<= threads of every tile shape)
extern const int kBatchTiles[kBatchNumTiles][2];
void launch_batch2d(int nop, int tile, const BatchShot *shots, const int4 *items, int nitems, int grid,
                    const BatchStep &p, cudaStream_t s);

// ---- host-side math (bit-identical to the reference's float evaluation) ----
void fd_coefficients(int nop, int ndim, const float *dd, int optfd, Coef &k);
void sponge_weights(int nb, std::vector<float> &w);   // fdutil.c sponge_make
void hybrid_damp(int ntransit, std::vector<float> &w);  // MAWEFDcart*cpu.c damp_make
// fdutil.c lint2d_make / lint3d_make for one point, in the reference's fdm
// axes (z, x, y): origin of the padded grid, spacing, padded size.
struct FdmAxes {
    float oz, ox, oy, dz, dx, dy;
    int nz, nx, ny;
};
struct Lint {
    int jz, jx, jy;
    float w[8];
};
Lint lint_make(int ndim, float x, float y, float z, const FdmAxes &f);
void expand_model(int ndim, const float *a, float *b, int nb, const int *n);

void set_error(const char *fmt, ...);
// the descriptor checks of awe_plan_create (sizes, spacing, time axis,
// scheme, order, intervals, precision)
awe_status check_desc(const awe_desc *d);

// ---- TMA-staged 3D 8th-order step (k_stepB3_tma.cu) ----
struct Step3Launch {
    int grid, L, ntz, ntx, nchunks, items;
    size_t smem;
};
bool stepB3_tma_eligible(int ndim, int nop, bool rho, const Grid &g);
bool stepB3_tma_maps(CUtensorMap *maps, float *const u[2], const float *vel, const Grid &g);
Step3Launch stepB3_tma_shape(const Grid &g, int num_sms, int L);
cudaError_t launch_stepB3_tma(bool exact, const CUtensorMap *maps, int icur, float *nxt, const StepBParams &sp,
                              const Step3Launch &sh, unsigned long long *counter, unsigned long long base, int *err,
                              cudaStream_t s);
// lap_out (AWE_FAST only, may be null): also store L(cur) of interior cells
cudaError_t launch_stepB3_tma_with(bool exact, const CUtensorMap &cur, const CUtensorMap &prv, const CUtensorMap &vel,
                                   float *nxt, const StepBParams &sp, const Step3Launch &sh,
                                   unsigned long long *counter, unsigned long long base, int *err, cudaStream_t s,
                                   float *lap_out);
cudaError_t launch_stepB3_adj(const CUtensorMap &g_halo, const CUtensorMap &y_tile, const CUtensorMap &x_tile,
                              float *Y, const float *lap_v, float2 *grad, const StepBParams &sp,
                              const Step3Launch &sh, unsigned long long *counter, unsigned long long base, int *err,
                              cudaStream_t s);
// g = I vel2 nu (cells at least nop from every face), elementwise
void launch_adj_g(const float *nu, const float *vel2, float *g, const Grid &gr, int nop, cudaStream_t s);
bool make_tmap_3d(CUtensorMap *m, const float *base, int n1, int n2, int n3, int b1, int b2);
// tensor-map boxes of the TMA step: the current level's halo box and the tile box
void stepB3_tma_boxes(int *halo1, int *halo2, int *tile1, int *tile2);

// TMA-staged spherical step (GPU-program scheme, AWE_FAST); Step3Launch's
// ntz/ntx count the r and theta tiles, items include the shots
bool sphA_tma_eligible(const Grid &g, int nb);
// maps: [0] u[0] halo box, [1] u[1] halo box, [2] u[0] tile, [3] u[1] tile, [4] vel tile
bool sphA_tma_maps(CUtensorMap *maps, float *const u[2], const float *vel, const Grid &g, int nshot);
Step3Launch sphA_tma_shape(const Grid &g, int nshot, int num_sms, int L);
// cur_f0, prv_f0: plane offsets of the two levels in their maps (levels
// stacked along phi, as the gradient's recompute slots); nxt: the new level
cudaError_t launch_stepA_sph_tma(const CUtensorMap &cur, const CUtensorMap &prv, const CUtensorMap &vel, float *nxt,
                                 const StepAParams &pa, const Step3Launch &sh, unsigned long long *counter,
                                 unsigned long long base, int *err, long long spin, cudaStream_t s, int cur_f0 = 0,
                                 int prv_f0 = 0);
// adjoint step of the spherical scheme (the k_adjA_sph2 update, TMA-staged):
// x_halo / v_halo / a_halo = 72 x 18 box maps of z_{j+1}, the velocity and the
// forward levels (A_j at plane offset a_f0); y_tile / g_tile = tile maps of
// Y (z_{j+2} in, z_j out) and of G (the gradient or image accumulators,
// sphA_tma_pair_map)
// halo-box (72 x 18) and, when tile is not null, tile-box (64 x 16) maps of
// nlevels fields stacked along phi from base
bool sphA_tma_level_maps(CUtensorMap *halo, CUtensorMap *tile, const float *base, const Grid &g, int nlevels);
bool sphA_tma_pair_map(CUtensorMap *m, const float2 *base, const Grid &g);
cudaError_t launch_adjA_sph_tma(const CUtensorMap &x_halo, const CUtensorMap &v_halo, const CUtensorMap &a_halo,
                                int a_f0, const CUtensorMap &y_tile, const CUtensorMap &g_tile, float *Y, float2 *G,
                                const StepAParams &pa, const Step3Launch &sh, unsigned long long *counter,
                                unsigned long long base, int *err, long long spin, bool xcorr, cudaStream_t s);

}  // namespace awe
