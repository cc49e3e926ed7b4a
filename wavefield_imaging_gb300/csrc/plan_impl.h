// The plan object behind the opaque awe_plan handle.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <utility>
#include <vector>

#include "awe_internal.h"

namespace awe {
struct GradState;
}

struct awe_plan {
    awe_desc d{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<std::pair<void *, size_t>> allocs;  // device allocations owned by the plan
    size_t device_bytes = 0;

    // grid
    int ndim = 2, nop = 1, nbd = 0;
    awe::Grid g{};          // padded, axis 1 fastest
    float opad[3] = {0, 0, 0};  // padded origin per axis
    awe::Coef k{};
    int nsmp = 0, nsnap = 0;
    size_t snap_elems = 0;
    int snap_f[3] = {0, 0, 0}, snap_m[3] = {1, 1, 1};  // snapshot window in padded indices

    // fields and model (device)
    float *u[2] = {nullptr, nullptr};
    float *vel = nullptr;  // scheme CPU: v^2 dt^2; scheme GPU: v
    float *den = nullptr;
    float *rfl = nullptr;
    float *w[3] = {nullptr, nullptr, nullptr};  // per-axis sponge factors
    int wlo[3] = {0, 0, 0}, whi[3] = {0, 0, 0};  // undamped range of each factor table
    float *abc[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    float *damp = nullptr;
    std::vector<float> h_vel_raw;  // padded raw velocity (scheme GPU injection reflectivity, ABC tables)

    // geometry
    int ns = 0, nr = 0;
    std::vector<int> shot_ns, shot_nr;  // points per shot (awe_set_shots; one shot: {ns}, {nr})
    awe::GeoPoint *src = nullptr, *rec = nullptr;
    long long *corner_off = nullptr;  // device [8]
    long long h_corner_off[8] = {0};
    std::vector<awe::GeoPoint> h_src, h_rec;
    std::vector<awe::Lint> h_src_lint;  // source corner indices in the reference's fdm axes
    bool sponge_deferred = false;  // a source node lies in the sponge band outside the boundary shell
    bool src_in_shell = false;     // a source node lies within nop + 2 of a face (3D)
    int src_cap = 0, rec_cap = 0;  // points the src / rec device buffers hold
    // moving geometry (awe_set_moving_geometry): src/rec hold ns*src_rows and
    // nr*rec_rows entries; move_mode < 0 = fixed points
    int move_mode = -1, src_rows = 1, rec_rows = 1;

    // scheme-GPU specific
    float *aux = nullptr;              // boundary values (phase 1 -> phase 2)
    awe::StepAParams pa{};             // step / boundary parameters
    std::vector<float> h_rfl_pad;      // padded reflectivity image (cart 2D refl=y)
    float *inj_scale = nullptr;        // per source corner injection scale
    int snap_transpose = 0;            // polar snapshots are theta-fastest

    bool model_set = false, geom_set = false;
    awe_snap_fn snap_cb = nullptr;
    void *snap_user = nullptr;
    float *snap_host[2] = {nullptr, nullptr};  // pinned frame buffers (double-buffered delivery)
    size_t snap_host_bytes = 0;
    cudaEvent_t snap_ev[2] = {nullptr, nullptr};
    int snap_pending = -1, snap_pending_isnap = 0, snap_pending_it = 0;
    float *d_snap_tmp = nullptr;
    long long launches = 0;

    // TMA-staged 3D step (scheme CPU, 8th order)
    bool use_tma = false;
    CUtensorMap tmaps[5];
    awe::Step3Launch tma_shape{};
    unsigned long long *sched_counter = nullptr;
    unsigned long long sched_base = 0;
    int *d_err = nullptr;
    // compact copies of the axis-1 line ends of the last two levels (3D
    // boundary launch, [n3][n2][16] each): inside a forward run (ends_run) the
    // boundary launch of step it reads the ends of its step's current level
    // from ends[ends_idx] and writes those of the new level to the other one
    float *ends[2] = {nullptr, nullptr};
    bool ends_run = false;
    int ends_idx = 0;
    // TMA-staged spherical step (GPU-program scheme, AWE_FAST): maps encoded
    // per run (the level fields are reallocated when the shot count changes)
    bool sph_tma = false;
    int num_sms = 0;
    CUtensorMap sph_maps[5];
    awe::Step3Launch sph_shape{};
    // polls of a pipeline wait before it reports a timeout (AWE_PIPELINE_SPIN_LIMIT;
    // < 0: the kernel default); a limit of 0 makes every first wait time out,
    // which the failure tests use to exercise the error path
    long long spin_limit = -1;

    // the forward time loop captured as a CUDA graph (CPU-program scheme, no
    // snapshots, no profiling), replayed while its device pointers stay the same
    cudaGraphExec_t gexec = nullptr;
    const float *g_wav = nullptr;
    float *g_dat = nullptr;
    int g_ncs = 0;
    long long g_launches = 0;
    float *stage_wav = nullptr, *stage_dat = nullptr;  // awe_forward's device staging buffers
    size_t stage_wav_bytes = 0, stage_dat_bytes = 0;
    float *stage_dsyn = nullptr;  // awe_gradient / awe_rtm staging (with stage_wav, stage_dat)
    double *stage_grad = nullptr;
    size_t stage_dsyn_bytes = 0, stage_grad_bytes = 0;

    // misfit gradient state (allocated by the first awe_gradient call)
    awe::GradState *grad = nullptr;

    // optional per-launch timing of the step kernel
    bool profile = false;
    std::vector<cudaEvent_t> prof_ev;  // pairs (start, stop)
    std::vector<int> prof_kind;         // AWE_PROF_* of each pair
    long long prof_n = 0;
};

namespace awe {
awe_status dev_alloc(awe_plan *p, void **ptr, size_t bytes);
// forget the captured time loop (the model, geometry or buffers it baked in changed)
void plan_graph_drop(awe_plan *p);
void dev_free(awe_plan *p, void *ptr);
awe_status deliver_snapshot(awe_plan *p, const float *d_frame, int isnap, int it, cudaStream_t s);
// hand the last queued frame to the callback (end of a run)
awe_status flush_snapshots(awe_plan *p);

awe_status set_geometry_common(awe_plan *p, int ns, const float *sou, int nr, const float *rec);

// The n points of a table active at step it: the first one and the stride
// between consecutive points (fixed points: the table itself, stride 1).
struct PointsAt {
    const GeoPoint *pts;
    int stride;
};
inline PointsAt points_at(const awe_plan *p, const GeoPoint *tab, int n, int rows, int it) {
    if (p->move_mode == AWE_MOVE_PER_STEP) return {tab + (size_t)(it < rows ? it : rows - 1) * n, 1};
    if (p->move_mode == AWE_MOVE_DYN) return {tab, it + 1};
    return {tab, 1};
}

// bracket one step-kernel launch with events when profiling is on
void prof_begin(awe_plan *p, cudaStream_t s, int kind = AWE_PROF_STEP);
void prof_end(awe_plan *p, cudaStream_t s);

awe_status planB_init(awe_plan *p);
awe_status planB_model(awe_plan *p, const float *vel, const float *den);
awe_status planB_run(awe_plan *p, const float *d_wav, int ncs, float *d_dat, float *d_wfl, cudaStream_t s);
// called at the start of step it with the two levels (prev = V_{it-1} with its
// second sponge pending, cur = V_it)
typedef std::function<awe_status(int it, const float *prev, const float *cur, cudaStream_t s)> StepHook;
awe_status planB_run_hooked(awe_plan *p, const float *d_wav, int ncs, float *d_dat, float *d_wfl, cudaStream_t s,
                            const StepHook *hook);
StepBParams stepB_params(const awe_plan *p);
// lap_out: the TMA path also stores L(cur) of interior cells there (gradient recompute)
// ext_*: 2D, the receivers of `cur` (pending sponge applied) gathered into
// ext_row by the same launch
awe_status stepB_full(awe_plan *p, const StepBParams &sp, const float *prv, const float *cur, float *nxt, int it,
                      const float *d_wav, int ncs, const CUtensorMap *cur_map, const CUtensorMap *prv_map,
                      cudaStream_t s, long long &launches, float *lap_out = nullptr, const GeoPoint *ext_pts = nullptr,
                      int ext_n = 0, int ext_stride = 1, float *ext_row = nullptr);
// 2D steps add the sources in the step kernel (one launch per step) up to this many sources
constexpr int kFusedSources = 8;
// 3D CPU-program scheme with sponge + one-way ABC: the boundary work of a step
// (ABC, shell sponge, receiver gather, injection) is one launch (k_bnd3)
bool stepB3_bnd(const awe_plan *p);
// image < 0: misfit gradient; else awe_image_condition (the residual is the data)
awe_status plan_gradient(awe_plan *p, const float *d_wav, int ncs, const float *d_dobs, const awe_grad_opts &o,
                         double *d_grad, double *misfit, float *d_dsyn, cudaStream_t s, int image = -1);
void plan_gradient_free(awe_plan *p);
// drops the gradient's captured graph and its per-cell point lists
void plan_gradient_graph_drop(awe_plan *p);

awe_status planA_init(awe_plan *p);
awe_status planA_model(awe_plan *p, const float *vel, const float *rfl);
awe_status planA_run(awe_plan *p, const float *d_wav, int ncs, float *d_dat, float *d_wfl, cudaStream_t s,
                     const StepHook *hook = nullptr);
}  // namespace awe
