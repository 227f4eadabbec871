// Host-side internals shared by the engine's translation units: the engine
// object behind fl_engine* and the kernel launchers each .cu file provides.
#pragma once

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/flowlab_gb300.h"
#include "fl_common.cuh"

namespace fl {

// Conversion target of launch_convert: the double-float pressure pairs.
constexpr int DT_DF = 2;
// fl_params.mixed values
constexpr int MIXED_F64 = 1, MIXED_DF = 2;

// One multigrid level (pressureMultigrid.ts:211-217). x is double-buffered so
// the temporally blocked smoother can read the pre-sweep values of its halo
// while neighbouring tiles write their results.
struct Level {
  int nx = 0, ny = 0;
  float* x[2] = {nullptr, nullptr};
  float* b = nullptr;
  uint8_t* label = nullptr;
  uint8_t* code = nullptr;
};

struct Engine {
  int device = 0;
  int nx = 0, ny = 0, dnx = 0, dny = 0, dye_scale = 1;
  float h = 0, dh = 0;
  fl_params prm{};
  cudaStream_t stream = nullptr;
  std::atomic<int> busy{0};
  std::string err;

  // velocity and dye: u[cur]/v[cur]/dye[cur] are the fields; the others are
  // the advection targets
  float* u[2] = {nullptr, nullptr};
  float* v[2] = {nullptr, nullptr};
  float* u_hat = nullptr;
  float* v_hat = nullptr;
  int cur = 0;
  // dye: 3 planes of dnx*dny each
  float* dye[2] = {nullptr, nullptr};
  float* dye_hat = nullptr;

  std::vector<Level> levels;  // levels[0].x[0] is the resident pressure
  int coarse_level = 0;       // first level solved inside the single-CTA kernel
  size_t coarse_smem = 0;

  // float64 pressure of the defect-correction solve (fl_params.mixed):
  // p64[ctl->par] is the pressure, r32 the float residual fed to each V-cycle.
  double* p64[2] = {nullptr, nullptr};
  float* r32 = nullptr;
  // the rounding error of the fine rhs b = (-scale) * div (b + b_lo is the
  // exact product): the defect correction's residual is formed against it,
  // so its tolerance test is on the unrounded rhs
  float* b_lo = nullptr;
  // the previous step's pressure of the second-order warm start
  float* pprev32 = nullptr;
  double* pprev64 = nullptr;
  SolveCtl* ctl = nullptr;       // device
  SolveCtl* ctl_host = nullptr;  // pinned mirror

  // whole-step CUDA graphs, one per velocity/dye buffer parity
  float2* bt_u = nullptr;  // MacCormack backtrace positions (u faces, v faces, dye cells)
  float2* bt_v = nullptr;
  float2* bt_d = nullptr;
  cudaStream_t stream2 = nullptr;  // capture stream of the cycle-loop body; copies of fl_step_host
  // fl_step_host: the dye upload on stream2 (waited for by the step's first
  // dye reader), the projection's end (velocity and pressure final), and
  // the stream's earlier work (before stream2 overwrites an input)
  cudaEvent_t ev_dye = nullptr, ev_proj = nullptr, ev_prior = nullptr;
  // the dye advection's end: fl_step_host reads the dye back from here on,
  // while the step's CFL scan runs
  cudaEvent_t ev_dye_done = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  // the same steps led by the clock reset and the CFL scalars of freshly
  // uploaded velocities (fl_step_host): one graph launch instead of two
  // kernel launches and a graph launch while the dye is still arriving,
  // which delays separately launched kernels (built on first use)
  cudaGraphExec_t graph_up[2] = {nullptr, nullptr};
  // the device-side work of fl_upload_fields after its copies (float32 p)
  cudaGraphExec_t upload_graph = nullptr;
  // fl_step_host's pressure arrives on the second stream (ev_p marks it and
  // its refined copies)
  cudaEvent_t ev_p = nullptr;
  // fl_step_host's label part of the upload (compare, rebuild when changed)
  // runs on a third stream while u and v are still arriving: ev_lab_sync
  // marks the finest labels (the step waits for them before it starts),
  // ev_lab_done the multigrid labels and codes (the step's first reader of
  // the codes waits for them, wait_codes)
  cudaStream_t stream3 = nullptr;
  cudaEvent_t ev_lab = nullptr, ev_lab_sync = nullptr, ev_lab_done = nullptr;
  cudaGraphExec_t upload_graph_labels = nullptr;
  // fl_upload_fields copies the labels here; the upload compares them with
  // levels[0].label and rebuilds the multigrid labels and codes only where
  // they changed (label_flag: set when any cell differs)
  uint8_t* label_in = nullptr;
  int* label_flag = nullptr;
  bool graphs_valid = false;
  // counts every destruction of the step graphs (parameters, patch, warm
  // start or levels changed): a batch rebuilds its own graphs when it moves
  unsigned long long graph_gen = 0;
  bool use_graphs = true;
  bool stats_on_device = false;  // the last solve's statistics live in ctl

  // learned warm start (fl_set_warm_start), run between divergence and solve
  struct Unet* warm = nullptr;
  float* ws_scales = nullptr;  // device: s_b, s_p, 1/s_b, 1/s_p of the last step

  float* w = nullptr;   // vorticity scratch
  float* fx = nullptr;  // confinement force scratch
  float* fy = nullptr;

  float* patch = nullptr;
  int pi0 = 0, pj0 = 0, pnx = 0, pny = 0;
  bool stir_pending = false;
  float stir[5] = {0, 0, 0, 0, 0};

  // the residual diagnostic (fl_params.residual_every): the post-step
  // divergence field and its statistics
  float* div_post = nullptr;
  DiagAccum* diag = nullptr;       // device
  DiagAccum* diag_host = nullptr;  // pinned mirror

  StepScalars* sc = nullptr;   // device
  StepAccum* acc = nullptr;    // device
  StepAccum* acc_host = nullptr;  // pinned mirror
  double* time_dev = nullptr;  // device-accumulated sim time

  // staging for dtype conversion and the per-pass entry points
  void* staging = nullptr;
  // the step's refined pressure rounded to float by the projection (the
  // defect-correction paths), which fl_step_host reads back
  float* p32_final = nullptr;
  size_t staging_bytes = 0;

  bool uploaded = false;
  bool labels_dirty = false;
  bool codes_valid = false;

  // phase profiling (fl_profile_enable / fl_profile_read)
  struct PendingPhase {
    int phase;
    cudaEvent_t a, b;
    double bytes;
    int launches;
  };
  bool profiling = false;
  std::vector<PendingPhase> pending;
  std::vector<cudaEvent_t> event_pool;
  double prof_ms[FL_PHASES] = {};
  double prof_bytes[FL_PHASES] = {};
  long long prof_launches[FL_PHASES] = {};

  // report
  double time = 0;
  int steps = 0;
  int last_iters = 0;
  double last_relres = -1;
  double last_relres0 = -1;
  double last_div_rms = 0;
  double last_dt = 0, last_scale = 0, last_grad_scale = 0;

  long cells() const { return (long)nx * ny; }
  long ufaces() const { return (long)(nx + 1) * ny; }
  long vfaces() const { return (long)nx * (ny + 1); }
  long dye_cells() const { return (long)dnx * dny; }
};

// Phase timing: prof_begin records the start event (returns -1 when
// profiling is off), prof_end the stop event with the phase's algorithmic
// bytes and launch count. Defined in fl_engine.cu.
int prof_begin(Engine& e, int phase);
void prof_end(Engine& e, int token, double bytes, int launches);

// Message for fl_last_error(NULL) (calls that have no engine). Defined in
// fl_engine.cu.
void set_global_error(const char* fmt, ...);

// ------------------------------------------------------------- launchers

// fl_advect.cu
// bt_u / bt_v / bt (optional): room for the MacCormack forward pass's
// backtrace positions, which the correction then reads instead of
// recomputing them (same values).
void launch_advect_velocity(cudaStream_t s, int nx, int ny, float h, int mac, const float* u_in, const float* v_in,
                            float* u_hat, float* v_hat, float* u_out, float* v_out, const uint8_t* label,
                            const StepScalars* sc, float2* bt_u = nullptr, float2* bt_v = nullptr);
void launch_advect_dye(cudaStream_t s, int nx, int ny, float h, int dnx, int dny, float dh, int mac, const float* u,
                       const float* v, const float* q_in, float* q_hat, float* q_out, const uint8_t* label,
                       const StepScalars* sc, bool tail, const float* patch, int pi0, int pj0, int pnx, int pny,
                       float2* bt = nullptr);
// Loads the velocity-advection kernels (so that later launches need no module load).
cudaError_t preload_advect_kernels();

// fl_project.cu
void launch_vorticity(cudaStream_t s, int nx, int ny, float h, const float* u, const float* v, float* w);
// vorticity + confinement force in one pass (the same values as the two launches)
void launch_vort_confine(cudaStream_t s, int nx, int ny, float h, const float* u, const float* v,
                         const uint8_t* label, float eps, float* fx, float* fy);
void launch_confinement_force(cudaStream_t s, int nx, int ny, float h, const float* w, const uint8_t* label,
                              float eps, float* fx, float* fy);
void launch_forces(cudaStream_t s, int nx, int ny, float h, int dnx, int dny, float dh, float* u, float* v,
                   const float* dye, const uint8_t* label, bool beta_on, bool alpha_on, bool conf_on,
                   const float* fx, const float* fy, const StepScalars* sc);
// out_lo (optional): the exact rounding error of each b = (-scale) * div (b + out_lo is the product)
void launch_divergence(cudaStream_t s, int nx, int ny, float h, const float* u, const float* v, float* out,
                       bool as_rhs, const uint8_t* label, const StepScalars* sc, StepAccum* acc,
                       float* out_lo = nullptr);
// The batched pressure solve of fl_batch (fl_multigrid.cu): the plan over
// the engines' buffers, or null with the reason when some engine does not
// qualify; the solve enqueued on a capturing stream (cycle body captured
// from `body`).
struct BatchSolve;
BatchSolve* batch_solve_create(const std::vector<Engine*>& engines, std::string& why);
void batch_solve_destroy(BatchSolve* b);
cudaError_t batch_solve_enqueue(const BatchSolve& b, cudaStream_t s, cudaStream_t body);

// Word fills and copies as kernels (not copy-engine nodes) in the graphs.
void launch_fill32(cudaStream_t s, void* p, long words, uint32_t v);
void launch_copy32(cudaStream_t s, const void* src, void* dst, long words);
// The end-of-step CFL scan with the residual diagnostic folded in (every
// residual_every steps: the post-step divergence and its statistics); the
// step's dt joins the clock and the next step's scalars are written.
void launch_cfl_residual(cudaStream_t s, int nx, int ny, float h, const float* u, const float* v, float* div_out,
                         const uint8_t* label, int every, DiagAccum* d, StepAccum* acc, StepScalars* sc_next,
                         double* time_dev, const fl_params* prm, bool write_scalars, bool add_time);
// p64a/p64b: the refined pressure (float64, or double-float pairs when df)
void launch_subtract_outflow(cudaStream_t s, int nx, int ny, const float* p, float* u, float* v,
                             const uint8_t* label, const StepScalars* sc, bool subtract, bool outflow,
                             const double* p64a = nullptr, const double* p64b = nullptr,
                             const SolveCtl* ctl = nullptr, bool df = false, float* p32_out = nullptr);
void launch_max_speed(cudaStream_t s, int nx, int ny, const float* u, const float* v, StepAccum* acc,
                      StepScalars* sc_next, double* time_dev, const fl_params* prm, float h, bool write_scalars,
                      bool add_time);
// b = (-scale)*div (b may be null: only accumulate div^2) with fluid sums.
void launch_scale_rhs(cudaStream_t s, long n, const float* div, float* b, float neg_scale, const uint8_t* label,
                      StepAccum* acc, float* b_lo = nullptr);
void launch_commit_labels(cudaStream_t s, int nx, int ny, const uint8_t* label, float* p, float* u, float* v,
                          float* dye, long dye_cells, double* p64a = nullptr, double* p64b = nullptr,
                          const SolveCtl* ctl = nullptr);
void launch_stir(cudaStream_t s, int nx, int ny, float h, float* u, float* v, const uint8_t* label,
                 const float* stir5);
void launch_dye_patch(cudaStream_t s, int dnx, int dny, float* dye, const float* patch, int pi0, int pj0, int pnx,
                      int pny);
void launch_hold(cudaStream_t s);
void launch_select_p64(cudaStream_t s, const SolveCtl* ctl, const double* p64a, const double* p64b, void* out,
                       bool as_f64, long n, bool df);
void launch_extrapolate(cudaStream_t s, long n, const uint8_t* label, float* p32, float* pp32, double* p64a,
                        double* p64b, double* pp64, const SolveCtl* ctl, bool df);
// dtypes: FL_F32, FL_F64, and DT_DF (to the double-float pressure)
void launch_convert(cudaStream_t s, const void* src, int src_dtype, void* dst, int dst_dtype, long n);

// fl_multigrid.cu
void mg_setup(Engine& e);  // allocates levels for e.nx, e.ny and the coarsest size
void mg_free(Engine& e);
void mg_build_codes(Engine& e);  // label chain + stencil codes from levels[0].label
void mg_build_codes_if(Engine& e, cudaStream_t s, int* flag);  // the same when *flag is set; clears it
void mg_vcycle(Engine& e, StepAccum* acc_for_residual);
void mg_vcycle_on(Engine& e, const float* b0, bool zero_start, StepAccum* acc_for_residual);
// the refined-pressure pass: float64, or double-float pairs in the same buffers when df
// test 1 / 2: the pass's last block also runs the begin / cycle test
// (k_solve_begin / k_solve_check) on the residual it accumulated and, with
// use_cond, sets the graph's conditional handle h.
void launch_update_resid64(cudaStream_t s, int nx, int ny, double* p64a, double* p64b, SolveCtl* ctl,
                           const float* e, const float* b, const float* b_lo, const uint8_t* code, bool update,
                           float* r32, StepAccum* acc, bool df, int test = 0, bool use_cond = false,
                           cudaGraphConditionalHandle h = 0);
void launch_solve_begin(cudaStream_t s, StepAccum* acc, SolveCtl* ctl, bool use_cond, cudaGraphConditionalHandle h);
void launch_solve_check(cudaStream_t s, StepAccum* acc, SolveCtl* ctl, bool use_cond, cudaGraphConditionalHandle h);
void launch_zero_if(cudaStream_t s, const SolveCtl* ctl, float* p32, double* p64a, double* p64b, long n);
void launch_rb_sweeps(cudaStream_t s, int nx, int ny, const float* x_in, float* x_out, const float* b,
                      const uint8_t* code, float scale, float omega, int pairs, const float* scale_dev = nullptr);
void launch_rms_remaining(cudaStream_t s, int nx, int ny, const float* p, const float* div, const uint8_t* code,
                          float scale, StepAccum* acc);
void launch_build_codes(cudaStream_t s, int nx, int ny, const uint8_t* label, uint8_t* code,
                        const int* only_if = nullptr);
// cur = in, raising *flag when any of the n labels changed
void launch_label_sync(cudaStream_t s, const uint8_t* in, uint8_t* cur, long n, int* flag);
// the conditional `h` = (*flag != 0), then *flag = 0
void launch_label_cond(cudaStream_t s, int* flag, cudaGraphConditionalHandle h);
void launch_rb_halfsweep(cudaStream_t s, int nx, int ny, float* p, const float* b, const uint8_t* code,
                         float scale, float omega, int color);

}  // namespace fl
