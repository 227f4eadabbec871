/*
 * flowlab_gb300 — C ABI of the GB300 (sm_103a) engine for flowlab's 2D
 * incompressible MAC-grid projection step.
 *
 * This is the drop-in boundary for the reference's three GPU seams:
 *   GpuStep        src/core/simulation.ts:35-84   (implemented by src/gpu/stepGpu.ts:89)
 *   PressureSolver src/core/pressureSolver.ts:21-41 (src/gpu/multigridGpu.ts:59,
 *                                                   src/gpu/pressureGpu.ts:68)
 *   Advector       src/core/advector.ts:28-63      (src/gpu/advectGpu.ts:54)
 * plus the per-kernel passes of src/core (one entry point each) so every pass
 * can be diffed against its CPU twin, as the reference's *.gputest.ts files do.
 *
 * Conventions
 *   - Plain C types only. Host arrays are caller-owned; the engine copies on
 *     upload and readback and never keeps a host pointer (the reference's
 *     writeBuffer/mapAsync discipline). Device buffers belong to the engine
 *     and are freed by fl_destroy.
 *   - MAC layout of src/core/grid.ts:1-36: p and label nx*ny (stride nx),
 *     u (nx+1)*ny (stride nx+1), v nx*(ny+1) (stride nx). Dye is the three
 *     channels' dnx*dny planes laid end to end (dnx = nx*dye_scale).
 *   - Labels are uint8: 0 Fluid, 1 Air, 2 Solid (grid.ts:41-45).
 *   - Every function returns an int status (FL_OK = 0). On failure
 *     fl_last_error(engine) describes it; fl_last_error(NULL) describes a
 *     failed fl_create. There is no CPU fallback: without a usable CUDA
 *     device every compute entry point fails with FL_EDEVICE.
 *   - An engine is not re-entrant: a call made while another call on the
 *     same engine is running returns FL_EBUSY (the reference throws
 *     "... is not re-entrant", stepGpu.ts:402, multigridGpu.ts:318).
 *   - Compute is float32 (the reference's WGSL precision), optionally with a
 *     refined fine-level pressure for iterative refinement (fl_params.mixed):
 *     float64, or a double-float pair of floats computed on the float32 pipe.
 */
#ifndef FLOWLAB_GB300_H
#define FLOWLAB_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FL_ABI_VERSION 3

typedef struct fl_engine fl_engine;

enum fl_status {
  FL_OK = 0,
  FL_EINVAL = 1,     /* bad argument or size */
  FL_EBUSY = 2,      /* engine already inside a call (not re-entrant) */
  FL_EDEVICE = 3,    /* CUDA error or no device ("GPU device lost", stepGpu.ts:403) */
  FL_ETIMEOUT = 4,   /* a bounded device wait gave up */
  FL_ENONFINITE = 5, /* the solve produced NaN/Inf */
  FL_ENOMEM = 6,     /* device allocation failed */
  FL_ESTATE = 7      /* call out of order (e.g. step before any upload) */
};

enum fl_dtype { FL_F32 = 0, FL_F64 = 1 };

/* src/core/advect.ts:21 AdvectionScheme */
enum fl_scheme { FL_SEMI_LAGRANGIAN = 0, FL_MACCORMACK = 1 };

/* Which pressure solver the fused step runs. */
enum fl_solver { FL_SOLVER_RBSOR = 0, FL_SOLVER_MG = 1 };

/*
 * Step parameters: src/core/simulation.ts:134-234 (SimulationParams) reduced
 * to what the projection step reads, the multigrid constants of
 * src/core/pressureMultigrid.ts:47-67 made runtime values, and the knobs the
 * reference does not have (alpha, confinement, mixed precision).
 */
typedef struct fl_params {
  double cfl_target;     /* simulation.ts:141 */
  double dt_max;         /* simulation.ts:150 */
  double rho;            /* simulation.ts:165 */
  int scheme;            /* enum fl_scheme */
  int solver;            /* enum fl_solver */
  int pressure_iters;    /* red-black sweep budget (simulation.ts:152) */
  int mg_max_cycles;     /* V-cycle cap (pressureMultigrid.ts:63 MG_CYCLES) */
  double omega;          /* SOR relaxation for the red-black solver */
  double tol;            /* relative residual target; <= 0 runs the full budget */
  double dye_decay[3];   /* per channel, per second of sim time (simulation.ts:184) */
  double beta;           /* buoyancy weight on dye channel 0 (simulation.ts:191) */
  double alpha;          /* soot weight on dye channel 1 (force -alpha*s) */
  double confinement;    /* vorticity confinement epsilon; 0 = off */
  int mg_pre, mg_post;   /* smoothing sweep pairs per level (reference 2, 2) */
  int mg_coarse_sweeps;  /* sweep pairs on the coarsest level (reference 8) */
  int mg_coarsest;       /* stop coarsening at <= this many cells a side (reference 4; at most 64) */
  double mg_omega;       /* smoother relaxation (reference 1.0) */
  int mixed;             /* defect correction around the multigrid: 0 off; 1 float64 fine pressure and
                            residual; 2 the same with a double-float pressure (hi + lo, two floats,
                            ~48 significand bits) and residual, all float32 arithmetic */
  int rb_pairs;          /* red-black sweep pairs per launch, 1..4 (0: 4): the temporal-blocking
                            depth, i.e. the tile/halo shape; results do not depend on it */
  int warm_extrapolate;  /* 1: the multigrid starts from 2 p(n) - p(n-1) on Fluid cells instead of
                            p(n) (no reference counterpart; pressureSolver.ts:28-30 uses p(n)) */
  int mg_tail_side;      /* the levels with both sides <= this (1..64; 0: 32) run inside one
                            single-CTA kernel per V-cycle, the finer ones as their own launches;
                            results do not depend on it */
  int residual_every;    /* simulation.ts:193-206 residualEvery: recompute the post-step divergence
                            (the residual diagnostic, simulation.ts:539-540) on the steps whose
                            index, counted from the engine's creation, is a multiple of this;
                            0 never (the reference's default is 1). Nothing in the step reads it. */
  int reserved[3];
} fl_params;

/* Per-step report (the reference's sim.iters / sim.dt plus the residual the
 * GPU path never computed). */
typedef struct fl_stats {
  double dt, scale, grad_scale;
  double time;           /* accumulated sim time */
  int cycles;            /* V-cycles (multigrid) or sweep pairs (red-black) of the last solve */
  int steps;             /* steps taken since the last upload */
  double rel_residual;   /* RMS remaining divergence / RMS fluid divergence, last solve; -1 if unchecked */
  double div_rms;        /* RMS of b = -scale*div over fluid cells, last solve */
  double max_face_speed; /* max |u|,|v| after the last step (CFL input of the next one) */
  /* The residual diagnostic of the last step that computed it
   * (fl_params.residual_every): RMS and max of |div| over FLUID cells of the
   * projected velocity, the inputs of viz/fieldView.ts:44-60 divergenceStats
   * before its normalisation by maxSpeed/h; post_div_step is that step's
   * index counted from the engine's creation (-1: never computed). */
  double post_div_rms;
  double post_div_max;
  long long post_div_step;
  /* The relative residual of the last solve's starting pressure (the warm
   * start), before any cycle: evaluated by the defect-correction solve
   * (fl_params.mixed), -1 otherwise. What a better warm start lowers. */
  double initial_rel_residual;
} fl_stats;

/* Per-phase device timing of fused steps, from CUDA events recorded on the
 * engine's stream around each phase while profiling is enabled. Profiled
 * steps run eagerly (not as a graph), and each phase is preceded by a short
 * fixed-duration hold kernel so that the phase's launches are queued before
 * the device reaches its first event: the events then bracket device work
 * only, not host submission. `bytes` is the algorithmic DRAM traffic the
 * engine attributes to the phase: each array a kernel must read or write,
 * counted once per launch. No counterpart in the reference (its profiler is
 * host-side phase timing, src/core/profiler.ts:39-113). */
#define FL_PHASES 15
/* phase indices: the multigrid phases separate the finest level's smoother
 * launches from the coarser levels'; CONTROL is the one-thread solve-control
 * kernels (tolerance test, cycle decision) and the p = 0 fill; WARM_START
 * is the learned warm start (input, network, correction) when attached;
 * CFL is the end-of-step scan, which also runs the post-step divergence
 * diagnostic (residual_every). */
enum fl_phase {
  FL_PH_ADVECT_VELOCITY = 0, FL_PH_BODY_FORCES = 1, FL_PH_DIVERGENCE = 2, FL_PH_MG_PRE_FINE = 3, FL_PH_MG_PRE = 4,
  FL_PH_MG_COARSE = 5, FL_PH_MG_POST = 6, FL_PH_MG_POST_FINE = 7, FL_PH_DEFECT64 = 8, FL_PH_RB_SWEEPS = 9,
  FL_PH_PROJECT = 10, FL_PH_ADVECT_DYE = 11, FL_PH_CFL = 12, FL_PH_CONTROL = 13, FL_PH_WARM_START = 14
};
typedef struct fl_profile {
  double ms[FL_PHASES];
  long long launches[FL_PHASES];
  double bytes[FL_PHASES];
} fl_profile;

/* Fills `p` with the reference defaults (simulation.ts:223-234,
 * pressureMultigrid.ts:47-67). */
void fl_default_params(fl_params* p);

int fl_abi_version(void);
const char* fl_last_error(const fl_engine* e);

/* ------------------------------------------------------------ lifecycle */

/* Builds the device side for an nx*ny grid with cell size h and a dye grid
 * refined by dye_scale (simulation.ts:353-374, stepGpu.ts:176-289). */
int fl_create(int nx, int ny, double h, int dye_scale, const fl_params* params, int device, fl_engine** out);
/* Frees every device buffer (advectGpu.ts:382-398, stepGpu.ts:674-689). */
int fl_destroy(fl_engine* e);
int fl_set_params(fl_engine* e, const fl_params* params);
/* The engine's CUDA stream (a cudaStream_t), for callers that time or order
 * work against it. */
void* fl_stream(fl_engine* e);
int fl_synchronize(fl_engine* e);

/* ------------------------------------------------- GpuStep (simulation.ts:35-84) */

/* invalidate() + the dirty upload of stepGpu.ts:419-433: the host holds truth
 * for u, v, p, label and dye. dtype is FL_F32 or FL_F64 for the float fields;
 * p may be NULL (zero warm start). */
int fl_upload_fields(fl_engine* e, int dtype, const void* u, const void* v, const void* p, const uint8_t* label,
                     const void* dye);
/* setLabels: labels changed under resident fields (stepGpu.ts:323-330); the
 * next step first zeroes faces touching new solids (commit_labels) and
 * re-coarsens. */
int fl_set_labels(fl_engine* e, const uint8_t* label);
/* setDyePatch (stepGpu.ts:337-362): data is 4 planes of pnx*pny floats (3 value
 * planes + coverage, dye.ts:108-127); NULL clears it. */
int fl_set_dye_patch(fl_engine* e, int i0, int j0, int pnx, int pny, const float* data);
/* setBuoyancy (stepGpu.ts:366-368), extended with the soot weight alpha. */
int fl_set_buoyancy(fl_engine* e, double beta, double alpha);
int fl_set_confinement(fl_engine* e, double eps);
/* setStir (stepGpu.ts:319-321): x, y, r, dx, dy in world units; consumed by
 * the next step. NULL clears. */
int fl_set_stir(fl_engine* e, const double* stir5);
/* step(f, scheme, dt, scale, gradScale, dyeKeep) (simulation.ts:36-38,
 * stepGpu.ts:393-559) with the caller's advection scheme, dt, scale,
 * gradScale and per-channel keep factors. The scheme is per call, as in the
 * seam; it also becomes the engine's fl_params.scheme for later
 * fl_step_auto calls. Returns the pressure iterations in *iters. */
int fl_step(fl_engine* e, int scheme, double dt, double scale, double grad_scale, const double keep[3], int* iters);
/* `nsteps` steps with dt from the CURRENT velocity on the device
 * (simulation.ts:474-479 without the host scan or the one-step-stale
 * readback). No host synchronisation between steps unless tol > 0 requires
 * a residual readback. */
int fl_step_auto(fl_engine* e, int nsteps, int* iters_last);
/* One step the way GpuStep.step (simulation.ts:35-84, GpuStepper.step in
 * stepGpu.ts:393-560) runs it, with host buffers of `dtype` (FL_F32 or
 * FL_F64: the reference's FieldArray is Float32Array or Float64Array,
 * grid.ts:53-54) for every float field in and out: when u is non-null the
 * host fields (u, v, p, label, dye; p may be null: zero) are uploaded first,
 * as after invalidate() (fl_upload_fields semantics); then one step with dt
 * from the device (fl_step_auto); then the results are copied into the
 * non-null outputs. With FL_F32 the dye upload overlaps the step's first
 * kernels, the velocity and pressure readback overlaps the dye advection
 * and the dye readback the final CFL scan; FL_F64 converts on the device
 * around synchronous copies.
 * Returns when every copy completed; results equal fl_upload_fields +
 * fl_step_auto + fl_read_* bit for bit. */
int fl_step_host(fl_engine* e, int dtype, const void* u, const void* v, const void* p, const uint8_t* label,
                 const void* dye, void* u_out, void* v_out, void* p_out, void* dye_out, int* iters);
int fl_get_stats(fl_engine* e, fl_stats* out);
/* Readbacks (drainReadback / readDye, stepGpu.ts:372-391, 578-604). */
int fl_read_velocity(fl_engine* e, int dtype, void* u, void* v);
int fl_read_dye(fl_engine* e, int dtype, void* dye);
int fl_read_pressure(fl_engine* e, int dtype, void* p);
/* The post-step divergence field (Simulation.div after a step that
 * recomputed it, simulation.ts:539-540; nx*ny cells, every label) of the
 * last step that computed it (fl_stats.post_div_step); zeros before any. */
int fl_read_divergence(fl_engine* e, int dtype, void* div);

/* Enables (1) or disables (0) phase timing and clears the counters. */
int fl_profile_enable(fl_engine* e, int on);
/* Synchronises and returns the counters accumulated since enabling. */
int fl_profile_read(fl_engine* e, fl_profile* out);

/* ------------------------------------ Advector (advector.ts:28-63), float32 host arrays */

/* advectVelocity / advectVelocityMacCormack (advect.ts:126-211). */
int fl_advect_velocity(fl_engine* e, int scheme, const float* u_in, const float* v_in, float* u_out, float* v_out,
                       const uint8_t* label, float dt);
/* dye(g, scheme, u, v, qIn[], qOut[], label, dt, dg) (advector.ts:52-62):
 * advectScalar / advectScalarMacCormack (advect.ts:241-312) of the three
 * channels on one backtrace; q_in and q_out are arrays of three plane
 * pointers of dnx*dny floats each (dnx = nx*dye_scale). */
int fl_advect_dye(fl_engine* e, int scheme, const float* u, const float* v, const float* const* q_in,
                  float* const* q_out, const uint8_t* label, float dt);

/* ---------------------------- PressureSolver (pressureSolver.ts:21-41), float32 host arrays */

/* Red-black SOR (pressureRedBlack.ts:88-113): p is the in/out warm start. */
int fl_rb_solve(fl_engine* e, float* p, const float* div, const uint8_t* label, float scale, int iterations,
                float omega, double tol, int* sweeps_used);
/* Geometric multigrid (pressureMultigrid.ts:284-319) with the engine's
 * V(pre,post)/coarsest shape; runs until the relative residual <= tol or
 * max_cycles. */
int fl_mg_solve(fl_engine* e, float* p, const float* div, const uint8_t* label, float scale, int max_cycles,
                double tol, int* cycles_used, double* rel_residual);

/* The same multigrid wrapped in defect correction (NEW, no reference
 * counterpart): p is a float64 in/out warm start; each pass forms
 * r = b - A p in extended precision, runs one float32 V-cycle on A e = r from
 * e = 0 and adds e back, until the relative residual <= tol or max_cycles.
 * The extended precision is the engine's fl_params.mixed: float64 (1), or
 * double-float pairs (2; p is converted to pairs on the way in and back to
 * float64 as hi + lo on the way out). This is what reaches relative
 * residuals below float32's ~1e-5 floor. */
int fl_mg_solve_mixed(fl_engine* e, double* p, const float* div, const uint8_t* label, float scale, int max_cycles,
                      double tol, int* cycles_used, double* rel_residual);

/* ------------------------------------------- single passes, float32 host arrays */

int fl_divergence(fl_engine* e, const float* u, const float* v, float* div);           /* divergence.ts:17-25 */
int fl_rb_sweep(fl_engine* e, float* p, const float* div, const uint8_t* label, float scale, float omega,
                int color);                                                           /* pressureRedBlack.ts:32-72 */
int fl_subtract_gradient(fl_engine* e, const float* p, float* u, float* v, const uint8_t* label,
                         float grad_scale);                                           /* subtractGradient.ts:40-61 */
int fl_outflow(fl_engine* e, float* u, float* v, const uint8_t* label);                /* boundaries.ts:115-143 */
int fl_commit_labels(fl_engine* e, float* p, float* u, float* v, float* dye,
                     const uint8_t* label);                                           /* boundaries.ts:45-64 */
/* buoyancy.ts:70-88 (+ alpha term) and vorticity confinement, in the step's
 * order: confinement force from the incoming velocity, buoyancy added, then
 * confinement added. */
int fl_body_forces(fl_engine* e, float* u, float* v, const float* dye, const uint8_t* label, float beta,
                   float alpha, float eps, float dt);
int fl_stir(fl_engine* e, float* u, float* v, const uint8_t* label, float x, float y, float r, float dx,
            float dy);                                                                /* stir.ts:49-83 */
int fl_dye_patch(fl_engine* e, float* dye, int i0, int j0, int pnx, int pny, const float* data); /* dye.ts:158-175 */

/* --------------------------------------------- no-allocation variant */

/*
 * Velocity advection (semi-Lagrangian or MacCormack, as fl_advect_velocity)
 * on the caller's own DEVICE buffers, allocating nothing. This entry point has
 * no counterpart in the reference. It is for callers that cannot call
 * cudaMalloc where they advect: real-time threads that must not block
 * (cudaMalloc can synchronise the device), hosts whose device memory all
 * comes from an arena or caching allocator they do not own, and processes
 * that reserve their whole device-memory budget up front. The MacCormack
 * scratch lives in one fixed array of the library's device memory (about
 * 8.8 MB on every GPU that loads the library, held until exit), so the grid
 * may have at most 2,200,000 faces, (nx+1)*ny + nx*(ny+1) (1024x1024 fits);
 * larger grids return FL_EINVAL. The outputs must not overlap each other or
 * the inputs (FL_EINVAL). The first call on each device looks the array up
 * and loads the kernels, so make it before any stream capture; calls after
 * cudaDeviceReset are not supported. Calls on one device share the array:
 * calls whose work overlaps on the GPU race, so order them on one stream.
 * Work is queued on `stream` (a cudaStream_t, NULL for the default stream)
 * and not waited for. Errors are reported by fl_last_error(NULL).
 */
int fl_advect_velocity_noalloc(int scheme, int nx, int ny, float h, float dt, const float* u_in, const float* v_in,
                               float* u_out, float* v_out, const uint8_t* label, void* stream);

/* ------------------------------------------------ learned warm start
 * No counterpart in the reference, whose warm start is the previous step's
 * pressure (src/core/pressureSolver.ts:28-30). A U-Net (4 levels of two
 * 3x3 convolutions + ReLU, 32/64/96/128 channels, average pooling down,
 * nearest upsampling with concatenated skips up, a 1x1 head; bf16 weights
 * and activations, float32 arithmetic) maps, per cell,
 *   x = (b / s_b, 1 if Fluid else 0, p_prev / s_p)     (NHWC, 3 channels)
 * to a correction: p_guess = p_prev + s_p * net(x) on Fluid cells, where
 * b = -scale * div, s_b = RMS of b and s_p = RMS of p_prev over Fluid cells
 * (s_p = s_b when p_prev vanishes). The multigrid then runs from p_guess to
 * the same tolerance as without it. Parameters are one float32 vector:
 * per layer the weights [cout][ky][kx][cin], then the biases, in the order
 * enc0a enc0b enc1a enc1b enc2a enc2b mida midb dec2a dec2b dec1a dec1b
 * dec0a dec0b head. */
typedef struct fl_unet fl_unet;

/* A network able to run batches of up to max_pixels = batch * height * width
 * (a multiple of 64) on `device`; parameters start at zero. */
int fl_unet_create(long long max_pixels, int device, fl_unet** out);
int fl_unet_destroy(fl_unet* u);
const char* fl_unet_last_error(const fl_unet* u);
long long fl_unet_num_params(void);
/* Parameters from / to a host float32 vector of fl_unet_num_params()
 * values; setting them also resets the Adam state. */
int fl_unet_set_params(fl_unet* u, const float* theta);
int fl_unet_get_params(fl_unet* u, float* theta);
/* x: batch*h*w*3 host floats (NHWC), out: batch*h*w; h and w multiples of 8. */
int fl_unet_forward(fl_unet* u, int batch, int h, int w, const float* x, float* out);
/* One training step on the masked mean squared error between the output and
 * `target` (mask: 1 to count a pixel, 0 to skip it): forward, backward and,
 * when `update` is nonzero, one Adam step (beta 0.9 / 0.999, eps 1e-8) with
 * learning rate lr. Returns the loss; `grad` (optional, host) receives the
 * gradient. */
int fl_unet_train_step(fl_unet* u, int batch, int h, int w, const float* x, const float* target, const float* mask,
                       double lr, int update, double* loss, float* grad);
/* Process-wide choice for the 3x3 convolutions with 32 or more input
 * channels: 0 CUDA cores; 1 tensor cores (tcgen05) for the forward pass and
 * for the backward pass's data and weight gradients, halo tiles loaded once
 * per 32 input channels by TMA and reused by all 9 taps (default); 2 tensor
 * cores for the forward pass only, each tap's input gathered per 32-channel
 * chunk (backward on CUDA cores). */
int fl_unet_use_tensor_cores(int mode);
/* The tensor-core kernels wait on their own copies and MMAs with bounded
 * mbarrier polls. A wait that gates progress gives up after `polls` polls
 * (<= 0 restores the default, about 4 million) and the call then returns
 * FL_ETIMEOUT; the waits that drain a CTA's own in-flight copies and MMAs
 * before it frees its tensor memory keep the default bound. For tests of
 * the timeout path (a limit of 1 makes the waits run out) and for callers
 * that need a call to fail fast. Applies to the current device. No
 * counterpart in the reference. */
int fl_unet_set_wait_limit(long long polls);
/* Attaches (or, with NULL, detaches) the network as the engine's warm start:
 * every multigrid step then runs it between the divergence and the solve.
 * The grid's sides must be multiples of 8 and fit the network's capacity;
 * the network must not be used elsewhere while the engine steps. */
int fl_set_warm_start(fl_engine* e, fl_unet* u);
/* The last step's (or solve's) pressure right-hand side, nx*ny values:
 * b = -scale * div for the multigrid (the training input of the warm
 * start), div itself for the red-black solver. */
int fl_read_rhs(fl_engine* e, int dtype, void* b);

/* ------------------------------------------------------- batched scenes
 * No counterpart in the reference (one scene per Simulation). A batch
 * steps several engines (scenes of any sizes on one device) together, one
 * graph launch per step. When every scene solves with the multigrid and
 * the same V-cycle shape (mg_pre, mg_post), the scenes' pressure solves run
 * as ONE launch per V-cycle phase over a work list of (scene, level, tile)
 * items of every scene, the scenes' single-CTA tails aligned, inside one
 * device-side cycle loop that runs while any scene iterates; a scene that
 * has converged leaves its items at once, so each scene runs the cycles it
 * would run alone, with bit-identical results. Each scene's passes before
 * and after the solve (advection, forces, divergence; projection, dye,
 * CFL) are concurrent branches of the same graph. Otherwise (a red-black
 * scene, differing shapes) each step launches every engine's own step
 * graph on the engine's own stream, largest scenes first, as many at once
 * as the process's hardware queues allow (CUDA_DEVICE_MAX_CONNECTIONS, read
 * when CUDA initialises; 8 by default, up to 32). The engines must have
 * uploaded fields and be eligible for graph steps (no profiling, pending
 * stir or label edit; multigrid, or red-black SOR with a fixed sweep
 * count). Statistics and fields are read per engine; an engine may be
 * stepped alone between batch steps, or change its parameters (the batch
 * then rebuilds its graphs). */
typedef struct fl_batch fl_batch;
int fl_batch_create(fl_engine* const* engines, int count, fl_batch** out);
int fl_batch_destroy(fl_batch* b);
const char* fl_batch_last_error(const fl_batch* b);
/* A stream (cudaStream_t) that completes after every engine's last step of
 * the latest fl_batch_step. */
void* fl_batch_stream(fl_batch* b);
/* 1 when the batch steps through the work-list solve (every scene solves
 * with the multigrid, one V-cycle shape), 0 when it launches each engine's
 * own step graph on its own stream. */
int fl_batch_worklist(const fl_batch* b);
/* Chooses the path: 1 the work-list solve (FL_EINVAL, and the message in
 * fl_batch_last_error, when some scene does not qualify), 0 every engine's
 * own step graph on its own stream. Results are identical either way;
 * which is faster depends on the scenes (flowlab_gb300/autotune.py times
 * both). A batch starts on the work list when every scene qualifies. */
int fl_batch_set_worklist(fl_batch* b, int on);
/* nsteps steps of every engine, asynchronous; each engine's steps are
 * ordered after its earlier work and before its later work (its stream),
 * and after the batch stream's earlier work. */
int fl_batch_step(fl_batch* b, int nsteps);

#ifdef __cplusplus
}
#endif
#endif /* FLOWLAB_GB300_H */
