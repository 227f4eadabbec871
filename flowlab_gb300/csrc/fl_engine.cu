// The C ABI (include/flowlab_gb300.h): the engine object, field residency,
// the fused step and the per-pass entry points.
//
// The step (stepGpu.ts:393-559 re-designed for one GB300):
//   advect u,v -> [stir] -> [confinement force] -> body forces -> divergence
//   -> pressure solve -> subtract gradient + outflow -> advect dye (+decay,
//   +inlet) -> CFL reduction that writes the NEXT step's dt on the device.
// u, v, p and the dye stay resident; nothing crosses the bus per step except
// the residual scalars the tolerance test needs (32 bytes per V-cycle).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>

#include "fl_internal.h"
#include "fl_unet.h"

using namespace fl;

namespace fl {
Unet* unet_of(fl_unet* h);
}

struct fl_engine {
  Engine e;
};

namespace fl {

int prof_begin(Engine& e, int phase) {
  if (!e.profiling) return -1;
  launch_hold(e.stream);
  Engine::PendingPhase p;
  p.phase = phase;
  for (cudaEvent_t* ev : {&p.a, &p.b}) {
    if (!e.event_pool.empty()) {
      *ev = e.event_pool.back();
      e.event_pool.pop_back();
    } else if (cudaEventCreate(ev) != cudaSuccess) {
      return -1;
    }
  }
  p.bytes = 0;
  p.launches = 0;
  cudaEventRecord(p.a, e.stream);
  e.pending.push_back(p);
  return (int)e.pending.size() - 1;
}

void prof_end(Engine& e, int token, double bytes, int launches) {
  if (token < 0 || token >= (int)e.pending.size()) return;
  Engine::PendingPhase& p = e.pending[token];
  p.bytes = bytes;
  p.launches = launches;
  cudaEventRecord(p.b, e.stream);
}

// Folds recorded phases into the counters (synchronises).
static void prof_drain(Engine& e) {
  if (e.pending.empty()) return;
  cudaStreamSynchronize(e.stream);
  for (auto& p : e.pending) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      e.prof_ms[p.phase] += ms;
      e.prof_bytes[p.phase] += p.bytes;
      e.prof_launches[p.phase] += p.launches;
    }
    e.event_pool.push_back(p.a);
    e.event_pool.push_back(p.b);
  }
  e.pending.clear();
}

}  // namespace fl

namespace {

thread_local std::string g_create_error;

}  // namespace

void fl::set_global_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_create_error = buf;
}

namespace {

int fail(Engine* e, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (e)
    e->err = buf;
  else
    g_create_error = buf;
  return code;
}

int cuda_status(Engine* e, cudaError_t err, const char* where) {
  if (err == cudaSuccess) return FL_OK;
  if (err == cudaErrorMemoryAllocation) return fail(e, FL_ENOMEM, "%s: %s", where, cudaGetErrorString(err));
  return fail(e, FL_EDEVICE, "%s: %s", where, cudaGetErrorString(err));
}

int check_launch(Engine* e, const char* where) { return cuda_status(e, cudaGetLastError(), where); }

int sync(Engine* e, const char* where) {
  cudaError_t err = cudaStreamSynchronize(e->stream);
  if (err == cudaSuccess) err = cudaGetLastError();
  return cuda_status(e, err, where);
}

// One call at a time per engine (the reference's busy flags,
// stepGpu.ts:160, 402-405).
struct Call {
  Engine* e;
  bool ok;
  explicit Call(fl_engine* h) : e(h ? &h->e : nullptr), ok(false) {
    if (!e) return;
    int expected = 0;
    ok = e->busy.compare_exchange_strong(expected, 1);
    if (ok) cudaSetDevice(e->device);
  }
  ~Call() {
    if (ok) e->busy.store(0);
  }
};

#define ENTER(h)                                                                    \
  if (!(h)) return fail(nullptr, FL_EINVAL, "null engine");                        \
  Call call_(h);                                                                    \
  Engine* e = call_.e;                                                              \
  if (!call_.ok) return fail(e, FL_EBUSY, "engine call is not re-entrant");

#define TRY(x)            \
  do {                    \
    int st_ = (x);        \
    if (st_) return st_;  \
  } while (0)

int dalloc(Engine* e, void** p, size_t bytes, const char* what) {
  cudaError_t err = cudaMalloc(p, bytes);
  if (err != cudaSuccess) return cuda_status(e, err, what);
  return cudaMemsetAsync(*p, 0, bytes, e->stream) == cudaSuccess ? FL_OK : cuda_status(e, cudaGetLastError(), what);
}

void destroy_graphs(Engine* e);

void free_all(Engine* e) {
  cudaFree(e->u[0]);
  cudaFree(e->u[1]);
  cudaFree(e->v[0]);
  cudaFree(e->v[1]);
  cudaFree(e->u_hat);
  cudaFree(e->v_hat);
  cudaFree(e->dye[0]);
  cudaFree(e->dye[1]);
  cudaFree(e->dye_hat);
  cudaFree(e->w);
  cudaFree(e->fx);
  cudaFree(e->fy);
  cudaFree(e->patch);
  cudaFree(e->sc);
  cudaFree(e->acc);
  cudaFree(e->time_dev);
  cudaFree(e->staging);
  cudaFree(e->p32_final);
  cudaFree(e->p64[0]);
  cudaFree(e->p64[1]);
  cudaFree(e->r32);
  cudaFree(e->b_lo);
  cudaFree(e->pprev32);
  cudaFree(e->pprev64);
  cudaFree(e->bt_u);
  cudaFree(e->bt_v);
  cudaFree(e->bt_d);
  cudaFree(e->ctl);
  cudaFree(e->ws_scales);
  cudaFree(e->label_in);
  cudaFree(e->label_flag);
  cudaFree(e->div_post);
  cudaFree(e->diag);
  destroy_graphs(e);
  if (!e->levels.empty()) cudaFree(e->levels[0].label);
  mg_free(*e);
  for (auto& p : e->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (cudaEvent_t ev : e->event_pool) cudaEventDestroy(ev);
  if (e->acc_host) cudaFreeHost(e->acc_host);
  if (e->ctl_host) cudaFreeHost(e->ctl_host);
  if (e->diag_host) cudaFreeHost(e->diag_host);
  if (e->ev_dye) cudaEventDestroy(e->ev_dye);
  if (e->ev_proj) cudaEventDestroy(e->ev_proj);
  if (e->ev_dye_done) cudaEventDestroy(e->ev_dye_done);
  if (e->ev_p) cudaEventDestroy(e->ev_p);
  if (e->ev_lab) cudaEventDestroy(e->ev_lab);
  if (e->ev_lab_done) cudaEventDestroy(e->ev_lab_done);
  if (e->ev_lab_sync) cudaEventDestroy(e->ev_lab_sync);
  if (e->stream3) cudaStreamDestroy(e->stream3);
  if (e->ev_prior) cudaEventDestroy(e->ev_prior);
  if (e->stream2) cudaStreamDestroy(e->stream2);
  if (e->stream) cudaStreamDestroy(e->stream);
}

int validate_params(Engine* e, const fl_params* p) {
  if (p->scheme != FL_SEMI_LAGRANGIAN && p->scheme != FL_MACCORMACK) return fail(e, FL_EINVAL, "scheme %d", p->scheme);
  if (p->solver != FL_SOLVER_RBSOR && p->solver != FL_SOLVER_MG) return fail(e, FL_EINVAL, "solver %d", p->solver);
  if (p->mg_pre < 0 || p->mg_pre > 4 || p->mg_post < 0 || p->mg_post > 4)
    return fail(e, FL_EINVAL, "mg_pre/mg_post must be in [0, 4] (got %d, %d)", p->mg_pre, p->mg_post);
  if (p->mg_coarse_sweeps < 0 || p->mg_max_cycles < 0 || p->pressure_iters < 0)
    return fail(e, FL_EINVAL, "negative sweep or cycle count");
  // the coarsest level is solved inside the single-CTA tail (sides <= 64 at most)
  if (p->mg_coarsest < 1 || p->mg_coarsest > 64) return fail(e, FL_EINVAL, "mg_coarsest must be in [1, 64]");
  if (p->rb_pairs < 0 || p->rb_pairs > 4) return fail(e, FL_EINVAL, "rb_pairs must be in [0, 4]");
  if (p->mixed < 0 || p->mixed > MIXED_DF) return fail(e, FL_EINVAL, "mixed must be 0, 1 or 2 (got %d)", p->mixed);
  // the tail kernel's ownership map holds levels of at most 64 x 64 cells
  if (p->mg_tail_side < 0 || p->mg_tail_side > 64) return fail(e, FL_EINVAL, "mg_tail_side must be in [0, 64]");
  if (p->residual_every < 0) return fail(e, FL_EINVAL, "residual_every must be >= 0");
  if (!(p->cfl_target > 0) || !(p->dt_max > 0) || !(p->rho > 0))
    return fail(e, FL_EINVAL, "cfl_target, dt_max and rho must be positive");
  return FL_OK;
}

// Host-side float32 evaluation of the step scalars (simulation.ts:477-479,
// buoyancy.ts:80) for calls that are handed dt.
StepScalars host_scalars(const Engine* e, float dt, float scale, float grad_scale, const double keep[3]) {
  StepScalars s{};
  s.dt = dt;
  s.scale = scale;
  s.grad_scale = grad_scale;
  for (int c = 0; c < 3; c++) s.keep[c] = keep ? (float)keep[c] : 1.0f;
  s.gain_beta = (float)e->prm.beta * dt;
  s.gain_alpha = -(float)e->prm.alpha * dt;
  s.half_dt = 0.5f * dt;
  s.neg_scale = -scale;
  return s;
}

// Ordered on the engine's (non-blocking) stream; a pageable source is staged
// before the call returns, so `s` may be a temporary.
int put_scalars(Engine* e, const StepScalars& s) {
  return cuda_status(e, cudaMemcpyAsync(e->sc, &s, sizeof s, cudaMemcpyHostToDevice, e->stream), "scalars");
}

int upload(Engine* e, void* dst, const void* src, long n, int dtype, const char* what) {
  if (!src) return fail(e, FL_EINVAL, "%s: null pointer", what);
  if (dtype == FL_F32) return cuda_status(e, cudaMemcpyAsync(dst, src, n * sizeof(float), cudaMemcpyHostToDevice, e->stream), what);
  if (dtype != FL_F64) return fail(e, FL_EINVAL, "%s: dtype %d", what, dtype);
  TRY(cuda_status(e, cudaMemcpyAsync(e->staging, src, n * sizeof(double), cudaMemcpyHostToDevice, e->stream), what));
  launch_convert(e->stream, e->staging, FL_F64, dst, FL_F32, n);
  TRY(check_launch(e, what));
  // the staging buffer is reused by the next conversion
  return sync(e, what);
}

int download(Engine* e, void* dst, const float* src, long n, int dtype, const char* what) {
  if (!dst) return fail(e, FL_EINVAL, "%s: null pointer", what);
  if (dtype == FL_F32) return cuda_status(e, cudaMemcpyAsync(dst, src, n * sizeof(float), cudaMemcpyDeviceToHost, e->stream), what);
  if (dtype != FL_F64) return fail(e, FL_EINVAL, "%s: dtype %d", what, dtype);
  launch_convert(e->stream, src, FL_F32, e->staging, FL_F64, n);
  TRY(check_launch(e, what));
  TRY(cuda_status(e, cudaMemcpyAsync(dst, e->staging, n * sizeof(double), cudaMemcpyDeviceToHost, e->stream), what));
  return sync(e, what);
}

int up32(Engine* e, void* dst, const void* src, size_t bytes, const char* what) {
  if (!src) return fail(e, FL_EINVAL, "%s: null pointer", what);
  return cuda_status(e, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, e->stream), what);
}
// Level-0 labels written by an entry point other than fl_upload_fields: the
// multigrid labels and codes no longer follow them (the next upload rebuilds
// them whatever it is given).
int put_labels(Engine* e, const uint8_t* label, const char* what) {
  e->codes_valid = false;
  return up32(e, e->levels[0].label, label, (size_t)e->cells(), what);
}
int down32(Engine* e, void* dst, const void* src, size_t bytes, const char* what) {
  if (!dst) return fail(e, FL_EINVAL, "%s: null pointer", what);
  return cuda_status(e, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, e->stream), what);
}

int zero_solve_accum(Engine* e) {
  return cuda_status(e, cudaMemsetAsync(e->acc, 0, 4 * sizeof(double), e->stream), "accumulators");
}
int zero_residual_accum(Engine* e) {
  StepAccum* a = e->acc;
  cudaError_t err = cudaMemsetAsync(&a->res_sq, 0, sizeof(double), e->stream);
  if (err == cudaSuccess) err = cudaMemsetAsync(&a->n_res, 0, sizeof(unsigned long long), e->stream);
  return cuda_status(e, err, "residual accumulators");
}
int read_accum(Engine* e) {
  TRY(cuda_status(e, cudaMemcpyAsync(e->acc_host, e->acc, sizeof(StepAccum), cudaMemcpyDeviceToHost, e->stream), "read accumulators"));
  return sync(e, "read accumulators");
}

double rms(double sq, unsigned long long n) { return n > 0 ? std::sqrt(sq / (double)n) : 0.0; }

// fluidDivRms of a host array (pressure.ts:177-186), used where the reference
// evaluates it on the host before the device solve (pressureGpu.ts:228,
// multigridGpu.ts:323).
double host_fluid_div_rms(const float* div, const uint8_t* label, long n) {
  double s = 0;
  long c = 0;
  for (long k = 0; k < n; k++) {
    if (label[k] != FLUID) continue;
    s += (double)div[k] * (double)div[k];
    c++;
  }
  return c > 0 ? std::sqrt(s / (double)c) : 0.0;
}

// ------------------------------------------------------------ the step
//
// A step is enqueued in three parts: the pre-solve passes, the pressure solve
// (prologue, a cycle body repeated while the device says so, epilogue) and the
// post-solve passes. The eager path repeats the body while a flag read back
// from the device is set; the graph path captures the same kernels once, with
// the body inside a CUDA-graph WHILE node that the check kernel drives, so a
// whole step is one graph launch with no host round trip.

bool solve_on_device(const Engine* e) { return e->prm.solver == FL_SOLVER_MG || e->prm.tol <= 0; }

// Writes the solve parameters into the device control block. The float64
// buffer parity is state, not a parameter: it is kept unless reset_par.
int put_ctl(Engine* e, int mode, double tol, int max_cycles, bool reset_par) {
  int par = 0;
  if (!reset_par) {
    TRY(cuda_status(e, cudaMemcpyAsync(e->ctl_host, e->ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, e->stream),
                    "read solve state"));
    TRY(sync(e, "read solve state"));
    par = e->ctl_host->par;
  }
  SolveCtl c{};
  c.tol = tol;
  c.max_cycles = max_cycles;
  c.mode = mode;
  c.rel = -1;
  c.par = par;
  // a pageable source is staged before the call returns: no synchronisation
  return cuda_status(e, cudaMemcpyAsync(e->ctl, &c, sizeof(SolveCtl), cudaMemcpyHostToDevice, e->stream),
                     "solve state");
}

bool step_mixed(const Engine* e) { return e->prm.solver == FL_SOLVER_MG && e->prm.mixed; }
// the refined pressure is double-float pairs (in the float64 buffers)
bool refined_df(const Engine* e) { return e->prm.mixed == MIXED_DF; }

// The step's solve settings from the engine parameters.
int put_step_ctl(Engine* e, bool reset_par) {
  if (e->prm.solver == FL_SOLVER_MG)
    return put_ctl(e, e->prm.mixed ? SOLVE_MIXED : SOLVE_MG, e->prm.tol, e->prm.mg_max_cycles, reset_par);
  return put_ctl(e, SOLVE_RB, e->prm.tol, e->prm.pressure_iters, reset_par);
}

int read_ctl(Engine* e) {
  TRY(cuda_status(e, cudaMemcpyAsync(e->ctl_host, e->ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, e->stream),
                  "read solve state"));
  return sync(e, "read solve state");
}

// fl_step_host uploads the dye on the second stream while the step's first
// kernels run: the first kernel that reads the dye waits here (an event wait
// node when captured; the event is recorded before every graph launch).
bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &st) == cudaSuccess && st == cudaStreamCaptureStatusActive;
}

void wait_dye(Engine* e, cudaStream_t s) {
  cudaStreamWaitEvent(s, e->ev_dye, capturing(s) ? cudaEventWaitExternal : 0);
}

// Likewise for the pressure fl_step_host uploads on the second stream: the
// first reader of p (the warm starts, the solve) waits here.
void wait_p(Engine* e, cudaStream_t s) {
  cudaStreamWaitEvent(s, e->ev_p, capturing(s) ? cudaEventWaitExternal : 0);
}

// And for the multigrid labels and stencil codes fl_step_host rebuilds on
// the third stream: the first reader of the codes (the solve) waits here.
void wait_codes(Engine* e, cudaStream_t s) {
  cudaStreamWaitEvent(s, e->ev_lab_done, capturing(s) ? cudaEventWaitExternal : 0);
}

// advect u,v -> [stir] -> [confinement] -> body forces -> divergence
void enqueue_pre(Engine* e, cudaStream_t s, int par, bool stir) {
  Level& L0 = e->levels[0];
  const int mac = e->prm.scheme == FL_MACCORMACK;
  const double N = (double)e->cells(), F = (double)(e->ufaces() + e->vfaces()), D = (double)e->dye_cells();
  int tok = prof_begin(*e, FL_PH_ADVECT_VELOCITY);
  launch_advect_velocity(s, e->nx, e->ny, e->h, mac, e->u[par], e->v[par], e->u_hat, e->v_hat, e->u[1 - par],
                         e->v[1 - par], L0.label, e->sc, e->bt_u, e->bt_v);
  // forward: carrier u,v + label in, faces out (MacCormack: + backtrace positions out);
  // correction: u,v + hat + positions + label in, faces out
  prof_end(*e, tok, mac ? (16 * F + N) + (20 * F + N) : 8 * F + N, mac ? 2 : 1);
  float* u = e->u[1 - par];
  float* v = e->v[1 - par];
  if (stir) launch_stir(s, e->nx, e->ny, e->h, u, v, L0.label, e->stir);
  const bool conf = e->prm.confinement != 0;
  const bool beta_on = e->prm.beta != 0, alpha_on = e->prm.alpha != 0;
  tok = prof_begin(*e, FL_PH_BODY_FORCES);
  double fbytes = 0;
  int flaunch = 0;
  if (conf) {
    launch_vort_confine(s, e->nx, e->ny, e->h, u, v, L0.label, (float)e->prm.confinement, e->fx, e->fy);
    fbytes += 4 * F + N + 8 * N;
    flaunch += 1;
  }
  if (beta_on || alpha_on) wait_dye(e, s);
  if (beta_on || alpha_on || conf) {
    launch_forces(s, e->nx, e->ny, e->h, e->dnx, e->dny, e->dh, u, v, e->dye[par], L0.label, beta_on, alpha_on, conf,
                  e->fx, e->fy, e->sc);
    fbytes += 8 * F + N + (beta_on ? 4 * D : 0) + (alpha_on ? 4 * D : 0) + (conf ? 8 * N : 0);
    flaunch += 1;
  }
  prof_end(*e, tok, fbytes, flaunch);
  launch_fill32(s, e->acc, 4 * sizeof(double) / 4, 0u);  // b_sq, res_sq, n_fluid, n_res
  tok = prof_begin(*e, FL_PH_DIVERGENCE);
  launch_divergence(s, e->nx, e->ny, e->h, u, v, L0.b, e->prm.solver == FL_SOLVER_MG, L0.label, e->sc, e->acc,
                    step_mixed(e) ? e->b_lo : nullptr);
  prof_end(*e, tok, 4 * F + N + 4 * N, 1);
  wait_p(e, s);
  wait_codes(e, s);
  if (e->prm.warm_extrapolate && e->prm.solver == FL_SOLVER_MG) {
    const bool mixed = e->prm.mixed != 0;
    launch_extrapolate(s, e->cells(), L0.label, L0.x[0], e->pprev32, mixed ? e->p64[0] : nullptr,
                       mixed ? e->p64[1] : nullptr, e->pprev64, e->ctl, refined_df(e));
  }
  if (e->warm != nullptr && e->prm.solver == FL_SOLVER_MG) {
    // p_prev -> p_guess in place: the float64 pressure of the defect
    // correction, or the float32 warm start of the plain multigrid
    const bool mixed = e->prm.mixed != 0;
    tok = prof_begin(*e, FL_PH_WARM_START);
    unet_warm_start(*e->warm, s, e->nx, e->ny, L0.b, L0.label, e->acc, mixed ? nullptr : L0.x[0],
                    mixed ? e->p64[0] : nullptr, mixed ? e->p64[1] : nullptr, &e->ctl->par, e->ws_scales,
                    refined_df(e));
    prof_end(*e, tok, 0, 0);
  }
}

// Solve prologue: the float64 path's initial residual, then the begin test.
void enqueue_solve_prologue(Engine* e, cudaStream_t s, bool mixed, bool use_cond, cudaGraphConditionalHandle h) {
  Level& L0 = e->levels[0];
  if (mixed) {
    // the begin test runs in the pass's last block
    const int tok = prof_begin(*e, FL_PH_DEFECT64);
    launch_update_resid64(s, e->nx, e->ny, e->p64[0], e->p64[1], e->ctl, nullptr, L0.b, e->b_lo, L0.code, false,
                          e->r32, e->acc, refined_df(e), 1, use_cond, h);
    // p64, b, code in; r32 out
    prof_end(*e, tok, 17.0 * e->cells(), 1);
    return;
  }
  const int tok = prof_begin(*e, FL_PH_CONTROL);
  launch_solve_begin(s, e->acc, e->ctl, use_cond, h);
  prof_end(*e, tok, 0, 1);
}

// One multigrid cycle: a V-cycle on b (float32 path, warm start in
// levels[0].x[0], residual accumulated by its last kernel) or on the float64
// path's residual followed by p64 += e and the new float64 residual.
void enqueue_solve_body(Engine* e, cudaStream_t s, bool mixed, bool use_cond, cudaGraphConditionalHandle h) {
  Level& L0 = e->levels[0];
  if (mixed) {
    // the cycle test runs in the pass's last block
    mg_vcycle_on(*e, e->r32, true, nullptr);
    const int tok = prof_begin(*e, FL_PH_DEFECT64);
    launch_update_resid64(s, e->nx, e->ny, e->p64[0], e->p64[1], e->ctl, L0.x[0], L0.b, e->b_lo, L0.code, true,
                          e->r32, e->acc, refined_df(e), 2, use_cond, h);
    // p64, e, b, code in; p64 (other buffer), r32 out
    prof_end(*e, tok, 29.0 * e->cells(), 1);
    return;
  }
  mg_vcycle_on(*e, L0.b, false, e->acc);
  const int tok = prof_begin(*e, FL_PH_CONTROL);
  launch_solve_check(s, e->acc, e->ctl, use_cond, h);
  prof_end(*e, tok, 0, 1);
}

void enqueue_solve_epilogue(Engine* e, cudaStream_t s, bool mixed) {
  const int tok = prof_begin(*e, FL_PH_CONTROL);
  launch_zero_if(s, e->ctl, mixed ? nullptr : e->levels[0].x[0], mixed ? e->p64[0] : nullptr,
                 mixed ? e->p64[1] : nullptr, e->cells());
  prof_end(*e, tok, 0, 1);
}

// Red-black SOR with a fixed budget (tol <= 0, the reference's browser
// setting): sweep pairs grouped up to four per launch, scale read from the
// step's scalars on the device, result back in levels[0].x[0].
void enqueue_rb_fixed(Engine* e, cudaStream_t s) {
  Level& L = e->levels[0];
  launch_solve_begin(s, e->acc, e->ctl, false, 0);
  int k = 0, src = 0;
  const int iters = e->prm.pressure_iters;
  const int per = e->prm.rb_pairs > 0 ? e->prm.rb_pairs : 4;
  while (k < iters) {
    const int chunk = std::min(per, iters - k);
    const int tok = prof_begin(*e, FL_PH_RB_SWEEPS);
    launch_rb_sweeps(s, L.nx, L.ny, L.x[src], L.x[1 - src], L.b, L.code, 0.0f, (float)e->prm.omega, chunk,
                     &e->sc->scale);
    prof_end(*e, tok, 13.0 * e->cells(), 1);
    src = 1 - src;
    k += chunk;
  }
  if (src == 1) launch_copy32(s, L.x[1], L.x[0], e->cells());
  launch_zero_if(s, e->ctl, L.x[0], nullptr, nullptr, e->cells());
}

// subtract gradient + outflow -> dye (advect, decay, inlet) -> CFL
cudaError_t enqueue_post(Engine* e, cudaStream_t s, int par, bool device_dt) {
  Level& L0 = e->levels[0];
  const int mac = e->prm.scheme == FL_MACCORMACK;
  const double N = (double)e->cells(), F = (double)(e->ufaces() + e->vfaces()), D = (double)e->dye_cells();
  const bool mixed = step_mixed(e);
  float* u = e->u[1 - par];
  float* v = e->v[1 - par];
  int tok = prof_begin(*e, FL_PH_PROJECT);
  launch_subtract_outflow(s, e->nx, e->ny, L0.x[0], u, v, L0.label, e->sc, true, true, mixed ? e->p64[0] : nullptr,
                          mixed ? e->p64[1] : nullptr, e->ctl, refined_df(e), mixed ? e->p32_final : nullptr);
  prof_end(*e, tok, (mixed ? 8 + 4 : 4) * N + 4 * F + N + 4 * F, 1);
  // velocity and pressure are final: fl_step_host reads them back from here
  // on while the dye advection runs
  cudaEventRecordWithFlags(e->ev_proj, s, capturing(s) ? cudaEventRecordExternal : 0);
  wait_dye(e, s);
  tok = prof_begin(*e, FL_PH_ADVECT_DYE);
  launch_advect_dye(s, e->nx, e->ny, e->h, e->dnx, e->dny, e->dh, mac, u, v, e->dye[par], e->dye_hat, e->dye[1 - par],
                    L0.label, e->sc, true, e->patch, e->pi0, e->pj0, e->pnx, e->pny, e->bt_d);
  // forward: u,v + 3 planes + label in, 3 planes out (MacCormack: + backtrace
  // positions out); correction adds the hat planes and the positions
  prof_end(*e, tok, mac ? (4 * F + 32 * D + N) + (4 * F + 44 * D + N) : 4 * F + 24 * D + N, mac ? 2 : 1);
  // the dye is final: fl_step_host reads it back from here on
  cudaEventRecordWithFlags(e->ev_dye_done, s, capturing(s) ? cudaEventRecordExternal : 0);
  tok = prof_begin(*e, FL_PH_CFL);
  if (e->prm.residual_every > 0) {
    // with the residual diagnostic (simulation.ts:539-540) on its cadence
    launch_cfl_residual(s, e->nx, e->ny, e->h, u, v, e->div_post, L0.label, e->prm.residual_every, e->diag, e->acc,
                        e->sc, e->time_dev, &e->prm, device_dt, device_dt);
    // u, v in; on diagnostic steps labels in and the divergence out
    prof_end(*e, tok, 4 * F + N + 4 * N, 1);
  } else {
    launch_max_speed(s, e->nx, e->ny, u, v, e->acc, e->sc, e->time_dev, &e->prm, e->h, device_dt, device_dt);
    prof_end(*e, tok, 4 * F, 1);
  }
  return cudaSuccess;
}

// Red-black SOR to a tolerance (pressureRedBlack.ts:88-113): checked every
// 12 sweeps on the host, pairs grouped up to four per launch and never
// across a check.
int rb_solve_device(Engine* e, float scale, int iterations, float omega, double tol, double div_rms, int* used) {
  Level& L = e->levels[0];
  *used = iterations;
  const double target = tol > 0 ? tol * div_rms : -1;
  int k = 0;
  int src = 0;
  const int per = e->prm.rb_pairs > 0 ? e->prm.rb_pairs : 4;
  while (k < iterations) {
    int chunk = std::min(per, iterations - k);
    if (target >= 0) chunk = std::min(chunk, 12 - (k % 12));
    const int tok = prof_begin(*e, FL_PH_RB_SWEEPS);
    launch_rb_sweeps(e->stream, L.nx, L.ny, L.x[src], L.x[1 - src], L.b, L.code, scale, omega, chunk);
    prof_end(*e, tok, 13.0 * e->cells(), 1);
    TRY(check_launch(e, "red-black sweeps"));
    src = 1 - src;
    k += chunk;
    if (target >= 0 && k % 12 == 0) {
      TRY(zero_residual_accum(e));
      launch_rms_remaining(e->stream, L.nx, L.ny, L.x[src], L.b, L.code, scale, e->acc);
      TRY(check_launch(e, "residual"));
      TRY(read_accum(e));
      const double r = rms(e->acc_host->res_sq, e->acc_host->n_res);
      e->last_relres = div_rms > 0 ? r / div_rms : 0;
      if (r <= target) {
        *used = k;
        break;
      }
    }
  }
  if (src == 1)
    TRY(cuda_status(e, cudaMemcpyAsync(L.x[0], L.x[1], e->cells() * sizeof(float), cudaMemcpyDeviceToDevice, e->stream),
                    "p copy"));
  return FL_OK;
}

// The multigrid solve, eager: the same kernels as the graph's, with the host
// reading the device's decision after each cycle.
int solve_mg_eager(Engine* e, bool mixed, int max_cycles) {
  cudaStream_t s = e->stream;
  enqueue_solve_prologue(e, s, mixed, false, 0);
  TRY(check_launch(e, "solve"));
  for (int guard = 0; guard <= max_cycles + 1; guard++) {
    TRY(read_ctl(e));
    if (e->ctl_host->nonfinite)
      return fail(e, FL_ENONFINITE, "non-finite %s", e->ctl_host->cycles ? "residual" : "divergence");
    if (!e->ctl_host->cont) break;
    enqueue_solve_body(e, s, mixed, false, 0);
    TRY(check_launch(e, "V-cycle"));
  }
  enqueue_solve_epilogue(e, s, mixed);
  return check_launch(e, "solve");
}

// One step, eager. device_dt: scalars from the previous CFL reduction;
// otherwise the caller put them in e->sc.
int step_eager(Engine* e, bool device_dt) {
  cudaStream_t s = e->stream;
  Level& L0 = e->levels[0];
  const int par = e->cur;
  if (e->labels_dirty) {
    const bool mixed = step_mixed(e);
    launch_commit_labels(s, e->nx, e->ny, L0.label, L0.x[0], e->u[par], e->v[par], e->dye[par], e->dye_cells(),
                         mixed ? e->p64[0] : nullptr, mixed ? e->p64[1] : nullptr, e->ctl);
    mg_build_codes(*e);
    TRY(check_launch(e, "commit labels"));
    e->labels_dirty = false;
  }
  if (e->pending.size() > 8192) prof_drain(*e);
  enqueue_pre(e, s, par, e->stir_pending);
  e->stir_pending = false;
  TRY(check_launch(e, "advect / forces / divergence"));
  e->stats_on_device = solve_on_device(e);
  if (e->prm.solver == FL_SOLVER_MG) {
    TRY(solve_mg_eager(e, step_mixed(e), e->prm.mg_max_cycles));
  } else if (e->prm.tol <= 0) {
    enqueue_rb_fixed(e, s);
  } else {
    TRY(read_accum(e));
    const double div_rms = rms(e->acc_host->b_sq, e->acc_host->n_fluid);
    e->last_div_rms = div_rms;
    StepScalars hs;
    TRY(cuda_status(e, cudaMemcpyAsync(&hs, e->sc, sizeof hs, cudaMemcpyDeviceToHost, s), "read scalars"));
    TRY(sync(e, "read scalars"));
    int iters = 0;
    if (div_rms == 0)
      TRY(cuda_status(e, cudaMemsetAsync(L0.x[0], 0, e->cells() * sizeof(float), s), "zero p"));
    else
      TRY(rb_solve_device(e, hs.scale, e->prm.pressure_iters, (float)e->prm.omega, e->prm.tol, div_rms, &iters));
    e->last_iters = iters;
  }
  TRY(cuda_status(e, enqueue_post(e, s, par, device_dt), "project / dye / CFL"));
  TRY(check_launch(e, "project / dye / CFL"));
  e->cur = 1 - par;
  e->steps++;
  return FL_OK;
}

void destroy_step_graphs(Engine* e) {
  for (auto& g : e->graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  for (auto& g : e->graph_up) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  e->graphs_valid = false;
  e->graph_gen++;
}

void destroy_graphs(Engine* e) {
  destroy_step_graphs(e);
  if (e->upload_graph) cudaGraphExecDestroy(e->upload_graph);
  e->upload_graph = nullptr;
  if (e->upload_graph_labels) cudaGraphExecDestroy(e->upload_graph_labels);
  e->upload_graph_labels = nullptr;
}

// Enqueues one whole step for buffer parity `par` on e->stream while that
// stream is being captured; the pressure solve becomes a WHILE node whose
// body is captured from e->stream2.
// cfl_first: led by the clock reset and the CFL scalars of the current
// velocity (the work an upload otherwise enqueues after its copies).
cudaError_t capture_step(Engine* e, int par, bool cfl_first) {
  cudaStream_t s = e->stream;
  cudaError_t err = cudaSuccess;
  if (cfl_first) {
    launch_fill32(s, e->time_dev, 2, 0u);
    launch_max_speed(s, e->nx, e->ny, e->u[par], e->v[par], e->acc, e->sc, e->time_dev, &e->prm, e->h, true, false);
  }
  enqueue_pre(e, s, par, false);
  if (e->prm.solver == FL_SOLVER_MG) {
    cudaStreamCaptureStatus cst;
    cudaGraph_t cap = nullptr;
    err = cudaStreamGetCaptureInfo(s, &cst, nullptr, &cap, nullptr, nullptr, nullptr);
    cudaGraphConditionalHandle h = 0;
    if (err == cudaSuccess) err = cudaGraphConditionalHandleCreate(&h, cap, 0, cudaGraphCondAssignDefault);
    if (err == cudaSuccess) {
      enqueue_solve_prologue(e, s, step_mixed(e), true, h);
      const cudaGraphNode_t* deps = nullptr;
      size_t ndeps = 0;
      err = cudaStreamGetCaptureInfo(s, &cst, nullptr, &cap, &deps, nullptr, &ndeps);
      cudaGraphNodeParams cp{};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t node = nullptr;
      if (err == cudaSuccess) err = cudaGraphAddNode(&node, cap, deps, nullptr, ndeps, &cp);
      if (err == cudaSuccess) err = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
      if (err == cudaSuccess) {
        // the body is captured from the second stream; the V-cycle launchers
        // enqueue on e->stream, so it points there meanwhile
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        e->stream = e->stream2;
        err = cudaStreamBeginCaptureToGraph(e->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (err == cudaSuccess) {
          enqueue_solve_body(e, e->stream, step_mixed(e), true, h);
          cudaGraph_t done = nullptr;
          err = cudaStreamEndCapture(e->stream, &done);
        }
        e->stream = s;
      }
    }
    if (err == cudaSuccess) enqueue_solve_epilogue(e, s, step_mixed(e));
  } else {
    enqueue_rb_fixed(e, s);
  }
  if (err == cudaSuccess) err = enqueue_post(e, s, par, true);
  return err;
}

// Captures the whole step for buffer parity `par` into an executable graph.
int build_graph(Engine* e, int par, cudaGraphExec_t* out, bool cfl_first = false) {
  cudaStream_t s = e->stream;
  cudaError_t err = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (err != cudaSuccess) return cuda_status(e, err, "begin capture");
  err = capture_step(e, par, cfl_first);
  cudaGraph_t graph = nullptr;
  cudaError_t end = cudaStreamEndCapture(s, &graph);
  if (err == cudaSuccess) err = end;
  if (err == cudaSuccess) err = cudaGetLastError();
  if (err == cudaSuccess) err = cudaGraphInstantiate(out, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (err != cudaSuccess) {
    cudaGetLastError();
    return cuda_status(e, err, "step graph");
  }
  return FL_OK;
}

bool graph_eligible(const Engine* e) {
  return e->use_graphs && !e->profiling && !e->stir_pending && !e->labels_dirty && solve_on_device(e);
}

// cfl_first: the step right after fl_step_host's upload, which left the
// clock reset and the CFL scalars to the step's graph.
int step_graph(Engine* e, bool cfl_first = false) {
  if (!e->graphs_valid) {
    destroy_step_graphs(e);
    for (int par = 0; par < 2; par++) TRY(build_graph(e, par, &e->graph[par]));
    e->graphs_valid = true;
  }
  cudaGraphExec_t& g = cfl_first ? e->graph_up[e->cur] : e->graph[e->cur];
  if (!g) TRY(build_graph(e, e->cur, &g, true));
  TRY(cuda_status(e, cudaGraphLaunch(g, e->stream), "graph launch"));
  e->cur = 1 - e->cur;
  e->steps++;
  e->stats_on_device = true;
  return FL_OK;
}

// Fills last_iters / last_relres / last_div_rms from the control block when
// the last solve ran under the device's control (synchronises).
int solve_stats(Engine* e, bool ctl_read = false) {
  if (!e->stats_on_device) return FL_OK;
  if (!ctl_read) TRY(read_ctl(e));
  const SolveCtl& c = *e->ctl_host;
  e->last_div_rms = c.b_rms;
  if (c.mode == SOLVE_RB) {
    e->last_iters = c.zero_p ? 0 : e->prm.pressure_iters;
    e->last_relres = -1;
  } else {
    e->last_iters = c.cycles;
    e->last_relres = c.rel;
  }
  e->last_relres0 = c.mode == SOLVE_MIXED ? c.rel0 : -1;
  if (c.nonfinite) return fail(e, FL_ENONFINITE, "non-finite %s", c.cycles ? "residual" : "divergence");
  if (e->warm != nullptr && unet_tc_take_error())
    return fail(e, FL_ETIMEOUT, "the warm start's tensor-core convolution gave up a bounded wait");
  return FL_OK;
}

}  // namespace

// ====================================================================== ABI

extern "C" {

void fl_default_params(fl_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->cfl_target = 2.0;
  p->dt_max = 1.0 / 30.0;
  p->rho = 1.0;
  p->scheme = FL_SEMI_LAGRANGIAN;
  p->solver = FL_SOLVER_MG;
  p->pressure_iters = 100;
  p->mg_max_cycles = 3;
  p->omega = 1.9;
  p->tol = 5e-3;
  p->mg_pre = 2;
  p->mg_post = 2;
  p->mg_coarse_sweeps = 8;
  p->mg_coarsest = 4;
  p->mg_omega = 1.0;
  p->residual_every = 1;  // simulation.ts:233
}

int fl_abi_version(void) { return FL_ABI_VERSION; }

const char* fl_last_error(const fl_engine* h) { return h ? h->e.err.c_str() : g_create_error.c_str(); }

int fl_create(int nx, int ny, double h, int dye_scale, const fl_params* params, int device, fl_engine** out) {
  if (!out) return fail(nullptr, FL_EINVAL, "null output pointer");
  *out = nullptr;
  if (nx < 2 || ny < 2 || nx > 32768 || ny > 32768) return fail(nullptr, FL_EINVAL, "grid %dx%d out of range", nx, ny);
  if (!(h > 0)) return fail(nullptr, FL_EINVAL, "cell size must be positive");
  if (dye_scale < 1 || dye_scale > 8) return fail(nullptr, FL_EINVAL, "dye_scale %d out of [1, 8]", dye_scale);
  // the samplers address one field with 32-bit offsets
  if ((long long)nx * dye_scale * ny * dye_scale >= (1LL << 31) || (long long)(nx + 1) * (ny + 1) >= (1LL << 31))
    return fail(nullptr, FL_EINVAL, "dye grid %dx%d too large (at most 2^31 - 1 cells)", nx * dye_scale,
                ny * dye_scale);
  int ndev = 0;
  cudaError_t err = cudaGetDeviceCount(&ndev);
  if (err != cudaSuccess || ndev == 0)
    return fail(nullptr, FL_EDEVICE, "no CUDA device (%s)", err != cudaSuccess ? cudaGetErrorString(err) : "count 0");
  if (device < 0 || device >= ndev) return fail(nullptr, FL_EINVAL, "device %d of %d", device, ndev);
  if (cudaSetDevice(device) != cudaSuccess) return fail(nullptr, FL_EDEVICE, "cudaSetDevice(%d) failed", device);

  fl_engine* H = new (std::nothrow) fl_engine();
  if (!H) return fail(nullptr, FL_ENOMEM, "host allocation");
  Engine* e = &H->e;
  e->device = device;
  e->nx = nx;
  e->ny = ny;
  e->dye_scale = dye_scale;
  e->dnx = nx * dye_scale;
  e->dny = ny * dye_scale;
  e->h = (float)h;
  e->dh = (float)(h / dye_scale);
  if (params) e->prm = *params; else fl_default_params(&e->prm);
  int st = validate_params(e, &e->prm);
  if (st) {
    g_create_error = e->err;
    delete H;
    return st;
  }
  auto bail = [&](int code) {
    g_create_error = e->err;
    free_all(e);
    delete H;
    return code;
  };
  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) {
    fail(e, FL_EDEVICE, "stream creation failed");
    return bail(FL_EDEVICE);
  }
  const size_t uf = (size_t)e->ufaces() * 4, vf = (size_t)e->vfaces() * 4, cf = (size_t)e->cells() * 4;
  const size_t df = (size_t)3 * e->dye_cells() * 4;
  e->staging_bytes = 2 * std::max(std::max(uf, vf), df);
  int s = FL_OK;
  s = s ? s : dalloc(e, (void**)&e->u[0], uf, "u");
  s = s ? s : dalloc(e, (void**)&e->u[1], uf, "u");
  s = s ? s : dalloc(e, (void**)&e->v[0], vf, "v");
  s = s ? s : dalloc(e, (void**)&e->v[1], vf, "v");
  s = s ? s : dalloc(e, (void**)&e->u_hat, uf, "u_hat");
  s = s ? s : dalloc(e, (void**)&e->v_hat, vf, "v_hat");
  s = s ? s : dalloc(e, (void**)&e->dye[0], df, "dye");
  s = s ? s : dalloc(e, (void**)&e->dye[1], df, "dye");
  s = s ? s : dalloc(e, (void**)&e->dye_hat, df, "dye_hat");
  s = s ? s : dalloc(e, (void**)&e->w, cf, "vorticity");
  s = s ? s : dalloc(e, (void**)&e->fx, cf, "force");
  s = s ? s : dalloc(e, (void**)&e->fy, cf, "force");
  s = s ? s : dalloc(e, (void**)&e->sc, sizeof(StepScalars), "scalars");
  s = s ? s : dalloc(e, (void**)&e->acc, sizeof(StepAccum), "accumulators");
  s = s ? s : dalloc(e, (void**)&e->time_dev, sizeof(double), "clock");
  s = s ? s : dalloc(e, &e->staging, e->staging_bytes, "staging");
  s = s ? s : dalloc(e, (void**)&e->p32_final, (size_t)e->cells() * sizeof(float), "rounded pressure");
  s = s ? s : dalloc(e, (void**)&e->p64[0], (size_t)e->cells() * 8, "p64");
  s = s ? s : dalloc(e, (void**)&e->p64[1], (size_t)e->cells() * 8, "p64");
  s = s ? s : dalloc(e, (void**)&e->r32, cf, "residual");
  s = s ? s : dalloc(e, (void**)&e->b_lo, cf, "rhs rounding error");
  s = s ? s : dalloc(e, (void**)&e->pprev32, cf, "previous pressure");
  s = s ? s : dalloc(e, (void**)&e->pprev64, (size_t)e->cells() * 8, "previous pressure");
  s = s ? s : dalloc(e, (void**)&e->bt_u, (size_t)e->ufaces() * sizeof(float2), "backtrace positions");
  s = s ? s : dalloc(e, (void**)&e->bt_v, (size_t)e->vfaces() * sizeof(float2), "backtrace positions");
  s = s ? s : dalloc(e, (void**)&e->bt_d, (size_t)e->dye_cells() * sizeof(float2), "backtrace positions");
  s = s ? s : dalloc(e, (void**)&e->ctl, sizeof(SolveCtl), "solve control");
  s = s ? s : dalloc(e, (void**)&e->ws_scales, 4 * sizeof(float), "warm-start scales");
  s = s ? s : dalloc(e, (void**)&e->label_in, (size_t)e->cells(), "uploaded labels");
  s = s ? s : dalloc(e, (void**)&e->label_flag, sizeof(int), "label flag");
  s = s ? s : dalloc(e, (void**)&e->div_post, cf, "post-step divergence");
  s = s ? s : dalloc(e, (void**)&e->diag, sizeof(DiagAccum), "residual diagnostic");
  if (s) return bail(s);
  {
    DiagAccum d0{};
    d0.last_step = -1;
    if (cudaMemset(e->label_flag, 0, sizeof(int)) != cudaSuccess || cudaMemset(e->div_post, 0, cf) != cudaSuccess ||
        cudaMemcpy(e->diag, &d0, sizeof d0, cudaMemcpyHostToDevice) != cudaSuccess) {
      fail(e, FL_EDEVICE, "label flag / diagnostic");
      return bail(FL_EDEVICE);
    }
  }
  if (cudaMallocHost(&e->acc_host, sizeof(StepAccum)) != cudaSuccess ||
      cudaMallocHost(&e->ctl_host, sizeof(SolveCtl)) != cudaSuccess ||
      cudaMallocHost(&e->diag_host, sizeof(DiagAccum)) != cudaSuccess) {
    fail(e, FL_ENOMEM, "pinned accumulator");
    return bail(FL_ENOMEM);
  }
  if (cudaStreamCreateWithFlags(&e->stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_dye, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_proj, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_dye_done, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_p, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_lab, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_lab_done, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_lab_sync, cudaEventDisableTiming) != cudaSuccess ||
      cudaStreamCreateWithFlags(&e->stream3, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->ev_prior, cudaEventDisableTiming) != cudaSuccess) {
    fail(e, FL_EDEVICE, "stream creation failed");
    return bail(FL_EDEVICE);
  }
  mg_setup(*e);
  uint8_t* label0 = nullptr;
  if (cuda_status(e, cudaGetLastError(), "multigrid levels")) return bail(FL_ENOMEM);
  s = dalloc(e, (void**)&label0, (size_t)e->cells(), "label");
  if (s) return bail(s);
  e->levels[0].label = label0;
  if (sync(e, "create")) return bail(FL_EDEVICE);
  if (put_step_ctl(e, true)) return bail(FL_EDEVICE);
  *out = H;
  return FL_OK;
}

int fl_destroy(fl_engine* h) {
  if (!h) return FL_OK;
  cudaSetDevice(h->e.device);
  cudaStreamSynchronize(h->e.stream);
  free_all(&h->e);
  delete h;
  return FL_OK;
}

int fl_set_params(fl_engine* h, const fl_params* p) {
  ENTER(h);
  if (!p) return fail(e, FL_EINVAL, "null params");
  TRY(validate_params(e, p));
  const bool reshape = p->mg_coarsest != e->prm.mg_coarsest || p->mg_tail_side != e->prm.mg_tail_side;
  e->prm = *p;
  destroy_graphs(e);
  TRY(put_step_ctl(e, false));
  if (reshape) {
    uint8_t* label0 = e->levels[0].label;
    float* p0 = nullptr;
    TRY(dalloc(e, (void**)&p0, (size_t)e->cells() * 4, "p"));
    cudaMemcpyAsync(p0, e->levels[0].x[0], (size_t)e->cells() * 4, cudaMemcpyDeviceToDevice, e->stream);
    TRY(sync(e, "set params"));
    e->levels[0].label = nullptr;
    mg_setup(*e);
    e->levels[0].label = label0;
    cudaMemcpyAsync(e->levels[0].x[0], p0, (size_t)e->cells() * 4, cudaMemcpyDeviceToDevice, e->stream);
    TRY(sync(e, "set params"));
    cudaFree(p0);
    mg_build_codes(*e);
  }
  // the CFL scalars depend on cfl_target / dt_max / decay / weights
  if (e->uploaded) {
    launch_max_speed(e->stream, e->nx, e->ny, e->u[e->cur], e->v[e->cur], e->acc, e->sc, e->time_dev, &e->prm, e->h,
                     true, false);
  }
  return sync(e, "set params");
}

void* fl_stream(fl_engine* h) { return h ? (void*)h->e.stream : nullptr; }

// Also reports what the last steps left for a synchronising call: a
// non-finite solve (FL_ENONFINITE) or a timed-out tensor-core wait of the
// warm start (FL_ETIMEOUT).
int fl_synchronize(fl_engine* h) {
  ENTER(h);
  TRY(sync(e, "synchronize"));
  return solve_stats(e);
}

// The device-side work of an upload once the fields have landed: p64 (the
// float64 pressure of the defect-correction solve) from the float32 p
// unless it came in float64, the second-order warm start's history, the
// multigrid labels and stencil codes, the clock and the CFL scalars.
// The labels arrive in label_in; k_label_sync copies the cells that changed
// into levels[0].label. Eagerly the multigrid labels and codes are rebuilt
// every time; captured (`capture`), the rebuild is the body of an IF node
// that runs only when some label changed (the caller forces it by filling
// levels[0].label with a value no label has, when the codes are stale).
// The pressure's part of it: the refined pressure from the float32 one (when
// it came as float32) and the warm-start history, on stream `s`.
void enqueue_p_after_upload(Engine* e, cudaStream_t s, bool p64_from_p32) {
  if (p64_from_p32) launch_convert(s, e->levels[0].x[0], FL_F32, e->p64[0], refined_df(e) ? DT_DF : FL_F64, e->cells());
  launch_copy32(s, e->levels[0].x[0], e->pprev32, e->cells());
  launch_copy32(s, e->p64[0], e->pprev64, 2 * e->cells());
}

cudaError_t enqueue_after_upload(Engine* e, bool p64_from_p32, bool capture) {
  cudaStream_t s = e->stream;
  cudaError_t err = cudaSuccess;
  enqueue_p_after_upload(e, s, p64_from_p32);
  launch_label_sync(s, e->label_in, e->levels[0].label, e->cells(), e->label_flag);
  if (!capture) {
    cudaMemsetAsync(e->label_flag, 0, sizeof(int), s);
    mg_build_codes(*e);
  } else {
    cudaStreamCaptureStatus cst;
    cudaGraph_t cap = nullptr;
    err = cudaStreamGetCaptureInfo(s, &cst, nullptr, &cap, nullptr, nullptr, nullptr);
    cudaGraphConditionalHandle h = 0;
    if (err == cudaSuccess) err = cudaGraphConditionalHandleCreate(&h, cap, 0, cudaGraphCondAssignDefault);
    if (err == cudaSuccess) {
      launch_label_cond(s, e->label_flag, h);
      const cudaGraphNode_t* deps = nullptr;
      size_t ndeps = 0;
      err = cudaStreamGetCaptureInfo(s, &cst, nullptr, &cap, &deps, nullptr, &ndeps);
      cudaGraphNodeParams cp{};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeIf;
      cp.conditional.size = 1;
      cudaGraphNode_t node = nullptr;
      if (err == cudaSuccess) err = cudaGraphAddNode(&node, cap, deps, nullptr, ndeps, &cp);
      if (err == cudaSuccess) err = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
      if (err == cudaSuccess) {
        // the body is captured from the second stream (mg_build_codes
        // enqueues on e->stream, which points there meanwhile)
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        e->stream = e->stream2;
        err = cudaStreamBeginCaptureToGraph(e->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (err == cudaSuccess) {
          mg_build_codes(*e);
          cudaGraph_t done = nullptr;
          err = cudaStreamEndCapture(e->stream, &done);
        }
        e->stream = s;
      }
    }
  }
  launch_fill32(s, e->time_dev, 2, 0u);
  launch_max_speed(s, e->nx, e->ny, e->u[0], e->v[0], e->acc, e->sc, e->time_dev, &e->prm, e->h, true, false);
  return err;
}

}  // extern "C"

namespace {

// The rebuild part of fl_step_host's upload as a graph on the third stream:
// the multigrid labels and codes rebuilt by kernels that run only when the
// label compare before them found a changed cell (a plain graph: an IF node
// here held up the engine stream's kernels meanwhile).
int label_graph(Engine* e) {
  if (e->upload_graph_labels) return FL_OK;
  cudaGraph_t g = nullptr;
  cudaError_t err = cudaStreamBeginCapture(e->stream3, cudaStreamCaptureModeThreadLocal);
  if (err == cudaSuccess) {
    mg_build_codes_if(*e, e->stream3, e->label_flag);
    err = cudaGetLastError();
    cudaError_t end = cudaStreamEndCapture(e->stream3, &g);
    if (err == cudaSuccess) err = end;
  }
  if (err == cudaSuccess) err = cudaGraphInstantiate(&e->upload_graph_labels, g, 0);
  if (g) cudaGraphDestroy(g);
  if (err != cudaSuccess) {
    cudaGetLastError();
    e->upload_graph_labels = nullptr;
    return cuda_status(e, err, "label graph");
  }
  return FL_OK;
}

// The body of fl_upload_fields. With `dye_async` the dye (float32) is copied
// on the second stream, after the stream's earlier work and the other
// fields' copies, and ev_dye marks its end; the step's first dye reader
// waits for it (wait_dye). Otherwise ev_dye is recorded on the second stream
// with nothing in flight. With cfl_deferred (fl_step_host's float32 upload),
// the clock reset and the CFL scalars are left to the caller (*cfl_deferred
// says so), which runs them at the head of the step's graph.
int upload_fields(Engine* e, int dtype, const void* u, const void* v, const void* p, const uint8_t* label,
                  const void* dye, bool dye_async, bool* cfl_deferred = nullptr) {
  if (cfl_deferred) *cfl_deferred = false;
  e->cur = 0;
  e->stats_on_device = false;
  if (dye_async && !dye) return fail(e, FL_EINVAL, "upload dye: null pointer");
  // fl_step_host's float32 upload, on three streams: the labels first, their
  // compare and the gated rebuild on the third stream while u and v arrive
  // on the engine's stream; the dye, then the pressure (and what is formed
  // from it) on the second stream behind u and v. The step (led by the CFL
  // scalars of the new velocity, cfl_deferred) starts once the finest labels
  // are compared and waits for the rest where it first reads each.
  const bool async_p = dye_async && dtype == FL_F32 && e->use_graphs;
  // stale codes (new levels, labels written by another entry point): every
  // cell is made to differ so that the rebuild runs. Read before a capture
  // of the rebuild, which marks the codes valid.
  const bool stale_codes = !e->codes_valid || e->labels_dirty;
  if (async_p) TRY(label_graph(e));
  TRY(put_step_ctl(e, true));
  if (async_p) {
    if (stale_codes)
      TRY(cuda_status(e, cudaMemsetAsync(e->levels[0].label, 0xff, (size_t)e->cells(), e->stream), "upload label"));
    TRY(up32(e, e->label_in, label, (size_t)e->cells(), "upload label"));
    TRY(cuda_status(e, cudaEventRecord(e->ev_lab, e->stream), "upload label"));
    TRY(cuda_status(e, cudaStreamWaitEvent(e->stream3, e->ev_lab, 0), "upload label"));
    launch_label_sync(e->stream3, e->label_in, e->levels[0].label, e->cells(), e->label_flag);
    TRY(check_launch(e, "upload label"));
    TRY(cuda_status(e, cudaEventRecord(e->ev_lab_sync, e->stream3), "upload label"));
    TRY(cuda_status(e, cudaGraphLaunch(e->upload_graph_labels, e->stream3), "label graph"));
    TRY(cuda_status(e, cudaEventRecord(e->ev_lab_done, e->stream3), "upload label"));
  }
  TRY(upload(e, e->u[0], u, e->ufaces(), dtype, "upload u"));
  TRY(upload(e, e->v[0], v, e->vfaces(), dtype, "upload v"));
  if (!async_p) {
    if (p)
      TRY(upload(e, e->levels[0].x[0], p, e->cells(), dtype, "upload p"));
    else
      TRY(cuda_status(e, cudaMemsetAsync(e->levels[0].x[0], 0, e->cells() * 4, e->stream), "zero p"));
  }
  const bool p64_direct = p && dtype == FL_F64;
  if (p64_direct && refined_df(e)) {
    // the double-float pairs from the float64 pressure
    TRY(cuda_status(e, cudaMemcpyAsync(e->staging, p, e->cells() * sizeof(double), cudaMemcpyHostToDevice, e->stream),
                    "upload p64"));
    launch_convert(e->stream, e->staging, FL_F64, e->p64[0], DT_DF, e->cells());
  } else if (p64_direct) {
    TRY(cuda_status(e, cudaMemcpyAsync(e->p64[0], p, e->cells() * sizeof(double), cudaMemcpyHostToDevice, e->stream),
                    "upload p64"));
  }
  if (!async_p) TRY(up32(e, e->label_in, label, (size_t)e->cells(), "upload label"));
  if (dye_async) {
    // after the copies the step starts with (which it would otherwise share
    // the host link with) and the stream's earlier work (which may still read
    // the dye and pressure buffers)
    TRY(cuda_status(e, cudaEventRecord(e->ev_prior, e->stream), "upload dye"));
    TRY(cuda_status(e, cudaStreamWaitEvent(e->stream2, e->ev_prior, 0), "upload dye"));
    // the dye first: the step's body forces read it before the solve reads p
    TRY(cuda_status(e, cudaMemcpyAsync(e->dye[0], dye, 3 * e->dye_cells() * sizeof(float), cudaMemcpyHostToDevice,
                                       e->stream2), "upload dye"));
    TRY(cuda_status(e, cudaEventRecord(e->ev_dye, e->stream2), "upload dye"));
    if (async_p) {
      if (p)
        TRY(cuda_status(e, cudaMemcpyAsync(e->levels[0].x[0], p, e->cells() * sizeof(float), cudaMemcpyHostToDevice,
                                           e->stream2), "upload p"));
      else
        TRY(cuda_status(e, cudaMemsetAsync(e->levels[0].x[0], 0, e->cells() * 4, e->stream2), "zero p"));
      enqueue_p_after_upload(e, e->stream2, true);
      TRY(check_launch(e, "upload p"));
    }
    TRY(cuda_status(e, cudaEventRecord(e->ev_p, e->stream2), "upload p"));
  } else {
    TRY(upload(e, e->dye[0], dye, 3 * e->dye_cells(), dtype, "upload dye"));
    TRY(cuda_status(e, cudaEventRecord(e->ev_dye, e->stream2), "upload dye"));
    TRY(cuda_status(e, cudaEventRecord(e->ev_p, e->stream2), "upload p"));
  }
  if (async_p) {
    // the clock and the first step's CFL scalars from the uploaded velocity
    // (here, or at the head of the caller's step graph); the step starts
    // once the finest labels are in place too (it waits for the rebuilt
    // codes where the solve first reads them)
    if (cfl_deferred) {
      *cfl_deferred = true;
    } else {
      launch_fill32(e->stream, e->time_dev, 2, 0u);
      launch_max_speed(e->stream, e->nx, e->ny, e->u[0], e->v[0], e->acc, e->sc, e->time_dev, &e->prm, e->h, true,
                       false);
    }
    TRY(cuda_status(e, cudaStreamWaitEvent(e->stream, e->ev_lab_sync, 0), "upload label"));
  } else {
    if (stale_codes)
      TRY(cuda_status(e, cudaMemsetAsync(e->levels[0].label, 0xff, (size_t)e->cells(), e->stream), "upload label"));
    if (p64_direct || !e->use_graphs) {
      TRY(cuda_status(e, enqueue_after_upload(e, !p64_direct, false), "upload"));
    } else {
      // one graph launch instead of ~20 launches (captured once per parameter
      // set); the label rebuild runs only when the labels changed
      if (!e->upload_graph) {
        cudaGraph_t g = nullptr;
        cudaError_t err = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal);
        if (err == cudaSuccess) {
          err = enqueue_after_upload(e, true, true);
          cudaError_t end = cudaStreamEndCapture(e->stream, &g);
          if (err == cudaSuccess) err = end;
        }
        if (err == cudaSuccess) err = cudaGraphInstantiate(&e->upload_graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (err != cudaSuccess) {
          cudaGetLastError();
          e->upload_graph = nullptr;
          return cuda_status(e, err, "upload graph");
        }
      }
      TRY(cuda_status(e, cudaGraphLaunch(e->upload_graph, e->stream), "upload graph"));
    }
  }
  TRY(check_launch(e, "upload"));
  e->codes_valid = true;
  e->uploaded = true;
  e->labels_dirty = false;
  e->steps = 0;
  e->time = 0;
  return FL_OK;
}

int sync2(Engine* e, const char* what) { return cuda_status(e, cudaStreamSynchronize(e->stream2), what); }

// fl_read_pressure's body: the refined pressure when there is one.
int read_pressure(Engine* e, int dtype, void* p) {
  if (step_mixed(e) && e->uploaded) {
    if (!p) return fail(e, FL_EINVAL, "read p: null pointer");
    if (dtype != FL_F32 && dtype != FL_F64) return fail(e, FL_EINVAL, "read p: dtype %d", dtype);
    const long n = e->cells();
    // the current float64 buffer is chosen on the device (no parity round trip)
    launch_select_p64(e->stream, e->ctl, e->p64[0], e->p64[1], e->staging, dtype == FL_F64, n, refined_df(e));
    TRY(check_launch(e, "read p"));
    TRY(cuda_status(e, cudaMemcpyAsync(p, e->staging, n * (dtype == FL_F64 ? sizeof(double) : sizeof(float)),
                                       cudaMemcpyDeviceToHost, e->stream),
                    "read p"));
    return sync(e, "read pressure");
  }
  TRY(download(e, p, e->levels[0].x[0], e->cells(), dtype, "read p"));
  return sync(e, "read pressure");
}

}  // namespace

extern "C" {

int fl_upload_fields(fl_engine* h, int dtype, const void* u, const void* v, const void* p, const uint8_t* label,
                     const void* dye) {
  ENTER(h);
  TRY(upload_fields(e, dtype, u, v, p, label, dye, false));
  return sync(e, "upload");
}

int fl_step_host(fl_engine* h, int dtype, const void* u, const void* v, const void* p, const uint8_t* label,
                 const void* dye, void* u_out, void* v_out, void* p_out, void* dye_out, int* iters) {
  ENTER(h);
  const bool upload_in = u != nullptr;
  if (dtype != FL_F32 && dtype != FL_F64) return fail(e, FL_EINVAL, "step_host: dtype %d", dtype);
  if (upload_in && (!v || !label || !dye)) return fail(e, FL_EINVAL, "step_host: u without v, label or dye");
  if (!upload_in && (v || p || label || dye)) return fail(e, FL_EINVAL, "step_host: inputs without u");
  if (!upload_in && !e->uploaded) return fail(e, FL_ESTATE, "step before fl_upload_fields");
  if (dtype == FL_F64) {
    // Float64Array fields: converted on the device around synchronous copies
    if (upload_in) TRY(upload_fields(e, FL_F64, u, v, p, label, dye, false));
    TRY(graph_eligible(e) ? step_graph(e) : step_eager(e, true));
    TRY(check_launch(e, "step"));
    if (u_out) TRY(download(e, u_out, e->u[e->cur], e->ufaces(), FL_F64, "read u"));
    if (v_out) TRY(download(e, v_out, e->v[e->cur], e->vfaces(), FL_F64, "read v"));
    if (p_out) TRY(read_pressure(e, FL_F64, p_out));
    if (dye_out) TRY(download(e, dye_out, e->dye[e->cur], 3 * e->dye_cells(), FL_F64, "read dye"));
    TRY(sync(e, "step"));
    TRY(solve_stats(e));
    if (iters) *iters = e->last_iters;
    return FL_OK;
  }
  bool cfl_first = false;
  if (upload_in) {
    TRY(upload_fields(e, FL_F32, u, v, p, label, dye, true, &cfl_first));
  } else {
    TRY(cuda_status(e, cudaEventRecord(e->ev_dye, e->stream2), "step"));
  }
  if (graph_eligible(e)) {
    TRY(step_graph(e, cfl_first));
  } else {
    if (cfl_first) {
      launch_fill32(e->stream, e->time_dev, 2, 0u);
      launch_max_speed(e->stream, e->nx, e->ny, e->u[e->cur], e->v[e->cur], e->acc, e->sc, e->time_dev, &e->prm, e->h,
                       true, false);
    }
    TRY(step_eager(e, true));
  }
  TRY(check_launch(e, "step"));
  // velocity and pressure on the second stream once the projection is done
  // (the step records ev_proj there), the dye once the dye advection is done
  TRY(cuda_status(e, cudaStreamWaitEvent(e->stream2, e->ev_proj, 0), "read back"));
  if (u_out)
    TRY(cuda_status(e, cudaMemcpyAsync(u_out, e->u[e->cur], e->ufaces() * sizeof(float), cudaMemcpyDeviceToHost,
                                       e->stream2), "read u"));
  if (v_out)
    TRY(cuda_status(e, cudaMemcpyAsync(v_out, e->v[e->cur], e->vfaces() * sizeof(float), cudaMemcpyDeviceToHost,
                                       e->stream2), "read v"));
  if (p_out) {
    const long n = e->cells();
    if (step_mixed(e)) {
      // rounded to float by the projection
      TRY(cuda_status(e, cudaMemcpyAsync(p_out, e->p32_final, n * sizeof(float), cudaMemcpyDeviceToHost,
                                         e->stream2), "read p"));
    } else {
      TRY(cuda_status(e, cudaMemcpyAsync(p_out, e->levels[0].x[0], n * sizeof(float), cudaMemcpyDeviceToHost,
                                         e->stream2), "read p"));
    }
  }
  if (dye_out) {
    // on the second stream once the dye advection is done (the step records
    // ev_dye_done there), overlapping the CFL scan
    TRY(cuda_status(e, cudaStreamWaitEvent(e->stream2, e->ev_dye_done, 0), "read back"));
    TRY(cuda_status(e, cudaMemcpyAsync(dye_out, e->dye[e->cur], 3 * e->dye_cells() * sizeof(float),
                                       cudaMemcpyDeviceToHost, e->stream2), "read dye"));
  }
  // the solve's control block comes back with the step (one synchronisation)
  const bool ctl_read = e->stats_on_device;
  if (ctl_read)
    TRY(cuda_status(e, cudaMemcpyAsync(e->ctl_host, e->ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, e->stream),
                    "read solve state"));
  TRY(sync2(e, "read back"));
  TRY(sync(e, "step"));
  TRY(solve_stats(e, ctl_read));
  if (iters) *iters = e->last_iters;
  return FL_OK;
}

int fl_set_labels(fl_engine* h, const uint8_t* label) {
  ENTER(h);
  TRY(put_labels(e, label, "upload label"));
  e->labels_dirty = true;
  return sync(e, "set labels");
}

int fl_set_dye_patch(fl_engine* h, int i0, int j0, int pnx, int pny, const float* data) {
  ENTER(h);
  cudaFree(e->patch);
  e->patch = nullptr;
  e->pnx = e->pny = 0;
  destroy_graphs(e);
  if (!data) return FL_OK;
  if (pnx <= 0 || pny <= 0) return fail(e, FL_EINVAL, "patch %dx%d", pnx, pny);
  const size_t bytes = (size_t)4 * pnx * pny * sizeof(float);
  TRY(dalloc(e, (void**)&e->patch, bytes, "patch"));
  TRY(up32(e, e->patch, data, bytes, "upload patch"));
  e->pi0 = i0;
  e->pj0 = j0;
  e->pnx = pnx;
  e->pny = pny;
  return sync(e, "set patch");
}

int fl_set_buoyancy(fl_engine* h, double beta, double alpha) {
  ENTER(h);
  e->prm.beta = beta;
  e->prm.alpha = alpha;
  destroy_graphs(e);
  if (e->uploaded)
    launch_max_speed(e->stream, e->nx, e->ny, e->u[e->cur], e->v[e->cur], e->acc, e->sc, e->time_dev, &e->prm, e->h,
                     true, false);
  return sync(e, "set buoyancy");
}

int fl_set_confinement(fl_engine* h, double eps) {
  ENTER(h);
  e->prm.confinement = eps;
  destroy_graphs(e);
  return FL_OK;
}

int fl_set_stir(fl_engine* h, const double* st) {
  ENTER(h);
  e->stir_pending = st != nullptr;
  if (st)
    for (int k = 0; k < 5; k++) e->stir[k] = (float)st[k];
  return FL_OK;
}

int fl_step(fl_engine* h, int scheme, double dt, double scale, double grad_scale, const double keep[3], int* iters) {
  ENTER(h);
  if (!e->uploaded) return fail(e, FL_ESTATE, "step before fl_upload_fields");
  if (scheme != FL_SEMI_LAGRANGIAN && scheme != FL_MACCORMACK) return fail(e, FL_EINVAL, "scheme %d", scheme);
  if (!(dt > 0)) return fail(e, FL_EINVAL, "dt must be positive");
  if (scheme != e->prm.scheme) {
    // the seam passes the scheme per step; the captured step graphs hold the old one
    e->prm.scheme = scheme;
    destroy_step_graphs(e);
  }
  TRY(put_scalars(e, host_scalars(e, (float)dt, (float)scale, (float)grad_scale, keep)));
  TRY(step_eager(e, false));
  e->time += dt;
  TRY(sync(e, "step"));
  TRY(solve_stats(e));
  if (iters) *iters = e->last_iters;
  return FL_OK;
}

int fl_step_auto(fl_engine* h, int nsteps, int* iters_last) {
  ENTER(h);
  if (!e->uploaded) return fail(e, FL_ESTATE, "step before fl_upload_fields");
  if (nsteps < 0) return fail(e, FL_EINVAL, "nsteps < 0");
  for (int n = 0; n < nsteps; n++) TRY(graph_eligible(e) ? step_graph(e) : step_eager(e, true));
  if (iters_last) {
    TRY(solve_stats(e));
    *iters_last = e->last_iters;
  }
  return check_launch(e, "step");
}

int fl_get_stats(fl_engine* h, fl_stats* out) {
  ENTER(h);
  if (!out) return fail(e, FL_EINVAL, "null stats");
  StepScalars s;
  double t = 0;
  TRY(sync(e, "stats"));
  TRY(cuda_status(e, cudaMemcpy(&s, e->sc, sizeof s, cudaMemcpyDeviceToHost), "stats"));
  TRY(cuda_status(e, cudaMemcpy(&t, e->time_dev, sizeof t, cudaMemcpyDeviceToHost), "stats"));
  TRY(read_accum(e));
  const int st = solve_stats(e);
  if (st && st != FL_ENONFINITE) return st;
  std::memset(out, 0, sizeof *out);
  out->dt = s.dt;
  out->scale = s.scale;
  out->grad_scale = s.grad_scale;
  out->time = e->time > 0 ? e->time : t;
  out->cycles = e->last_iters;
  out->steps = e->steps;
  out->rel_residual = e->last_relres;
  out->div_rms = e->last_div_rms;
  unsigned int bits = e->acc_host->last_max_bits;
  float m;
  std::memcpy(&m, &bits, 4);
  out->max_face_speed = m;
  TRY(cuda_status(e, cudaMemcpyAsync(e->diag_host, e->diag, sizeof(DiagAccum), cudaMemcpyDeviceToHost, e->stream),
                  "stats"));
  TRY(sync(e, "stats"));
  const DiagAccum& d = *e->diag_host;
  out->post_div_step = d.last_step;
  out->initial_rel_residual = e->last_relres0;
  out->post_div_rms = d.last_step >= 0 ? rms(d.last_sq, d.last_n) : 0.0;
  std::memcpy(&m, &d.last_max_bits, 4);
  out->post_div_max = d.last_step >= 0 ? m : 0.0;
  return FL_OK;
}

int fl_read_divergence(fl_engine* h, int dtype, void* div) {
  ENTER(h);
  TRY(download(e, div, e->div_post, e->cells(), dtype, "read divergence"));
  return sync(e, "read divergence");
}

int fl_read_velocity(fl_engine* h, int dtype, void* u, void* v) {
  ENTER(h);
  TRY(download(e, u, e->u[e->cur], e->ufaces(), dtype, "read u"));
  TRY(download(e, v, e->v[e->cur], e->vfaces(), dtype, "read v"));
  return sync(e, "read velocity");
}

int fl_read_dye(fl_engine* h, int dtype, void* dye) {
  ENTER(h);
  TRY(download(e, dye, e->dye[e->cur], 3 * e->dye_cells(), dtype, "read dye"));
  return sync(e, "read dye");
}

int fl_read_pressure(fl_engine* h, int dtype, void* p) {
  ENTER(h);
  return read_pressure(e, dtype, p);
}

int fl_profile_enable(fl_engine* h, int on) {
  ENTER(h);
  prof_drain(*e);
  for (int k = 0; k < FL_PHASES; k++) {
    e->prof_ms[k] = 0;
    e->prof_bytes[k] = 0;
    e->prof_launches[k] = 0;
  }
  e->profiling = on != 0;
  return FL_OK;
}

int fl_profile_read(fl_engine* h, fl_profile* out) {
  ENTER(h);
  if (!out) return fail(e, FL_EINVAL, "null profile");
  prof_drain(*e);
  for (int k = 0; k < FL_PHASES; k++) {
    out->ms[k] = e->prof_ms[k];
    out->bytes[k] = e->prof_bytes[k];
    out->launches[k] = e->prof_launches[k];
  }
  return check_launch(e, "profile");
}

// ----------------------------------------------------------- Advector seam

int fl_advect_velocity(fl_engine* h, int scheme, const float* u_in, const float* v_in, float* u_out, float* v_out,
                       const uint8_t* label, float dt) {
  ENTER(h);
  e->uploaded = false;
  TRY(up32(e, e->u[0], u_in, e->ufaces() * 4, "u"));
  TRY(up32(e, e->v[0], v_in, e->vfaces() * 4, "v"));
  TRY(put_labels(e, label, "label"));
  TRY(put_scalars(e, host_scalars(e, dt, 0, 0, nullptr)));
  launch_advect_velocity(e->stream, e->nx, e->ny, e->h, scheme == FL_MACCORMACK, e->u[0], e->v[0], e->u_hat,
                         e->v_hat, e->u[1], e->v[1], e->levels[0].label, e->sc);
  TRY(check_launch(e, "advect velocity"));
  TRY(down32(e, u_out, e->u[1], e->ufaces() * 4, "u"));
  TRY(down32(e, v_out, e->v[1], e->vfaces() * 4, "v"));
  return sync(e, "advect velocity");
}

int fl_advect_dye(fl_engine* h, int scheme, const float* u, const float* v, const float* const* q_in,
                  float* const* q_out, const uint8_t* label, float dt) {
  ENTER(h);
  if (!q_in || !q_out) return fail(e, FL_EINVAL, "advect dye: null plane array");
  e->uploaded = false;
  TRY(up32(e, e->u[0], u, e->ufaces() * 4, "u"));
  TRY(up32(e, e->v[0], v, e->vfaces() * 4, "v"));
  // the planes land end to end, the layout the kernels read
  for (int c = 0; c < 3; c++) TRY(up32(e, e->dye[0] + (size_t)c * e->dye_cells(), q_in[c], e->dye_cells() * 4, "dye"));
  TRY(put_labels(e, label, "label"));
  TRY(put_scalars(e, host_scalars(e, dt, 0, 0, nullptr)));
  launch_advect_dye(e->stream, e->nx, e->ny, e->h, e->dnx, e->dny, e->dh, scheme == FL_MACCORMACK, e->u[0], e->v[0],
                    e->dye[0], e->dye_hat, e->dye[1], e->levels[0].label, e->sc, false, nullptr, 0, 0, 0, 0);
  TRY(check_launch(e, "advect dye"));
  for (int c = 0; c < 3; c++) TRY(down32(e, q_out[c], e->dye[1] + (size_t)c * e->dye_cells(), e->dye_cells() * 4, "dye"));
  return sync(e, "advect dye");
}

// ------------------------------------------------------ PressureSolver seam

int fl_rb_solve(fl_engine* h, float* p, const float* div, const uint8_t* label, float scale, int iterations,
                float omega, double tol, int* used) {
  ENTER(h);
  e->uploaded = false;
  if (!p || !div || !label) return fail(e, FL_EINVAL, "null pointer");
  const long n = e->cells();
  // pressureRedBlack.ts:335-339 — zero divergence: p = 0, no sweeps.
  const double div_rms = host_fluid_div_rms(div, label, n);
  e->stats_on_device = false;
  e->last_div_rms = div_rms;
  e->last_relres = div_rms == 0 ? 0.0 : -1.0;
  e->last_iters = 0;
  if (used) *used = 0;
  if (div_rms == 0) {
    std::memset(p, 0, n * sizeof(float));
    return FL_OK;
  }
  if (iterations <= 0) return FL_OK;
  Level& L = e->levels[0];
  TRY(up32(e, L.x[0], p, n * 4, "p"));
  TRY(up32(e, L.b, div, n * 4, "div"));
  TRY(put_labels(e, label, "label"));
  launch_build_codes(e->stream, L.nx, L.ny, L.label, L.code);
  e->codes_valid = false;
  int u = 0;
  TRY(rb_solve_device(e, scale, iterations, omega, tol, div_rms, &u));
  e->last_iters = u;
  if (used) *used = u;
  TRY(down32(e, p, L.x[0], n * 4, "p"));
  return sync(e, "rb solve");
}

int fl_mg_solve(fl_engine* h, float* p, const float* div, const uint8_t* label, float scale, int max_cycles,
                double tol, int* cycles_used, double* rel_residual) {
  ENTER(h);
  e->uploaded = false;
  if (!p || !div || !label) return fail(e, FL_EINVAL, "null pointer");
  const long n = e->cells();
  Level& L = e->levels[0];
  TRY(up32(e, L.x[0], p, n * 4, "p"));
  TRY(up32(e, e->u_hat, div, n * 4, "div"));  // u_hat is free scratch of >= n floats here
  TRY(put_labels(e, label, "label"));
  mg_build_codes(*e);
  TRY(zero_solve_accum(e));
  launch_scale_rhs(e->stream, n, e->u_hat, L.b, -scale, L.label, e->acc, e->b_lo);
  TRY(check_launch(e, "rhs"));
  TRY(put_ctl(e, SOLVE_MG, tol, max_cycles, true));
  e->stats_on_device = true;
  TRY(solve_mg_eager(e, false, max_cycles));
  if (cycles_used) *cycles_used = e->ctl_host->cycles;
  if (rel_residual) *rel_residual = e->ctl_host->rel;
  TRY(down32(e, p, L.x[0], n * 4, "p"));
  return sync(e, "mg solve");
}

int fl_mg_solve_mixed(fl_engine* h, double* p, const float* div, const uint8_t* label, float scale, int max_cycles,
                      double tol, int* cycles_used, double* rel_residual) {
  ENTER(h);
  e->uploaded = false;
  if (!p || !div || !label) return fail(e, FL_EINVAL, "null pointer");
  const long n = e->cells();
  Level& L = e->levels[0];
  TRY(put_ctl(e, SOLVE_MIXED, tol, max_cycles, true));
  e->stats_on_device = true;
  if (refined_df(e)) {
    TRY(cuda_status(e, cudaMemcpyAsync(e->staging, p, n * sizeof(double), cudaMemcpyHostToDevice, e->stream), "p"));
    launch_convert(e->stream, e->staging, FL_F64, e->p64[0], DT_DF, n);
  } else {
    TRY(cuda_status(e, cudaMemcpyAsync(e->p64[0], p, n * sizeof(double), cudaMemcpyHostToDevice, e->stream), "p"));
  }
  TRY(up32(e, e->u_hat, div, n * 4, "div"));
  TRY(put_labels(e, label, "label"));
  mg_build_codes(*e);
  TRY(zero_solve_accum(e));
  launch_scale_rhs(e->stream, n, e->u_hat, L.b, -scale, L.label, e->acc, e->b_lo);
  TRY(check_launch(e, "rhs"));
  TRY(solve_mg_eager(e, true, max_cycles));
  TRY(read_ctl(e));
  if (cycles_used) *cycles_used = e->ctl_host->cycles;
  if (rel_residual) *rel_residual = e->ctl_host->rel;
  if (refined_df(e)) {
    launch_select_p64(e->stream, e->ctl, e->p64[0], e->p64[1], e->staging, true, n, true);
    TRY(check_launch(e, "p"));
    TRY(cuda_status(e, cudaMemcpyAsync(p, e->staging, n * sizeof(double), cudaMemcpyDeviceToHost, e->stream), "p"));
  } else {
    TRY(cuda_status(e, cudaMemcpyAsync(p, e->p64[e->ctl_host->par], n * sizeof(double), cudaMemcpyDeviceToHost,
                                       e->stream), "p"));
  }
  return sync(e, "mg solve mixed");
}

// ------------------------------------------------------------ single passes

int fl_divergence(fl_engine* h, const float* u, const float* v, float* div) {
  ENTER(h);
  e->uploaded = false;
  TRY(up32(e, e->u[0], u, e->ufaces() * 4, "u"));
  TRY(up32(e, e->v[0], v, e->vfaces() * 4, "v"));
  launch_divergence(e->stream, e->nx, e->ny, e->h, e->u[0], e->v[0], e->levels[0].b, false, nullptr, e->sc, nullptr);
  TRY(check_launch(e, "divergence"));
  TRY(down32(e, div, e->levels[0].b, e->cells() * 4, "div"));
  return sync(e, "divergence");
}

int fl_rb_sweep(fl_engine* h, float* p, const float* div, const uint8_t* label, float scale, float omega, int color) {
  ENTER(h);
  e->uploaded = false;
  if (color != 0 && color != 1) return fail(e, FL_EINVAL, "color %d", color);
  Level& L = e->levels[0];
  const long n = e->cells();
  TRY(up32(e, L.x[0], p, n * 4, "p"));
  TRY(up32(e, L.b, div, n * 4, "div"));
  TRY(put_labels(e, label, "label"));
  launch_build_codes(e->stream, L.nx, L.ny, L.label, L.code);
  e->codes_valid = false;
  launch_rb_halfsweep(e->stream, L.nx, L.ny, L.x[0], L.b, L.code, scale, omega, color);
  TRY(check_launch(e, "rb sweep"));
  TRY(down32(e, p, L.x[0], n * 4, "p"));
  return sync(e, "rb sweep");
}

int fl_subtract_gradient(fl_engine* h, const float* p, float* u, float* v, const uint8_t* label, float grad_scale) {
  ENTER(h);
  e->uploaded = false;
  Level& L = e->levels[0];
  TRY(up32(e, L.x[0], p, e->cells() * 4, "p"));
  TRY(up32(e, e->u[0], u, e->ufaces() * 4, "u"));
  TRY(up32(e, e->v[0], v, e->vfaces() * 4, "v"));
  TRY(put_labels(e, label, "label"));
  TRY(put_scalars(e, host_scalars(e, 1.0f, 1.0f, grad_scale, nullptr)));
  launch_subtract_outflow(e->stream, e->nx, e->ny, L.x[0], e->u[0], e->v[0], L.label, e->sc, true, false);
  TRY(check_launch(e, "subtract gradient"));
  TRY(down32(e, u, e->u[0], e->ufaces() * 4, "u"));
  TRY(down32(e, v, e->v[0], e->vfaces() * 4, "v"));
  return sync(e, "subtract gradient");
}

int fl_outflow(fl_engine* h, float* u, float* v, const uint8_t* label) {
  ENTER(h);
  e->uploaded = false;
  Level& L = e->levels[0];
  TRY(up32(e, e->u[0], u, e->ufaces() * 4, "u"));
  TRY(up32(e, e->v[0], v, e->vfaces() * 4, "v"));
  TRY(put_labels(e, label, "label"));
  launch_subtract_outflow(e->stream, e->nx, e->ny, L.x[0], e->u[0], e->v[0], L.label, e->sc, false, true);
  TRY(check_launch(e, "outflow"));
  TRY(down32(e, u, e->u[0], e->ufaces() * 4, "u"));
  TRY(down32(e, v, e->v[0], e->vfaces() * 4, "v"));
  return sync(e, "outflow");
}

int fl_commit_labels(fl_engine* h, float* p, float* u, float* v, float* dye, const uint8_t* label) {
  ENTER(h);
  e->uploaded = false;
  Level& L = e->levels[0];
  TRY(up32(e, L.x[0], p, e->cells() * 4, "p"));
  TRY(up32(e, e->u[0], u, e->ufaces() * 4, "u"));
  TRY(up32(e, e->v[0], v, e->vfaces() * 4, "v"));
  TRY(up32(e, e->dye[0], dye, 3 * e->dye_cells() * 4, "dye"));
  TRY(put_labels(e, label, "label"));
  launch_commit_labels(e->stream, e->nx, e->ny, L.label, L.x[0], e->u[0], e->v[0], e->dye[0], e->dye_cells());
  TRY(check_launch(e, "commit labels"));
  TRY(down32(e, p, L.x[0], e->cells() * 4, "p"));
  TRY(down32(e, u, e->u[0], e->ufaces() * 4, "u"));
  TRY(down32(e, v, e->v[0], e->vfaces() * 4, "v"));
  TRY(down32(e, dye, e->dye[0], 3 * e->dye_cells() * 4, "dye"));
  return sync(e, "commit labels");
}

int fl_body_forces(fl_engine* h, float* u, float* v, const float* dye, const uint8_t* label, float beta, float alpha,
                   float eps, float dt) {
  ENTER(h);
  e->uploaded = false;
  Level& L = e->levels[0];
  TRY(up32(e, e->u[0], u, e->ufaces() * 4, "u"));
  TRY(up32(e, e->v[0], v, e->vfaces() * 4, "v"));
  TRY(up32(e, e->dye[0], dye, 3 * e->dye_cells() * 4, "dye"));
  TRY(put_labels(e, label, "label"));
  StepScalars s{};
  s.dt = dt;
  s.gain_beta = beta * dt;
  s.gain_alpha = -alpha * dt;
  s.half_dt = 0.5f * dt;
  TRY(put_scalars(e, s));
  const bool conf = eps != 0.0f;
  if (conf) {
    launch_vorticity(e->stream, e->nx, e->ny, e->h, e->u[0], e->v[0], e->w);
    launch_confinement_force(e->stream, e->nx, e->ny, e->h, e->w, L.label, eps, e->fx, e->fy);
  }
  if (beta != 0.0f || alpha != 0.0f || conf)
    launch_forces(e->stream, e->nx, e->ny, e->h, e->dnx, e->dny, e->dh, e->u[0], e->v[0], e->dye[0], L.label,
                  beta != 0.0f, alpha != 0.0f, conf, e->fx, e->fy, e->sc);
  TRY(check_launch(e, "body forces"));
  TRY(down32(e, u, e->u[0], e->ufaces() * 4, "u"));
  TRY(down32(e, v, e->v[0], e->vfaces() * 4, "v"));
  return sync(e, "body forces");
}

int fl_stir(fl_engine* h, float* u, float* v, const uint8_t* label, float x, float y, float r, float dx, float dy) {
  ENTER(h);
  e->uploaded = false;
  Level& L = e->levels[0];
  TRY(up32(e, e->u[0], u, e->ufaces() * 4, "u"));
  TRY(up32(e, e->v[0], v, e->vfaces() * 4, "v"));
  TRY(put_labels(e, label, "label"));
  const float st[5] = {x, y, r, dx, dy};
  launch_stir(e->stream, e->nx, e->ny, e->h, e->u[0], e->v[0], L.label, st);
  TRY(check_launch(e, "stir"));
  TRY(down32(e, u, e->u[0], e->ufaces() * 4, "u"));
  TRY(down32(e, v, e->v[0], e->vfaces() * 4, "v"));
  return sync(e, "stir");
}

int fl_dye_patch(fl_engine* h, float* dye, int i0, int j0, int pnx, int pny, const float* data) {
  ENTER(h);
  e->uploaded = false;
  if (!data || pnx <= 0 || pny <= 0) return fail(e, FL_EINVAL, "patch");
  const size_t pbytes = (size_t)4 * pnx * pny * sizeof(float);
  if (pbytes > e->staging_bytes) return fail(e, FL_EINVAL, "patch larger than the staging buffer");
  TRY(up32(e, e->dye[0], dye, 3 * e->dye_cells() * 4, "dye"));
  TRY(up32(e, e->staging, data, pbytes, "patch"));
  launch_dye_patch(e->stream, e->dnx, e->dny, e->dye[0], (const float*)e->staging, i0, j0, pnx, pny);
  TRY(check_launch(e, "dye patch"));
  TRY(down32(e, dye, e->dye[0], 3 * e->dye_cells() * 4, "dye"));
  return sync(e, "dye patch");
}

// ------------------------------------------------------ learned warm start

int fl_set_warm_start(fl_engine* h, fl_unet* net) {
  ENTER(h);
  Unet* u = unet_of(net);
  if (u != nullptr) {
    if (e->nx % 8 || e->ny % 8) return fail(e, FL_EINVAL, "warm start needs sides that are multiples of 8");
    if ((long)e->nx * e->ny > u->cap) return fail(e, FL_EINVAL, "grid exceeds the network's capacity");
    if (u->device != e->device) return fail(e, FL_EINVAL, "network and engine are on different devices");
  }
  e->warm = u;
  destroy_graphs(e);
  return FL_OK;
}

int fl_read_rhs(fl_engine* h, int dtype, void* b) {
  ENTER(h);
  TRY(download(e, b, e->levels[0].b, e->cells(), dtype, "read rhs"));
  return sync(e, "read rhs");
}

// ------------------------------------------------------- batched scenes

}  // extern "C"

struct fl_batch {
  std::vector<fl_engine*> engines;
  std::vector<int> order;  // launch order: most cells first
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t start = nullptr;
  std::vector<cudaEvent_t> events;
  std::string err;
  // The work-list path: every scene's pressure solve batched into one
  // launch per V-cycle phase (BatchSolve), inside one graph per step with
  // the scenes' own passes before and after it as concurrent branches.
  // Null when some scene does not qualify (why_not): then every engine's
  // own step graph is launched on its own stream instead.
  BatchSolve* solve = nullptr;
  std::string why_not;
  cudaStream_t body = nullptr;  // capture stream of the solve's cycle body
  cudaEvent_t mid = nullptr;    // the solve's end, where the post-solve branches fork
  std::vector<cudaEvent_t> joins;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // [0]: every engine at its built parity, [1]: flipped
  std::vector<int> built_cur;
  std::vector<unsigned long long> built_gen;
};

namespace {

int bfail(fl_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (b)
    b->err = buf;
  else
    set_global_error("%s", buf);
  return code;
}

void batch_graphs_free(fl_batch* b) {
  for (auto& g : b->graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  b->built_cur.clear();
  b->built_gen.clear();
}

void batch_free(fl_batch* b) {
  batch_graphs_free(b);
  batch_solve_destroy(b->solve);
  b->solve = nullptr;
  for (cudaEvent_t ev : b->events) cudaEventDestroy(ev);
  for (cudaEvent_t ev : b->joins) cudaEventDestroy(ev);
  if (b->mid) cudaEventDestroy(b->mid);
  if (b->start) cudaEventDestroy(b->start);
  if (b->body) cudaStreamDestroy(b->body);
  if (b->stream) cudaStreamDestroy(b->stream);
}

std::vector<Engine*> batch_engines(fl_batch* b) {
  std::vector<Engine*> es;
  for (int k : b->order) es.push_back(&b->engines[k]->e);
  return es;
}

// Captures one batch step for the engines at parity cur ^ flip: each
// engine's passes up to the divergence on its own stream (forked from the
// batch stream), the batched solve on the batch stream, then each engine's
// projection, dye and CFL passes on its own stream again, joined back.
int batch_capture(fl_batch* b, int flip, cudaGraphExec_t* out) {
  cudaStream_t s = b->stream;
  cudaError_t err = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (err != cudaSuccess) return bfail(b, FL_EDEVICE, "batch capture: %s", cudaGetErrorString(err));
  cudaEventRecord(b->start, s);
  for (int k : b->order) {
    Engine* e = &b->engines[k]->e;
    cudaStreamWaitEvent(e->stream, b->start, 0);
    enqueue_pre(e, e->stream, e->cur ^ flip, false);
    cudaEventRecord(b->events[k], e->stream);
    cudaStreamWaitEvent(s, b->events[k], 0);
  }
  err = batch_solve_enqueue(*b->solve, s, b->body);
  cudaEventRecord(b->mid, s);
  for (int k : b->order) {
    Engine* e = &b->engines[k]->e;
    cudaStreamWaitEvent(e->stream, b->mid, 0);
    const cudaError_t pe = enqueue_post(e, e->stream, e->cur ^ flip, true);
    if (err == cudaSuccess) err = pe;
    cudaEventRecord(b->joins[k], e->stream);
    cudaStreamWaitEvent(s, b->joins[k], 0);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t end = cudaStreamEndCapture(s, &g);
  if (err == cudaSuccess) err = end;
  if (err == cudaSuccess) err = cudaGetLastError();
  if (err == cudaSuccess) err = cudaGraphInstantiate(out, g, 0);
  if (g) cudaGraphDestroy(g);
  if (err != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return bfail(b, FL_EDEVICE, "batch graph: %s", cudaGetErrorString(err));
  }
  return FL_OK;
}

// The graph for the engines' current parities: rebuilt (with the solve's
// plan) when an engine's step graphs changed since, or when the engines'
// parities no longer move together.
int batch_graph_for_now(fl_batch* b, cudaGraphExec_t* out) {
  const size_t n = b->engines.size();
  const bool fresh = b->built_gen.empty();  // no graphs yet: the plan is current
  bool stale = false;
  for (size_t k = 0; !fresh && !stale && k < n; k++) stale = b->built_gen[k] != b->engines[k]->e.graph_gen;
  int flip = -1;
  if (!fresh && !stale) {
    bool same = true, flipped = true;
    for (size_t k = 0; k < n; k++) {
      same = same && b->engines[k]->e.cur == b->built_cur[k];
      flipped = flipped && b->engines[k]->e.cur != b->built_cur[k];
    }
    flip = same ? 0 : flipped ? 1 : -1;
  }
  if (fresh || stale || flip < 0) {
    batch_graphs_free(b);
    if (stale) {
      batch_solve_destroy(b->solve);
      b->solve = batch_solve_create(batch_engines(b), b->why_not);
      if (!b->solve) return bfail(b, FL_EDEVICE, "batched solve: %s", b->why_not.c_str());
    }
    for (size_t k = 0; k < n; k++) {
      b->built_cur.push_back(b->engines[k]->e.cur);
      b->built_gen.push_back(b->engines[k]->e.graph_gen);
    }
    for (int f = 0; f < 2; f++) TRY(batch_capture(b, f, &b->graph[f]));
    flip = 0;
  }
  *out = b->graph[flip];
  return FL_OK;
}

}  // namespace

extern "C" {

int fl_batch_create(fl_engine* const* engines, int count, fl_batch** out) {
  if (!out) return bfail(nullptr, FL_EINVAL, "null output pointer");
  *out = nullptr;
  if (!engines || count < 1) return bfail(nullptr, FL_EINVAL, "empty batch");
  fl_batch* b = new (std::nothrow) fl_batch();
  if (!b) return bfail(nullptr, FL_ENOMEM, "host allocation");
  b->device = engines[0]->e.device;
  for (int k = 0; k < count; k++) {
    Engine* e = engines[k] ? &engines[k]->e : nullptr;
    const char* why = !e                        ? "null engine"
                      : e->device != b->device  ? "engines on different devices"
                      : !e->uploaded            ? "engine without fields"
                      : !graph_eligible(e)      ? "engine not eligible for graph steps (profiling, stir, label edit "
                                                  "or a host-checked red-black tolerance)"
                                                : nullptr;
    if (!why)
      for (int q = 0; q < k; q++)
        if (engines[q] == engines[k]) why = "engine listed twice";
    if (why) {
      delete b;
      return bfail(nullptr, FL_EINVAL, "engine %d: %s", k, why);
    }
    b->engines.push_back(engines[k]);
    b->order.push_back(k);
  }
  std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) {
    return b->engines[x]->e.cells() > b->engines[y]->e.cells();
  });
  cudaSetDevice(b->device);
  cudaError_t err = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&b->body, cudaStreamNonBlocking);
  if (err == cudaSuccess) err = cudaEventCreateWithFlags(&b->start, cudaEventDisableTiming);
  if (err == cudaSuccess) err = cudaEventCreateWithFlags(&b->mid, cudaEventDisableTiming);
  b->events.resize(count, nullptr);
  b->joins.resize(count, nullptr);
  for (int k = 0; k < count && err == cudaSuccess; k++) {
    err = cudaEventCreateWithFlags(&b->events[k], cudaEventDisableTiming);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&b->joins[k], cudaEventDisableTiming);
  }
  if (err != cudaSuccess) {
    batch_free(b);
    delete b;
    return bfail(nullptr, FL_EDEVICE, "batch: %s", cudaGetErrorString(err));
  }
  // the work-list solve when every scene qualifies (multigrid, one V-cycle
  // shape); otherwise b->why_not says why and the engines' own graphs run
  bool worklist = true;
  for (int k = 0; k < count; k++) worklist = worklist && engines[k]->e.prm.solver == FL_SOLVER_MG;
  if (worklist) b->solve = batch_solve_create(batch_engines(b), b->why_not);
  else b->why_not = "a scene solves with red-black SOR";
  // (the step graphs are captured on the first fl_batch_step)
  *out = b;
  return FL_OK;
}

int fl_batch_destroy(fl_batch* b) {
  if (!b) return FL_OK;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  batch_free(b);
  delete b;
  return FL_OK;
}

const char* fl_batch_last_error(const fl_batch* b) { return b ? b->err.c_str() : fl_last_error(nullptr); }

void* fl_batch_stream(fl_batch* b) { return b ? (void*)b->stream : nullptr; }

int fl_batch_worklist(const fl_batch* b) { return b && b->solve ? 1 : 0; }

int fl_batch_set_worklist(fl_batch* b, int on) {
  if (!b) return bfail(nullptr, FL_EINVAL, "null batch");
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  batch_graphs_free(b);
  batch_solve_destroy(b->solve);
  b->solve = nullptr;
  if (!on) return FL_OK;
  b->why_not.clear();
  b->solve = batch_solve_create(batch_engines(b), b->why_not);
  return b->solve ? FL_OK : bfail(b, FL_EINVAL, "work-list solve: %s", b->why_not.c_str());
}

int fl_batch_step(fl_batch* b, int nsteps) {
  if (!b) return bfail(nullptr, FL_EINVAL, "null batch");
  if (nsteps < 0) return bfail(b, FL_EINVAL, "nsteps < 0");
  cudaSetDevice(b->device);
  for (size_t k = 0; k < b->engines.size(); k++) {
    Engine* e = &b->engines[k]->e;
    if (e->busy.load() != 0) return bfail(b, FL_EBUSY, "engine %zu is inside a call", k);
    if (!graph_eligible(e)) return bfail(b, FL_EINVAL, "engine %zu is no longer eligible for graph steps", k);
  }
  if (b->solve) {
    // the batch stream follows every engine's earlier work, then runs the
    // steps; each engine's later work follows the batch's
    for (size_t k = 0; k < b->engines.size(); k++) {
      cudaEventRecord(b->events[k], b->engines[k]->e.stream);
      cudaStreamWaitEvent(b->stream, b->events[k], 0);
    }
    for (int n = 0; n < nsteps; n++) {
      cudaGraphExec_t g = nullptr;
      const int st = batch_graph_for_now(b, &g);
      if (st != FL_OK) return st;
      cudaError_t err = cudaGraphLaunch(g, b->stream);
      if (err != cudaSuccess) return bfail(b, FL_EDEVICE, "batch step: %s", cudaGetErrorString(err));
      for (auto* h : b->engines) {
        Engine* e = &h->e;
        e->cur = 1 - e->cur;
        e->steps++;
        e->stats_on_device = true;
      }
    }
    cudaEventRecord(b->start, b->stream);
    for (auto* h : b->engines) cudaStreamWaitEvent(h->e.stream, b->start, 0);
    cudaError_t err = cudaGetLastError();
    return err == cudaSuccess ? FL_OK : bfail(b, FL_EDEVICE, "batch step: %s", cudaGetErrorString(err));
  }
  // each engine's steps follow its earlier work (its own stream) and the
  // batch stream's earlier work
  cudaEventRecord(b->start, b->stream);
  for (size_t k = 0; k < b->engines.size(); k++) cudaStreamWaitEvent(b->engines[k]->e.stream, b->start, 0);
  for (int n = 0; n < nsteps; n++)
    for (int k : b->order) {
      Engine* e = &b->engines[k]->e;
      const int st = step_graph(e);
      if (st != FL_OK) return bfail(b, st, "engine %d: %s", k, e->err.c_str());
    }
  // the batch stream (fl_batch_stream) completes after every engine's last step
  for (size_t k = 0; k < b->engines.size(); k++) {
    Engine* e = &b->engines[k]->e;
    cudaEventRecord(b->events[k], e->stream);
    cudaStreamWaitEvent(b->stream, b->events[k], 0);
  }
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? FL_OK : bfail(b, FL_EDEVICE, "batch step: %s", cudaGetErrorString(err));
}

}  // extern "C"
