// C entry points over the templated oracle, one set per precision
// (suffix _f64 / _f32). TEST INFRASTRUCTURE ONLY — see flowlab_oracle.hpp.
//
// Field layouts follow grid.ts:1-36: p/label nx*ny, u (nx+1)*ny, v nx*(ny+1),
// dye = 3 planes of dnx*dny laid end to end.
#include "flowlab_oracle.hpp"

using namespace orc;

extern "C" {

// Mirrors StepParams for ctypes. Field order is part of the ABI of this file.
struct orc_params {
  double cflTarget, dtMax, rho;
  int macCormack, solver, pressureIters, mgMaxCycles;
  double omega, tol;
  double dyeDecay[3];
  double beta, alpha, confinement;
  int mgPre, mgPost, mgCoarseSweeps, mgCoarsest;
  double mgOmega;
  int mixed;
  int warmExtrapolate;
  int residualEvery;
};

int orc_abi_version(void) { return 1; }

}  // extern "C"

static StepParams toParams(const orc_params* c) {
  StepParams p;
  p.cflTarget = c->cflTarget;
  p.dtMax = c->dtMax;
  p.rho = c->rho;
  p.macCormack = c->macCormack;
  p.solver = c->solver;
  p.pressureIters = c->pressureIters;
  p.mgMaxCycles = c->mgMaxCycles;
  p.omega = c->omega;
  p.tol = c->tol;
  for (int k = 0; k < 3; k++) p.dyeDecay[k] = c->dyeDecay[k];
  p.beta = c->beta;
  p.alpha = c->alpha;
  p.confinement = c->confinement;
  p.mg.pre = c->mgPre;
  p.mg.post = c->mgPost;
  p.mg.coarseSweeps = c->mgCoarseSweeps;
  p.mg.coarsest = c->mgCoarsest;
  p.mg.omega = c->mgOmega;
  p.mixed = c->mixed;
  p.warmExtrapolate = c->warmExtrapolate;
  p.residualEvery = c->residualEvery;
  return p;
}

#define ORC_DEFINE(T, SUF)                                                                              \
  extern "C" {                                                                                          \
  void orc_advect_velocity_##SUF(int nx, int ny, T h, int mac, const T* uIn, const T* vIn, T* uOut,     \
                                 T* vOut, const uint8_t* label, T dt) {                                 \
    Grid<T> g{nx, ny, h};                                                                               \
    if (mac) {                                                                                          \
      std::vector<T> uHat((size_t)(nx + 1) * ny), vHat((size_t)nx * (ny + 1));                          \
      advectVelocityMacCormack(g, uIn, vIn, uHat.data(), vHat.data(), uOut, vOut, label, dt);           \
    } else {                                                                                            \
      advectVelocity(g, uIn, vIn, uOut, vOut, label, dt);                                               \
    }                                                                                                   \
  }                                                                                                     \
  void orc_advect_dye_##SUF(int nx, int ny, T h, int dnx, int dny, T dh, int mac, const T* u,           \
                            const T* v, const T* qIn, T* qOut, const uint8_t* label, T dt) {            \
    Grid<T> g{nx, ny, h}, dg{dnx, dny, dh};                                                             \
    long cells = (long)dnx * dny;                                                                       \
    std::vector<T> qHat(cells);                                                                         \
    for (int c = 0; c < DYE_CHANNELS; c++) {                                                            \
      if (mac)                                                                                          \
        advectScalarMacCormack(g, u, v, qIn + c * cells, qHat.data(), qOut + c * cells, label, dt, dg); \
      else                                                                                              \
        advectScalar(g, u, v, qIn + c * cells, qOut + c * cells, label, dt, dg);                        \
    }                                                                                                   \
  }                                                                                                     \
  void orc_divergence_##SUF(int nx, int ny, T h, const T* u, const T* v, T* out) {                      \
    computeDivergence(Grid<T>{nx, ny, h}, u, v, out);                                                   \
  }                                                                                                     \
  void orc_rb_sweep_##SUF(int nx, int ny, T* p, const T* div, const uint8_t* label, T scale, T omega,   \
                          int color) {                                                                  \
    redBlackSweep(Grid<T>{nx, ny, T(1)}, p, div, label, scale, omega, color);                           \
  }                                                                                                     \
  int orc_rb_solve_##SUF(int nx, int ny, T* p, const T* div, const uint8_t* label, T scale, int iters,  \
                         T omega, double tol) {                                                         \
    return solvePressureRedBlack(Grid<T>{nx, ny, T(1)}, p, div, label, scale, iters, omega, tol);       \
  }                                                                                                     \
  void orc_gs_sweep_##SUF(int nx, int ny, T* p, const T* div, const uint8_t* label, T scale, T omega,   \
                          int rx, int ry) {                                                             \
    gaussSeidelSweep(Grid<T>{nx, ny, T(1)}, p, div, label, scale, omega, rx != 0, ry != 0);             \
  }                                                                                                     \
  int orc_sor_solve_##SUF(int nx, int ny, T* p, const T* div, const uint8_t* label, T scale, int iters, \
                          T omega, double tol) {                                                        \
    return solvePressure(Grid<T>{nx, ny, T(1)}, p, div, label, scale, iters, omega, tol);               \
  }                                                                                                     \
  double orc_rms_remaining_##SUF(int nx, int ny, const T* p, const T* div, const uint8_t* label,        \
                                 T scale) {                                                             \
    return rmsRemainingDivergence(Grid<T>{nx, ny, T(1)}, p, div, label, scale);                         \
  }                                                                                                     \
  double orc_fluid_div_rms_##SUF(long n, const T* div, const uint8_t* label) {                          \
    return fluidDivRms(div, label, n);                                                                  \
  }                                                                                                     \
  double orc_relres_b_##SUF(int nx, int ny, const T* x, const T* b, const uint8_t* label) {             \
    return relativeResidualB(Grid<T>{nx, ny, T(1)}, x, b, label);                                       \
  }                                                                                                     \
  int orc_mg_solve_##SUF(int nx, int ny, T* p, const T* div, const uint8_t* label, T scale, int cycles, \
                         double tol, int pre, int post, int coarseSweeps, int coarsest, double omega,   \
                         double* relRes) {                                                              \
    Multigrid<T> mg;                                                                                    \
    mg.shape.pre = pre;                                                                                 \
    mg.shape.post = post;                                                                               \
    mg.shape.coarseSweeps = coarseSweeps;                                                               \
    mg.shape.coarsest = coarsest;                                                                       \
    mg.shape.omega = omega;                                                                             \
    return mg.solve(Grid<T>{nx, ny, T(1)}, p, div, label, scale, cycles, tol, relRes);                  \
  }                                                                                                     \
  int orc_mg_solve_mixed_##SUF(int nx, int ny, double* p, const T* div, const uint8_t* label, T scale,         \
                               int cycles, double tol, int pre, int post, int coarseSweeps, int coarsest,      \
                               double omega, double* relRes) {                                                 \
    Multigrid<T> mg;                                                                                    \
    mg.shape.pre = pre;                                                                                 \
    mg.shape.post = post;                                                                               \
    mg.shape.coarseSweeps = coarseSweeps;                                                               \
    mg.shape.coarsest = coarsest;                                                                       \
    mg.shape.omega = omega;                                                                             \
    return solveMixed(mg, Grid<T>{nx, ny, T(1)}, p, div, label, scale, cycles, tol, relRes);           \
  }                                                                                                     \
  void orc_sim_get_p64_##SUF(void* sp, double* p) {                                                     \
    Simulation<T>* s = (Simulation<T>*)sp;                                                              \
    if (s->useDF())                                                                                     \
      for (size_t k = 0; k < s->p.size(); k++) p[k] = df::toDouble(df::at(s->pdf.data(), (long)k));     \
    else                                                                                                \
      std::copy(s->p64.begin(), s->p64.end(), p);                                                       \
  }                                                                                                     \
  void orc_residual_##SUF(int nx, int ny, const T* x, const T* b, const uint8_t* label, T* r) {         \
    computeResidual(Grid<T>{nx, ny, T(1)}, x, b, label, r);                                             \
  }                                                                                                     \
  void orc_restrict_##SUF(int fnx, int fny, const T* r, int cnx, int cny, T* bC, T* eC) {               \
    restrictResidual(fnx, fny, r, cnx, cny, bC, eC);                                                    \
  }                                                                                                     \
  void orc_prolong_##SUF(int fnx, int fny, T* x, const uint8_t* label, int cnx, int cny, const T* e) {  \
    prolongAdd(fnx, fny, x, label, cnx, cny, e);                                                        \
  }                                                                                                     \
  void orc_subtract_gradient_##SUF(int nx, int ny, const T* p, T* u, T* v, const uint8_t* label,        \
                                   T gradScale) {                                                       \
    subtractGradient(Grid<T>{nx, ny, T(1)}, p, u, v, label, gradScale);                                 \
  }                                                                                                     \
  void orc_commit_labels_##SUF(int nx, int ny, T* p, T* u, T* v, const uint8_t* label, T* dye,          \
                               long dyeCells) {                                                         \
    T* planes[3] = {dye, dye ? dye + dyeCells : nullptr, dye ? dye + 2 * dyeCells : nullptr};           \
    commitLabels(Grid<T>{nx, ny, T(1)}, p, u, v, label, dye ? planes : nullptr, dyeCells);              \
  }                                                                                                     \
  void orc_outflow_##SUF(int nx, int ny, T* u, T* v, const uint8_t* label) {                            \
    applyOutflow(Grid<T>{nx, ny, T(1)}, u, v, label);                                                   \
  }                                                                                                     \
  void orc_buoyancy_##SUF(int nx, int ny, T h, int dnx, int dny, T dh, T* v, const T* heat,             \
                          const T* smoke, const uint8_t* label, T beta, T alpha, T dt) {                \
    applyBuoyancy(Grid<T>{nx, ny, h}, Grid<T>{dnx, dny, dh}, v, heat, smoke, label, beta, alpha, dt);   \
  }                                                                                                     \
  void orc_vorticity_##SUF(int nx, int ny, T h, const T* u, const T* v, T* out) {                       \
    computeVorticity(Grid<T>{nx, ny, h}, u, v, out);                                                    \
  }                                                                                                     \
  void orc_confine_##SUF(int nx, int ny, T h, T* u, T* v, const uint8_t* label, T eps, T dt) {          \
    Grid<T> g{nx, ny, h};                                                                               \
    std::vector<T> fx((size_t)nx * ny), fy((size_t)nx * ny);                                            \
    confinementForce(g, u, v, label, eps, fx.data(), fy.data());                                        \
    applyConfinement(g, u, v, label, fx.data(), fy.data(), dt);                                         \
  }                                                                                                     \
  /* Body forces at the step's seam: confinement evaluated on the incoming                           */ \
  /* velocity, buoyancy added, then confinement added (the Simulation order).                        */ \
  void orc_body_forces_##SUF(int nx, int ny, T h, int dnx, int dny, T dh, T* u, T* v, const T* heat,    \
                             const T* smoke, const uint8_t* label, T beta, T alpha, T eps, T dt) {      \
    Grid<T> g{nx, ny, h}, dg{dnx, dny, dh};                                                             \
    std::vector<T> fx((size_t)nx * ny), fy((size_t)nx * ny);                                            \
    if (eps != T(0)) confinementForce(g, u, v, label, eps, fx.data(), fy.data());                       \
    applyBuoyancy(g, dg, v, heat, smoke, label, beta, alpha, dt);                                       \
    if (eps != T(0)) applyConfinement(g, u, v, label, fx.data(), fy.data(), dt);                        \
  }                                                                                                     \
  void orc_stir_##SUF(int nx, int ny, T h, T* u, T* v, const uint8_t* label, T x, T y, T r, T dx,       \
                      T dy) {                                                                           \
    applyStir(Grid<T>{nx, ny, h}, u, v, label, x, y, r, dx, dy);                                        \
  }                                                                                                     \
  void orc_dye_patch_##SUF(int dnx, int dny, T* dye, int pi0, int pj0, int pnx, int pny,                \
                           const float* data) {                                                         \
    long cells = (long)dnx * dny;                                                                       \
    T* planes[3] = {dye, dye + cells, dye + 2 * cells};                                                 \
    applyDyePatch(Grid<T>{dnx, dny, T(1)}, planes, pi0, pj0, pnx, pny, data);                           \
  }                                                                                                     \
  void orc_coarsen_labels_##SUF(int fnx, int fny, const uint8_t* fine, int cnx, int cny,                \
                                uint8_t* coarse) {                                                      \
    coarsenLabels(fnx, fny, fine, cnx, cny, coarse);                                                    \
  }                                                                                                     \
  /* ---- whole-step simulation (simulation.ts) ---- */                                                 \
  void* orc_sim_create_##SUF(int nx, int ny, int dyeScale, const orc_params* prm) {                     \
    return new Simulation<T>(nx, ny, dyeScale, toParams(prm));                                          \
  }                                                                                                     \
  void orc_sim_destroy_##SUF(void* s) { delete (Simulation<T>*)s; }                                     \
  void orc_sim_set_fields_##SUF(void* sp, const T* u, const T* v, const T* p, const uint8_t* label,     \
                                const T* dye) {                                                         \
    Simulation<T>* s = (Simulation<T>*)sp;                                                              \
    std::copy(u, u + s->u.size(), s->u.begin());                                                       \
    std::copy(v, v + s->v.size(), s->v.begin());                                                       \
    std::copy(p, p + s->p.size(), s->p.begin());                                                       \
    std::copy(label, label + s->label.size(), s->label.begin());                                       \
    std::copy(p, p + s->p.size(), s->pPrev.begin());                                                   \
    s->seedRefined();                                                                                   \
    long cells = (long)s->dye[0].size();                                                                \
    for (int c = 0; c < DYE_CHANNELS; c++)                                                              \
      std::copy(dye + c * cells, dye + (c + 1) * cells, s->dye[c].begin());                             \
  }                                                                                                     \
  void orc_sim_get_fields_##SUF(void* sp, T* u, T* v, T* p, T* dye) {                                   \
    Simulation<T>* s = (Simulation<T>*)sp;                                                              \
    std::copy(s->u.begin(), s->u.end(), u);                                                             \
    std::copy(s->v.begin(), s->v.end(), v);                                                             \
    std::copy(s->p.begin(), s->p.end(), p);                                                             \
    long cells = (long)s->dye[0].size();                                                                \
    for (int c = 0; c < DYE_CHANNELS; c++) std::copy(s->dye[c].begin(), s->dye[c].end(), dye + c * cells); \
  }                                                                                                     \
  void orc_sim_set_patch_##SUF(void* sp, int pi0, int pj0, int pnx, int pny, const float* data) {       \
    Simulation<T>* s = (Simulation<T>*)sp;                                                              \
    s->pi0 = pi0;                                                                                       \
    s->pj0 = pj0;                                                                                       \
    s->pnx = data ? pnx : 0;                                                                            \
    s->pny = data ? pny : 0;                                                                            \
    s->patch.assign(data, data ? data + (size_t)4 * pnx * pny : data);                                  \
  }                                                                                                     \
  void orc_sim_set_stir_##SUF(void* sp, const double* st) {                                            \
    Simulation<T>* s = (Simulation<T>*)sp;                                                              \
    s->stirPending = st != nullptr;                                                                     \
    for (int k = 0; k < 5; k++) s->stir[k] = st ? (T)st[k] : T(0);                                      \
  }                                                                                                     \
  int orc_sim_step_##SUF(void* sp) { return ((Simulation<T>*)sp)->step(); }                             \
  /* the last step's divergence (the pressure solve's input) */                                         \
  void orc_sim_get_div_##SUF(void* sp, T* div) {                                                        \
    Simulation<T>* s = (Simulation<T>*)sp;                                                              \
    std::copy(s->div.begin(), s->div.end(), div);                                                       \
  }                                                                                                     \
  /* the post-step divergence and the index of the step that computed it */                               \
  long long orc_sim_get_div_post_##SUF(void* sp, T* div) {                                              \
    Simulation<T>* s = (Simulation<T>*)sp;                                                              \
    std::copy(s->divPost.begin(), s->divPost.end(), div);                                                 \
    return s->divPostStep;                                                                              \
  }                                                                                                     \
  /* the last step's scale rho*h^2/dt */                                                                \
  double orc_sim_scale_##SUF(void* sp) {                                                                \
    Simulation<T>* s = (Simulation<T>*)sp;                                                              \
    return (double)((T(s->prm.rho) * s->g.h * s->g.h) / s->dt);                                         \
  }                                                                                                     \
  void orc_sim_info_##SUF(void* sp, double* dt, double* time, double* relRes) {                         \
    Simulation<T>* s = (Simulation<T>*)sp;                                                              \
    *dt = (double)s->dt;                                                                                \
    *time = s->time;                                                                                    \
    *relRes = s->lastRelRes;                                                                            \
  }                                                                                                     \
  }

ORC_DEFINE(double, f64)
ORC_DEFINE(float, f32)

// Double-float defect correction (mixed = 2), float32 only: p is 2n floats
// (hi, lo per cell), in/out.
extern "C" int orc_mg_solve_df_f32(int nx, int ny, float* p, const float* div, const uint8_t* label, float scale,
                                   int cycles, double tol, int pre, int post, int coarseSweeps, int coarsest,
                                   double omega, double* relRes) {
  Multigrid<float> mg;
  mg.shape.pre = pre;
  mg.shape.post = post;
  mg.shape.coarseSweeps = coarseSweeps;
  mg.shape.coarsest = coarsest;
  mg.shape.omega = omega;
  return solveMixedDF(mg, Grid<float>{nx, ny, 1.0f}, p, div, label, scale, cycles, tol, relRes);
}

// One double-float residual pass: r32 and the norm ratio rms(r) / rms(b).
extern "C" double orc_residual_df_f32(int nx, int ny, const float* p, const float* b, const uint8_t* label,
                                      float* r32) {
  double bSq;
  long nb;
  std::vector<float> bLo((size_t)nx * ny, 0.0f);
  const double rr = residualDF(Grid<float>{nx, ny, 1.0f}, p, b, bLo.data(), label, r32, bSq, nb);
  const double bRms = nb > 0 ? std::sqrt(bSq / (double)nb) : 0.0;
  return bRms > 0 ? rr / bRms : 0.0;
}
