// flowlab oracle: a CPU restatement of flowlab's src/core numerics.
//
// TEST INFRASTRUCTURE ONLY. This is the checker, never the product: only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
// The CUDA engine in flowlab_gb300/ never links or calls it and has no CPU
// fallback.
//
// Every function below restates one function of the reference (file:line in
// its comment) with the SAME floating-point operation order, templated on the
// scalar type:
//   - T = double reproduces the reference's float64 CPU path (the numbers its
//     own tests assert) and is the precision oracle for the GPU's float32.
//   - T = float reproduces the same operations in float32. Compiled without
//     FMA contraction it is the ORDERING oracle: the CUDA kernels (built with
//     -fmad=false) perform the identical sequence of IEEE float operations and
//     must match it bit for bit, which separates an ordering or indexing bug
//     from a precision difference.
// Reductions (RMS norms) accumulate in double for both instantiations; they
// only feed stopping decisions and reports.
//
// Parts with no counterpart in the reference (vorticity confinement, the
// -alpha*s buoyancy term, runtime V(pre,post)/coarsest multigrid shapes,
// float64 defect correction) are written from their published definitions and
// marked NEW below.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

namespace orc {

// grid.ts:41-45
enum : uint8_t { FLUID = 0, AIR = 1, SOLID = 2 };
// grid.ts:73
constexpr int DYE_CHANNELS = 3;

// grid.ts:57-62 (h kept in the field precision, as the GPU receives it)
template <class T>
struct Grid {
  int nx, ny;
  T h;
};

inline long idxP(int nx, int i, int j) { return i + (long)j * nx; }             // grid.ts:119-121
inline long idxU(int nx, int i, int j) { return i + (long)j * (nx + 1); }       // grid.ts:129-131
inline long idxV(int nx, int i, int j) { return i + (long)j * nx; }             // grid.ts:139-141

// grid.ts:159-161 — off-grid counts as solid; bounds test first.
template <class T>
inline bool solidOrOutside(const Grid<T>& g, const uint8_t* label, int i, int j) {
  return i < 0 || j < 0 || i >= g.nx || j >= g.ny || label[idxP(g.nx, i, j)] == SOLID;
}

// boundaries.ts:23-25 — in-domain AND solid.
template <class T>
inline bool solidCell(const Grid<T>& g, const uint8_t* label, int i, int j) {
  return i >= 0 && j >= 0 && i < g.nx && j < g.ny && label[idxP(g.nx, i, j)] == SOLID;
}

template <class T>
struct Axis {
  int i0;
  T f;
};

// grid.ts:173-177
template <class T>
inline Axis<T> clampedAxis(T pos, int count) {
  T clamped = std::min(std::max(pos, T(0)), T(count - 1));
  int i0 = std::min((int)std::floor(clamped), count - 2);
  return {i0, clamped - T(i0)};
}

// grid.ts:180-191 — nested lerps, this exact order.
template <class T>
inline T bilerp(T v00, T v10, T v01, T v11, T fx, T fy) {
  T lo = v00 + fx * (v10 - v00);
  T hi = v01 + fx * (v11 - v01);
  return lo + fy * (hi - lo);
}

// grid.ts:197-208
template <class T>
inline T sampleU(const Grid<T>& g, const T* u, T x, T y) {
  Axis<T> a = clampedAxis(x / g.h, g.nx + 1);
  Axis<T> b = clampedAxis(y / g.h - T(0.5), g.ny);
  long s = g.nx + 1;
  long k = a.i0 + b.i0 * s;
  return bilerp(u[k], u[k + 1], u[k + s], u[k + s + 1], a.f, b.f);
}

// grid.ts:214-225
template <class T>
inline T sampleV(const Grid<T>& g, const T* v, T x, T y) {
  Axis<T> a = clampedAxis(x / g.h - T(0.5), g.nx);
  Axis<T> b = clampedAxis(y / g.h, g.ny + 1);
  long s = g.nx;
  long k = a.i0 + b.i0 * s;
  return bilerp(v[k], v[k + 1], v[k + s], v[k + s + 1], a.f, b.f);
}

// grid.ts:239-250
template <class T>
inline T sampleP(const Grid<T>& g, const T* q, T x, T y) {
  Axis<T> a = clampedAxis(x / g.h - T(0.5), g.nx);
  Axis<T> b = clampedAxis(y / g.h - T(0.5), g.ny);
  long s = g.nx;
  long k = a.i0 + b.i0 * s;
  return bilerp(q[k], q[k + 1], q[k + s], q[k + s + 1], a.f, b.f);
}

// grid.ts:268-270
template <class T>
inline T clampToRange(T q, T a, T b, T c, T d) {
  T lo = std::min(std::min(a, b), std::min(c, d));
  T hi = std::max(std::max(a, b), std::max(c, d));
  return std::min(std::max(q, lo), hi);
}

// grid.ts:273-283
template <class T>
inline T clampToStencilU(const Grid<T>& g, const T* u, T x, T y, T q) {
  int i0 = clampedAxis(x / g.h, g.nx + 1).i0;
  int j0 = clampedAxis(y / g.h - T(0.5), g.ny).i0;
  long s = g.nx + 1;
  long k = i0 + j0 * s;
  return clampToRange(q, u[k], u[k + 1], u[k + s], u[k + s + 1]);
}

// grid.ts:286-296
template <class T>
inline T clampToStencilV(const Grid<T>& g, const T* v, T x, T y, T q) {
  int i0 = clampedAxis(x / g.h - T(0.5), g.nx).i0;
  int j0 = clampedAxis(y / g.h, g.ny + 1).i0;
  long s = g.nx;
  long k = i0 + j0 * s;
  return clampToRange(q, v[k], v[k + 1], v[k + s], v[k + s + 1]);
}

// grid.ts:299-315
template <class T>
inline T clampToStencilP(const Grid<T>& g, const T* q, T x, T y, T value) {
  int i0 = clampedAxis(x / g.h - T(0.5), g.nx).i0;
  int j0 = clampedAxis(y / g.h - T(0.5), g.ny).i0;
  long s = g.nx;
  long k = i0 + j0 * s;
  return clampToRange(value, q[k], q[k + 1], q[k + s], q[k + s + 1]);
}

// ---------------------------------------------------------------- advection

// advect.ts:41-55 — RK2 midpoint; dt < 0 traces forward.
template <class T>
inline void backtrace(const Grid<T>& g, const T* uCar, const T* vCar, T x, T y, T u0, T v0, T dt,
                      T& bx, T& by) {
  T midX = x - T(0.5) * dt * u0;
  T midY = y - T(0.5) * dt * v0;
  bx = x - dt * sampleU(g, uCar, midX, midY);
  by = y - dt * sampleV(g, vCar, midX, midY);
}

// advect.ts:72-112
template <class T>
void advectFaces(const Grid<T>& g, const T* uCar, const T* vCar, const T* uSrc, const T* vSrc,
                 T* uOut, T* vOut, const uint8_t* label, T dt) {
  const T h = g.h;
  for (int j = 0; j < g.ny; j++) {
    T y = (T(j) + T(0.5)) * h;
    for (int i = 0; i <= g.nx; i++) {
      long k = idxU(g.nx, i, j);
      if (solidOrOutside(g, label, i - 1, j) || solidOrOutside(g, label, i, j)) {
        uOut[k] = uSrc[k];
        continue;
      }
      T x = T(i) * h;
      T bx, by;
      backtrace(g, uCar, vCar, x, y, uCar[k], sampleV(g, vCar, x, y), dt, bx, by);
      uOut[k] = sampleU(g, uSrc, bx, by);
    }
  }
  for (int j = 0; j <= g.ny; j++) {
    T y = T(j) * h;
    for (int i = 0; i < g.nx; i++) {
      long k = idxV(g.nx, i, j);
      if (solidOrOutside(g, label, i, j - 1) || solidOrOutside(g, label, i, j)) {
        vOut[k] = vSrc[k];
        continue;
      }
      T x = (T(i) + T(0.5)) * h;
      T bx, by;
      backtrace(g, uCar, vCar, x, y, sampleU(g, uCar, x, y), vCar[k], dt, bx, by);
      vOut[k] = sampleV(g, vSrc, bx, by);
    }
  }
}

// advect.ts:126-136
template <class T>
void advectVelocity(const Grid<T>& g, const T* uIn, const T* vIn, T* uOut, T* vOut,
                    const uint8_t* label, T dt) {
  advectFaces(g, uIn, vIn, uIn, vIn, uOut, vOut, label, dt);
}

// advect.ts:166-211 — forward, reverse (same carrier), corrected + clamped.
template <class T>
void advectVelocityMacCormack(const Grid<T>& g, const T* uIn, const T* vIn, T* uHat, T* vHat,
                              T* uOut, T* vOut, const uint8_t* label, T dt) {
  advectFaces(g, uIn, vIn, uIn, vIn, uHat, vHat, label, dt);
  advectFaces(g, uIn, vIn, uHat, vHat, uOut, vOut, label, -dt);
  const T h = g.h;
  for (int j = 0; j < g.ny; j++) {
    T y = (T(j) + T(0.5)) * h;
    for (int i = 0; i <= g.nx; i++) {
      long k = idxU(g.nx, i, j);
      if (solidOrOutside(g, label, i - 1, j) || solidOrOutside(g, label, i, j)) {
        uOut[k] = uIn[k];
        continue;
      }
      T x = T(i) * h;
      T corrected = uHat[k] + T(0.5) * (uIn[k] - uOut[k]);
      T bx, by;
      backtrace(g, uIn, vIn, x, y, uIn[k], sampleV(g, vIn, x, y), dt, bx, by);
      uOut[k] = clampToStencilU(g, uIn, bx, by, corrected);
    }
  }
  for (int j = 0; j <= g.ny; j++) {
    T y = T(j) * h;
    for (int i = 0; i < g.nx; i++) {
      long k = idxV(g.nx, i, j);
      if (solidOrOutside(g, label, i, j - 1) || solidOrOutside(g, label, i, j)) {
        vOut[k] = vIn[k];
        continue;
      }
      T x = (T(i) + T(0.5)) * h;
      T corrected = vHat[k] + T(0.5) * (vIn[k] - vOut[k]);
      T bx, by;
      backtrace(g, uIn, vIn, x, y, sampleU(g, uIn, x, y), vIn[k], dt, bx, by);
      vOut[k] = clampToStencilV(g, vIn, bx, by, corrected);
    }
  }
}

// advect.ts:241-270 — dg is the dye grid (dyeScale refinement of g).
template <class T>
void advectScalar(const Grid<T>& g, const T* u, const T* v, const T* qIn, T* qOut,
                  const uint8_t* label, T dt, const Grid<T>& dg) {
  const T h = dg.h;
  const T ratio = dg.h / g.h;
  for (int j = 0; j < dg.ny; j++) {
    T y = (T(j) + T(0.5)) * h;
    int lj = (int)std::floor((T(j) + T(0.5)) * ratio);
    for (int i = 0; i < dg.nx; i++) {
      long k = idxP(dg.nx, i, j);
      if (solidOrOutside(g, label, (int)std::floor((T(i) + T(0.5)) * ratio), lj)) {
        qOut[k] = qIn[k];
        continue;
      }
      T x = (T(i) + T(0.5)) * h;
      T bx, by;
      backtrace(g, u, v, x, y, sampleU(g, u, x, y), sampleV(g, v, x, y), dt, bx, by);
      qOut[k] = sampleP(dg, qIn, bx, by);
    }
  }
}

// advect.ts:280-312
template <class T>
void advectScalarMacCormack(const Grid<T>& g, const T* u, const T* v, const T* qIn, T* qHat,
                            T* qOut, const uint8_t* label, T dt, const Grid<T>& dg) {
  advectScalar(g, u, v, qIn, qHat, label, dt, dg);
  advectScalar(g, u, v, qHat, qOut, label, -dt, dg);
  const T h = dg.h;
  const T ratio = dg.h / g.h;
  for (int j = 0; j < dg.ny; j++) {
    T y = (T(j) + T(0.5)) * h;
    int lj = (int)std::floor((T(j) + T(0.5)) * ratio);
    for (int i = 0; i < dg.nx; i++) {
      long k = idxP(dg.nx, i, j);
      if (solidOrOutside(g, label, (int)std::floor((T(i) + T(0.5)) * ratio), lj)) {
        qOut[k] = qIn[k];
        continue;
      }
      T x = (T(i) + T(0.5)) * h;
      T corrected = qHat[k] + T(0.5) * (qIn[k] - qOut[k]);
      T bx, by;
      backtrace(g, u, v, x, y, sampleU(g, u, x, y), sampleV(g, v, x, y), dt, bx, by);
      qOut[k] = clampToStencilP(dg, qIn, bx, by, corrected);
    }
  }
}

// -------------------------------------------------------------- divergence

// divergence.ts:17-25
template <class T>
void computeDivergence(const Grid<T>& g, const T* u, const T* v, T* out) {
  const T coef = T(1) / g.h;
  for (int j = 0; j < g.ny; j++)
    for (int i = 0; i < g.nx; i++)
      out[idxP(g.nx, i, j)] = coef * (u[idxU(g.nx, i + 1, j)] - u[idxU(g.nx, i, j)] +
                                      v[idxV(g.nx, i, j + 1)] - v[idxV(g.nx, i, j)]);
}

// ---------------------------------------------------------------- pressure

// pressure.ts:65-116 — lexicographic GS/SOR; neighbour order +x, +y, -x, -y.
template <class T>
void gaussSeidelSweep(const Grid<T>& g, T* p, const T* div, const uint8_t* label, T scale, T omega,
                      bool reverseX, bool reverseY) {
  const int iStep = reverseX ? -1 : 1, iFrom = reverseX ? g.nx - 1 : 0, iTo = reverseX ? -1 : g.nx;
  const int jStep = reverseY ? -1 : 1, jFrom = reverseY ? g.ny - 1 : 0, jTo = reverseY ? -1 : g.ny;
  for (int j = jFrom; j != jTo; j += jStep) {
    for (int i = iFrom; i != iTo; i += iStep) {
      if (label[idxP(g.nx, i, j)] != FLUID) continue;
      T count = 0, sum = 0;
      if (!solidOrOutside(g, label, i + 1, j)) { count += T(1); sum += p[idxP(g.nx, i + 1, j)]; }
      if (!solidOrOutside(g, label, i, j + 1)) { count += T(1); sum += p[idxP(g.nx, i, j + 1)]; }
      if (!solidOrOutside(g, label, i - 1, j)) { count += T(1); sum += p[idxP(g.nx, i - 1, j)]; }
      if (!solidOrOutside(g, label, i, j - 1)) { count += T(1); sum += p[idxP(g.nx, i, j - 1)]; }
      if (count == T(0)) continue;
      T pGS = (sum - scale * div[idxP(g.nx, i, j)]) / count;
      long k = idxP(g.nx, i, j);
      p[k] = (T(1) - omega) * p[k] + omega * pGS;
    }
  }
}

// pressure.ts:127-167 — sum-of-squares and fluid count, accumulated in double.
template <class T>
void remainingDivergenceSums(const Grid<T>& g, const T* p, const T* div, const uint8_t* label, T scale,
                             double& sumSq, long& n) {
  sumSq = 0;
  n = 0;
  for (int j = 0; j < g.ny; j++) {
    for (int i = 0; i < g.nx; i++) {
      if (label[idxP(g.nx, i, j)] != FLUID) continue;
      T count = 0, sum = 0;
      if (!solidOrOutside(g, label, i + 1, j)) { count += T(1); sum += p[idxP(g.nx, i + 1, j)]; }
      if (!solidOrOutside(g, label, i, j + 1)) { count += T(1); sum += p[idxP(g.nx, i, j + 1)]; }
      if (!solidOrOutside(g, label, i - 1, j)) { count += T(1); sum += p[idxP(g.nx, i - 1, j)]; }
      if (!solidOrOutside(g, label, i, j - 1)) { count += T(1); sum += p[idxP(g.nx, i, j - 1)]; }
      if (count == T(0)) continue;
      long k = idxP(g.nx, i, j);
      double r = (double)div[k] + ((double)count * (double)p[k] - (double)sum) / (double)scale;
      sumSq += r * r;
      n += 1;
    }
  }
}

template <class T>
double rmsRemainingDivergence(const Grid<T>& g, const T* p, const T* div, const uint8_t* label, T scale) {
  double s;
  long n;
  remainingDivergenceSums(g, p, div, label, scale, s, n);
  return n > 0 ? std::sqrt(s / (double)n) : 0.0;
}

// pressure.ts:177-186
template <class T>
double fluidDivRms(const T* div, const uint8_t* label, long n) {
  double sumSq = 0;
  long c = 0;
  for (long k = 0; k < n; k++) {
    if (label[k] != FLUID) continue;
    sumSq += (double)div[k] * (double)div[k];
    c += 1;
  }
  return c > 0 ? std::sqrt(sumSq / (double)c) : 0.0;
}

// pressure.ts:207-237 — 4-direction cycling, check every 12 sweeps.
template <class T>
int solvePressure(const Grid<T>& g, T* p, const T* div, const uint8_t* label, T scale, int iterations,
                  T omega, double tol) {
  const long n = (long)g.nx * g.ny;
  const double divRms = fluidDivRms(div, label, n);
  if (divRms == 0) {
    std::fill(p, p + n, T(0));
    return 0;
  }
  const double target = tol > 0 ? tol * divRms : -1;
  for (int k = 0; k < iterations; k++) {
    gaussSeidelSweep(g, p, div, label, scale, omega, k % 2 == 1, k % 4 >= 2);
    if (target >= 0 && k % 12 == 11)
      if (rmsRemainingDivergence(g, p, div, label, scale) <= target) return k + 1;
  }
  return iterations;
}

// pressureRedBlack.ts:32-72 — colour (i+j)&1; neighbour order +x, -x, +y, -y.
template <class T>
void redBlackSweep(const Grid<T>& g, T* p, const T* div, const uint8_t* label, T scale, T omega, int color) {
  for (int j = 0; j < g.ny; j++) {
    for (int i = (j & 1) ^ color; i < g.nx; i += 2) {
      long k = idxP(g.nx, i, j);
      if (label[k] != FLUID) continue;
      T count = 0, sum = 0;
      if (!solidOrOutside(g, label, i + 1, j)) { count += T(1); sum += p[k + 1]; }
      if (!solidOrOutside(g, label, i - 1, j)) { count += T(1); sum += p[k - 1]; }
      if (!solidOrOutside(g, label, i, j + 1)) { count += T(1); sum += p[k + g.nx]; }
      if (!solidOrOutside(g, label, i, j - 1)) { count += T(1); sum += p[k - g.nx]; }
      if (count == T(0)) continue;
      T pGS = (sum - scale * div[k]) / count;
      p[k] = (T(1) - omega) * p[k] + omega * pGS;
    }
  }
}

// pressureRedBlack.ts:88-113
template <class T>
int solvePressureRedBlack(const Grid<T>& g, T* p, const T* div, const uint8_t* label, T scale,
                          int iterations, T omega, double tol) {
  const long n = (long)g.nx * g.ny;
  const double divRms = fluidDivRms(div, label, n);
  if (divRms == 0) {
    std::fill(p, p + n, T(0));
    return 0;
  }
  const double target = tol > 0 ? tol * divRms : -1;
  for (int k = 0; k < iterations; k++) {
    redBlackSweep(g, p, div, label, scale, omega, 0);
    redBlackSweep(g, p, div, label, scale, omega, 1);
    if (target >= 0 && k % 12 == 11)
      if (rmsRemainingDivergence(g, p, div, label, scale) <= target) return k + 1;
  }
  return iterations;
}

// ---------------------------------------------------------------- multigrid

// pressureMultigrid.ts:71-78 — ceil halving down to `coarsest` (reference: 4;
// the plume configuration asks for 8).
inline std::vector<std::pair<int, int>> levelSizes(int nx, int ny, int coarsest) {
  std::vector<std::pair<int, int>> s{{nx, ny}};
  while (s.back().first > coarsest || s.back().second > coarsest)
    s.push_back({(s.back().first + 1) / 2, (s.back().second + 1) / 2});
  return s;
}

// pressureMultigrid.ts:92-110 — priority Air > Fluid > Solid.
inline void coarsenLabels(int fnx, int fny, const uint8_t* fine, int cnx, int cny, uint8_t* coarse) {
  for (int J = 0; J < cny; J++)
    for (int I = 0; I < cnx; I++) {
      bool air = false, fluid = false;
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
          int i = 2 * I + di, j = 2 * J + dj;
          if (i >= fnx || j >= fny) continue;
          uint8_t l = fine[idxP(fnx, i, j)];
          air = air || l == AIR;
          fluid = fluid || l == FLUID;
        }
      coarse[idxP(cnx, I, J)] = air ? AIR : fluid ? FLUID : SOLID;
    }
}

// pressureMultigrid.ts:117-151 — neighbour order +x, -x, +y, -y.
template <class T>
void computeResidual(const Grid<T>& g, const T* x, const T* b, const uint8_t* label, T* r) {
  for (int j = 0; j < g.ny; j++)
    for (int i = 0; i < g.nx; i++) {
      long k = idxP(g.nx, i, j);
      r[k] = 0;
      if (label[k] != FLUID) continue;
      T count = 0, sum = 0;
      if (!solidOrOutside(g, label, i + 1, j)) { count += T(1); sum += x[k + 1]; }
      if (!solidOrOutside(g, label, i - 1, j)) { count += T(1); sum += x[k - 1]; }
      if (!solidOrOutside(g, label, i, j + 1)) { count += T(1); sum += x[k + g.nx]; }
      if (!solidOrOutside(g, label, i, j - 1)) { count += T(1); sum += x[k - g.nx]; }
      if (count == T(0)) continue;
      r[k] = b[k] - (count * x[k] - sum);
    }
}

// The same relative residual stated on the multigrid's own unknowns: with
// b = -scale*div, the remaining divergence of pressure.ts:161 is
// -(b - (count*x - sum))/scale, so its RMS over the RMS of the fluid
// divergence is rms(b - (count*x - sum)) / rms(b). The residual is formed in
// T with computeResidual's neighbour order (pressureMultigrid.ts:131-146),
// squared and summed in double — the arithmetic the CUDA tolerance check does.
template <class T>
void residualSumsB(const Grid<T>& g, const T* x, const T* b, const uint8_t* label, double& sumSq, long& n,
                   double& bSq, long& nb) {
  sumSq = 0; n = 0; bSq = 0; nb = 0;
  for (int j = 0; j < g.ny; j++)
    for (int i = 0; i < g.nx; i++) {
      long k = idxP(g.nx, i, j);
      if (label[k] != FLUID) continue;
      bSq += (double)b[k] * (double)b[k];
      nb += 1;
      T count = 0, sum = 0;
      if (!solidOrOutside(g, label, i + 1, j)) { count += T(1); sum += x[k + 1]; }
      if (!solidOrOutside(g, label, i - 1, j)) { count += T(1); sum += x[k - 1]; }
      if (!solidOrOutside(g, label, i, j + 1)) { count += T(1); sum += x[k + g.nx]; }
      if (!solidOrOutside(g, label, i, j - 1)) { count += T(1); sum += x[k - g.nx]; }
      if (count == T(0)) continue;
      T r = b[k] - (count * x[k] - sum);
      sumSq += (double)r * (double)r;
      n += 1;
    }
}

template <class T>
double relativeResidualB(const Grid<T>& g, const T* x, const T* b, const uint8_t* label) {
  double s, bs;
  long n, nb;
  residualSumsB(g, x, b, label, s, n, bs, nb);
  double num = n > 0 ? std::sqrt(s / (double)n) : 0.0;
  double den = nb > 0 ? std::sqrt(bs / (double)nb) : 0.0;
  return den > 0 ? num / den : 0.0;
}

// pressureMultigrid.ts:156-178
template <class T>
void restrictResidual(int fnx, int fny, const T* r, int cnx, int cny, T* bC, T* eC) {
  for (int J = 0; J < cny; J++)
    for (int I = 0; I < cnx; I++) {
      T sum = 0;
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
          int i = 2 * I + di, j = 2 * J + dj;
          if (i < fnx && j < fny) sum += r[idxP(fnx, i, j)];
        }
      long K = idxP(cnx, I, J);
      bC[K] = sum;
      eC[K] = 0;
    }
}

// pressureMultigrid.ts:192-207 — 9/16, 3/16, 3/16, 1/16 with clamped neighbours.
template <class T>
void prolongAdd(int fnx, int fny, T* x, const uint8_t* label, int cnx, int cny, const T* e) {
  for (int j = 0; j < fny; j++) {
    int J = j >> 1;
    int J2 = (j & 1) ? std::min(J + 1, cny - 1) : std::max(J - 1, 0);
    for (int i = 0; i < fnx; i++) {
      long k = idxP(fnx, i, j);
      if (label[k] != FLUID) continue;
      int I = i >> 1;
      int I2 = (i & 1) ? std::min(I + 1, cnx - 1) : std::max(I - 1, 0);
      x[k] += T(0.5625) * e[idxP(cnx, I, J)] + T(0.1875) * (e[idxP(cnx, I2, J)] + e[idxP(cnx, I, J2)]) +
              T(0.0625) * e[idxP(cnx, I2, J2)];
    }
  }
}

// pressureMultigrid.ts:47-63 constants, made runtime parameters (NEW: the
// plume configuration runs V(3,3) to an 8x8 coarsest grid).
struct MgShape {
  int pre = 2, post = 2, coarseSweeps = 8, coarsest = 4;
  double omega = 1.0;
};

// pressureMultigrid.ts:219-320 (CpuMultigridSolver), levels rebuilt per solve.
template <class T>
struct Multigrid {
  struct Level {
    Grid<T> g;
    std::vector<uint8_t> label;
    std::vector<T> x, b, r;
  };
  MgShape shape;
  std::vector<Level> levels;

  void ensure(const Grid<T>& g) {
    if (!levels.empty() && levels[0].g.nx == g.nx && levels[0].g.ny == g.ny) return;
    levels.clear();
    auto sizes = levelSizes(g.nx, g.ny, shape.coarsest);
    T hl = g.h;
    for (auto& s : sizes) {
      long n = (long)s.first * s.second;
      Level L;
      L.g = {s.first, s.second, hl};
      L.label.assign(n, 0);
      L.x.assign(n, 0);
      L.b.assign(n, 0);
      L.r.assign(n, 0);
      levels.push_back(std::move(L));
      hl = hl * T(2);
    }
  }

  void smoothPairs(int l, T* x, int pairs) {
    Level& L = levels[l];
    for (int s = 0; s < pairs; s++) {
      redBlackSweep(L.g, x, L.b.data(), L.label.data(), T(-1), T(shape.omega), 0);
      redBlackSweep(L.g, x, L.b.data(), L.label.data(), T(-1), T(shape.omega), 1);
    }
  }

  // pressureMultigrid.ts:253-275
  void vcycle(int l, T* x) {
    Level& L = levels[l];
    if (l == (int)levels.size() - 1) {
      smoothPairs(l, x, shape.coarseSweeps);
      return;
    }
    smoothPairs(l, x, shape.pre);
    computeResidual(L.g, x, L.b.data(), L.label.data(), L.r.data());
    Level& N = levels[l + 1];
    restrictResidual(L.g.nx, L.g.ny, L.r.data(), N.g.nx, N.g.ny, N.b.data(), N.x.data());
    vcycle(l + 1, N.x.data());
    prolongAdd(L.g.nx, L.g.ny, x, L.label.data(), N.g.nx, N.g.ny, N.x.data());
    smoothPairs(l, x, shape.post);
  }

  // Coarsens the label chain and sets the fine rhs b = -scale * div
  // (pressureMultigrid.ts:302-311).
  void prepare(const Grid<T>& g, const T* div, const uint8_t* label, T scale) {
    ensure(g);
    long n = (long)g.nx * g.ny;
    std::memcpy(levels[0].label.data(), label, n);
    for (size_t l = 1; l < levels.size(); l++)
      coarsenLabels(levels[l - 1].g.nx, levels[l - 1].g.ny, levels[l - 1].label.data(), levels[l].g.nx,
                    levels[l].g.ny, levels[l].label.data());
    for (long k = 0; k < n; k++) levels[0].b[k] = -scale * div[k];
  }

  // pressureMultigrid.ts:284-319. Returns cycles used; `relRes` receives the
  // final remaining-divergence RMS over the fluid divergence RMS when a check
  // ran (tol > 0), else -1.
  int solve(const Grid<T>& g, T* p, const T* div, const uint8_t* label, T scale, int cycles, double tol,
            double* relRes) {
    const long n = (long)g.nx * g.ny;
    const double divRms = fluidDivRms(div, label, n);
    if (relRes) *relRes = -1;
    if (divRms == 0) {
      std::fill(p, p + n, T(0));
      if (relRes) *relRes = 0;
      return 0;
    }
    prepare(g, div, label, scale);
    for (int c = 0; c < cycles; c++) {
      vcycle(0, p);
      if (tol > 0) {
        // float64: the reference's own test (pressureMultigrid.ts:316).
        // float32: the same ratio on b, as the CUDA engine evaluates it.
        if (std::is_same<T, double>::value) {
          double rr = rmsRemainingDivergence(g, p, div, label, scale);
          if (relRes) *relRes = rr / divRms;
          if (rr <= tol * divRms) return c + 1;
        } else {
          double rel = relativeResidualB(g, p, levels[0].b.data(), label);
          if (relRes) *relRes = rel;
          if (rel <= tol) return c + 1;
        }
      }
    }
    return cycles;
  }
};

// NEW — float64 defect correction (iterative refinement) around the float32
// multigrid: the pressure is kept in double; each outer pass
// forms the residual r = b - A p in double (neighbour sum in the order +x,
// -x, +y, -y), runs ONE float32 V-cycle on A e = float(r) from e = 0, and
// adds e back in double. The rhs of the residual is the unrounded product
// -scale * div: the float b plus its rounding error bLo = fma(-scale, div,
// -b) (exact), so the tolerance is met by the reference's own quantity
// (rmsRemainingDivergence / fluidDivRms, pressure.ts:102-186) and not only
// by the rounded rhs, whose rounding alone leaves ~3e-8 of it. The relative
// residual is rms(r over fluid cells with links) / rms(b over fluid cells),
// tested before each pass, so an already converged warm start costs no
// cycle.
template <class T>
double residual64(const Grid<T>& g, const double* p, const T* b, const T* bLo, const uint8_t* label, T* r32,
                  double& bSq, long& nb) {
  double sumSq = 0;
  long n = 0;
  bSq = 0;
  nb = 0;
  for (int j = 0; j < g.ny; j++)
    for (int i = 0; i < g.nx; i++) {
      long k = idxP(g.nx, i, j);
      r32[k] = 0;
      if (label[k] != FLUID) continue;
      bSq += (double)b[k] * (double)b[k];
      nb += 1;
      double count = 0, sum = 0;
      if (!solidOrOutside(g, label, i + 1, j)) { count += 1.0; sum += p[k + 1]; }
      if (!solidOrOutside(g, label, i - 1, j)) { count += 1.0; sum += p[k - 1]; }
      if (!solidOrOutside(g, label, i, j + 1)) { count += 1.0; sum += p[k + g.nx]; }
      if (!solidOrOutside(g, label, i, j - 1)) { count += 1.0; sum += p[k - g.nx]; }
      if (count == 0) continue;
      // b + bLo: the rhs with its rounding error restored (exact in double)
      double r = ((double)b[k] + (double)bLo[k]) - (count * p[k] - sum);
      r32[k] = (T)r;
      sumSq += r * r;
      n += 1;
    }
  return n > 0 ? std::sqrt(sumSq / (double)n) : 0.0;
}

template <class T>
int solveMixed(Multigrid<T>& mg, const Grid<T>& g, double* p, const T* div, const uint8_t* label, T scale,
               int cycles, double tol, double* relRes) {
  const long n = (long)g.nx * g.ny;
  mg.prepare(g, div, label, scale);  // labels + levels[0].b = -scale*div
  std::vector<T> b(mg.levels[0].b), bLo(n);
  for (long k = 0; k < n; k++) bLo[k] = std::fma(-scale, div[k], -b[k]);
  std::vector<T> e(n);
  double bSq;
  long nb;
  double rr = residual64(g, p, b.data(), bLo.data(), label, mg.levels[0].b.data(), bSq, nb);
  const double bRms = nb > 0 ? std::sqrt(bSq / (double)nb) : 0.0;
  if (relRes) *relRes = -1;
  if (bRms == 0) {
    std::fill(p, p + n, 0.0);
    if (relRes) *relRes = 0;
    return 0;
  }
  double rel = rr / bRms;
  if (relRes) *relRes = rel;
  int c = 0;
  while (c < cycles && !(rel <= tol)) {
    std::fill(e.begin(), e.end(), T(0));
    mg.vcycle(0, e.data());  // levels[0].b holds float(r)
    for (long k = 0; k < n; k++) p[k] += (double)e[k];
    rr = residual64(g, p, b.data(), bLo.data(), label, mg.levels[0].b.data(), bSq, nb);
    rel = rr / bRms;
    if (relRes) *relRes = rel;
    c++;
  }
  return c;
}

// NEW — double-float defect correction (mixed = 2): the outer loop of
// solveMixed with the pressure kept as an unevaluated sum hi + lo of two
// floats (about 48 significand bits) instead of a double, and the residual
// formed with error-free float transformations: TwoSum (Knuth, TAOCP vol. 2,
// 4.2.2), FastTwoSum and the double-length sum of Dekker ("A floating-point
// technique for extending the available precision", 1971), and an FMA-based
// exact product for the count 3. Every operation is one IEEE float32
// operation (or a fused multiply-add where written), so the CUDA kernels
// reproduce the results bit for bit. The pressure lives in pairs
// (p[2k] = hi, p[2k+1] = lo).
namespace df {
struct F2 {
  float hi, lo;
};
// s + e = a + b exactly.
inline F2 twoSum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
// s + e = a + b exactly when |a| >= |b| (or a == 0).
inline F2 fastTwoSum(float a, float b) {
  const float s = a + b;
  const float e = b - (s - a);
  return {s, e};
}
// (x.hi + x.lo) + (y.hi + y.lo), renormalised.
inline F2 add(F2 x, F2 y) {
  const F2 s = twoSum(x.hi, y.hi);
  const float e = s.lo + (x.lo + y.lo);
  return fastTwoSum(s.hi, e);
}
inline F2 neg(F2 x) { return {-x.hi, -x.lo}; }
// (x.hi + x.lo) + f, renormalised.
inline F2 addF(F2 x, float f) {
  const F2 s = twoSum(x.hi, f);
  const float e = s.lo + x.lo;
  return fastTwoSum(s.hi, e);
}
// count * x for a link count 1..4 (2 and 4 scale exactly; 3 through the
// exact product 3*hi = p + fma(3, hi, -p)).
inline F2 mulCount(F2 x, int count) {
  if (count == 4) return {4.0f * x.hi, 4.0f * x.lo};
  if (count == 2) return {2.0f * x.hi, 2.0f * x.lo};
  if (count == 1) return x;
  const float p = 3.0f * x.hi;
  float e = std::fma(3.0f, x.hi, -p);
  e = std::fma(3.0f, x.lo, e);
  return fastTwoSum(p, e);
}
// The pair rounded to one float.
inline float round(F2 x) { return x.hi + x.lo; }
// a - b of two pairs, rounded to one float (the projection's pressure
// difference).
inline float diff(F2 a, F2 b) {
  const F2 s = twoSum(a.hi, -b.hi);
  const float e = s.lo + (a.lo - b.lo);
  return s.hi + e;
}
inline double toDouble(F2 x) { return (double)x.hi + (double)x.lo; }
inline F2 fromDouble(double d) {
  const float hi = (float)d;
  return {hi, (float)(d - (double)hi)};
}
inline F2 at(const float* p, long k) { return {p[2 * k], p[2 * k + 1]}; }
inline void put(float* p, long k, F2 x) {
  p[2 * k] = x.hi;
  p[2 * k + 1] = x.lo;
}
}  // namespace df

// r = (b + bLo) - (count*p - sum) in double-float arithmetic (bLo: the
// rhs's rounding error, as in solveMixed), the neighbour sum in
// the order +x, -x, +y, -y starting from the first linked neighbour; r32 is
// the result rounded to float (0 off-fluid and on cells without links). The
// norm is the sum of r32^2 (squares exact in double) over fluid cells with
// links; bSq/nb are the rhs sums over fluid cells, as residual64.
inline double residualDF(const Grid<float>& g, const float* p, const float* b, const float* bLo,
                         const uint8_t* label, float* r32, double& bSq, long& nb) {
  double sumSq = 0;
  long n = 0;
  bSq = 0;
  nb = 0;
  for (int j = 0; j < g.ny; j++)
    for (int i = 0; i < g.nx; i++) {
      const long k = idxP(g.nx, i, j);
      r32[k] = 0;
      if (label[k] != FLUID) continue;
      bSq += (double)b[k] * (double)b[k];
      nb += 1;
      const bool links[4] = {!solidOrOutside(g, label, i + 1, j), !solidOrOutside(g, label, i - 1, j),
                             !solidOrOutside(g, label, i, j + 1), !solidOrOutside(g, label, i, j - 1)};
      const long nbk[4] = {k + 1, k - 1, k + g.nx, k - g.nx};
      int count = 0;
      df::F2 sum{0.0f, 0.0f};
      for (int q = 0; q < 4; q++) {
        if (!links[q]) continue;
        sum = count == 0 ? df::at(p, nbk[q]) : df::add(sum, df::at(p, nbk[q]));
        count += 1;
      }
      if (count == 0) continue;
      const df::F2 d = df::add(df::mulCount(df::at(p, k), count), df::neg(sum));
      const df::F2 s = df::twoSum(b[k], -d.hi);
      const float e = s.lo + (bLo[k] - d.lo);
      const float r = s.hi + e;
      r32[k] = r;
      sumSq += (double)r * (double)r;
      n += 1;
    }
  return n > 0 ? std::sqrt(sumSq / (double)n) : 0.0;
}

// solveMixed with the double-float pressure `p` (2n floats): the same loop,
// tests and cycle count rule; each pass adds the V-cycle's e to every
// cell's pair (p = p + e, renormalised).
inline int solveMixedDF(Multigrid<float>& mg, const Grid<float>& g, float* p, const float* div, const uint8_t* label,
                        float scale, int cycles, double tol, double* relRes) {
  const long n = (long)g.nx * g.ny;
  mg.prepare(g, div, label, scale);
  std::vector<float> b(mg.levels[0].b), bLo(n);
  for (long k = 0; k < n; k++) bLo[k] = std::fma(-scale, div[k], -b[k]);
  std::vector<float> e(n);
  double bSq;
  long nb;
  double rr = residualDF(g, p, b.data(), bLo.data(), label, mg.levels[0].b.data(), bSq, nb);
  const double bRms = nb > 0 ? std::sqrt(bSq / (double)nb) : 0.0;
  if (relRes) *relRes = -1;
  if (bRms == 0) {
    std::fill(p, p + 2 * n, 0.0f);
    if (relRes) *relRes = 0;
    return 0;
  }
  double rel = rr / bRms;
  if (relRes) *relRes = rel;
  int c = 0;
  while (c < cycles && !(rel <= tol)) {
    std::fill(e.begin(), e.end(), 0.0f);
    mg.vcycle(0, e.data());
    for (long k = 0; k < n; k++) df::put(p, k, df::addF(df::at(p, k), e[k]));
    rr = residualDF(g, p, b.data(), bLo.data(), label, mg.levels[0].b.data(), bSq, nb);
    rel = rr / bRms;
    if (relRes) *relRes = rel;
    c++;
  }
  return c;
}

// ------------------------------------------------------------- projection

// subtractGradient.ts:40-61
template <class T>
void subtractGradient(const Grid<T>& g, const T* p, T* u, T* v, const uint8_t* label, T gradScale) {
  for (int j = 0; j < g.ny; j++)
    for (int i = 1; i < g.nx; i++) {
      if (solidOrOutside(g, label, i - 1, j) || solidOrOutside(g, label, i, j)) continue;
      u[idxU(g.nx, i, j)] -= gradScale * (p[idxP(g.nx, i, j)] - p[idxP(g.nx, i - 1, j)]);
    }
  for (int j = 1; j < g.ny; j++)
    for (int i = 0; i < g.nx; i++) {
      if (solidOrOutside(g, label, i, j - 1) || solidOrOutside(g, label, i, j)) continue;
      v[idxV(g.nx, i, j)] -= gradScale * (p[idxP(g.nx, i, j)] - p[idxP(g.nx, i, j - 1)]);
    }
}

// subtractGradient with a float64 pressure: the difference is formed in
// double and rounded once before the float update.
template <class T>
void subtractGradient64(const Grid<T>& g, const double* p, T* u, T* v, const uint8_t* label, T gradScale) {
  for (int j = 0; j < g.ny; j++)
    for (int i = 1; i < g.nx; i++) {
      if (solidOrOutside(g, label, i - 1, j) || solidOrOutside(g, label, i, j)) continue;
      u[idxU(g.nx, i, j)] -= gradScale * (T)(p[idxP(g.nx, i, j)] - p[idxP(g.nx, i - 1, j)]);
    }
  for (int j = 1; j < g.ny; j++)
    for (int i = 0; i < g.nx; i++) {
      if (solidOrOutside(g, label, i, j - 1) || solidOrOutside(g, label, i, j)) continue;
      v[idxV(g.nx, i, j)] -= gradScale * (T)(p[idxP(g.nx, i, j)] - p[idxP(g.nx, i, j - 1)]);
    }
}

// subtractGradient with the double-float pressure (pairs): the difference
// of two pairs rounded once (df::diff) before the float update.
inline void subtractGradientDF(const Grid<float>& g, const float* p, float* u, float* v, const uint8_t* label,
                               float gradScale) {
  for (int j = 0; j < g.ny; j++)
    for (int i = 1; i < g.nx; i++) {
      if (solidOrOutside(g, label, i - 1, j) || solidOrOutside(g, label, i, j)) continue;
      u[idxU(g.nx, i, j)] -= gradScale * df::diff(df::at(p, idxP(g.nx, i, j)), df::at(p, idxP(g.nx, i - 1, j)));
    }
  for (int j = 1; j < g.ny; j++)
    for (int i = 0; i < g.nx; i++) {
      if (solidOrOutside(g, label, i, j - 1) || solidOrOutside(g, label, i, j)) continue;
      v[idxV(g.nx, i, j)] -= gradScale * df::diff(df::at(p, idxP(g.nx, i, j)), df::at(p, idxP(g.nx, i, j - 1)));
    }
}

// boundaries.ts:45-64
template <class T>
void commitLabels(const Grid<T>& g, T* p, T* u, T* v, const uint8_t* label, T* const* dye, long dyeCells) {
  const long n = (long)g.nx * g.ny;
  for (long k = 0; k < n; k++) {
    if (label[k] == FLUID) continue;
    p[k] = 0;
    // The reference clears dye[c][k] with the velocity-grid index k: with a
    // refined dye grid that is a different cell, and it is restated as is.
    if (label[k] == SOLID && dye)
      for (int c = 0; c < DYE_CHANNELS; c++)
        if (k < dyeCells) dye[c][k] = 0;
  }
  for (int j = 0; j < g.ny; j++)
    for (int i = 0; i <= g.nx; i++)
      if (solidCell(g, label, i - 1, j) || solidCell(g, label, i, j)) u[idxU(g.nx, i, j)] = 0;
  for (int j = 0; j <= g.ny; j++)
    for (int i = 0; i < g.nx; i++)
      if (solidCell(g, label, i, j - 1) || solidCell(g, label, i, j)) v[idxV(g.nx, i, j)] = 0;
}

// boundaries.ts:115-143
template <class T>
void applyOutflow(const Grid<T>& g, T* u, T* v, const uint8_t* label) {
  for (int j = 0; j < g.ny; j++) {
    if (label[idxP(g.nx, 0, j)] == AIR) {
      T out = std::min(u[idxU(g.nx, 1, j)], T(0));
      u[idxU(g.nx, 1, j)] = out;
      u[idxU(g.nx, 0, j)] = out;
    }
    if (label[idxP(g.nx, g.nx - 1, j)] == AIR) {
      T out = std::max(u[idxU(g.nx, g.nx - 1, j)], T(0));
      u[idxU(g.nx, g.nx - 1, j)] = out;
      u[idxU(g.nx, g.nx, j)] = out;
    }
  }
  for (int i = 0; i < g.nx; i++) {
    if (label[idxP(g.nx, i, 0)] == AIR) {
      T out = std::min(v[idxV(g.nx, i, 1)], T(0));
      v[idxV(g.nx, i, 1)] = out;
      v[idxV(g.nx, i, 0)] = out;
    }
    if (label[idxP(g.nx, i, g.ny - 1)] == AIR) {
      T out = std::max(v[idxV(g.nx, i, g.ny - 1)], T(0));
      v[idxV(g.nx, i, g.ny - 1)] = out;
      v[idxV(g.nx, i, g.ny)] = out;
    }
  }
}

// ------------------------------------------------------------- body forces

// buoyancy.ts:70-88, plus the NEW soot term of Fedkiw, Stam & Jensen (2001):
//   v += (beta*dt) * T  +  (-alpha*dt) * s,    T = dye[0], s = dye[1]
// Each term is skipped when its weight is 0, so with alpha = 0 this is the
// reference's arithmetic exactly.
template <class T>
void applyBuoyancy(const Grid<T>& g, const Grid<T>& dg, T* v, const T* heat, const T* smoke,
                   const uint8_t* label, T beta, T alpha, T dt) {
  if (beta == T(0) && alpha == T(0)) return;
  const T gainB = beta * dt;
  const T gainA = -alpha * dt;
  for (int j = 1; j < g.ny; j++) {
    T y = T(j) * g.h;
    for (int i = 0; i < g.nx; i++) {
      if (solidCell(g, label, i, j - 1) || solidCell(g, label, i, j)) continue;
      T x = (T(i) + T(0.5)) * g.h;
      long k = idxV(g.nx, i, j);
      if (beta != T(0)) v[k] += gainB * sampleP(dg, heat, x, y);
      if (alpha != T(0)) v[k] += gainA * sampleP(dg, smoke, x, y);
    }
  }
}

// vorticity.ts:9-14 — curl at corner (i*h, j*h).
template <class T>
inline T curlAtCorner(const Grid<T>& g, const T* u, const T* v, int i, int j) {
  return (v[idxV(g.nx, i, j)] - v[idxV(g.nx, i - 1, j)]) / g.h -
         (u[idxU(g.nx, i, j)] - u[idxU(g.nx, i, j - 1)]) / g.h;
}

// vorticity.ts:24-42 — corner curls averaged to centres, clamped at walls.
template <class T>
void computeVorticity(const Grid<T>& g, const T* u, const T* v, T* out) {
  const int hiI = g.nx - 1, hiJ = g.ny - 1;
  for (int j = 0; j < g.ny; j++) {
    int j0 = std::min(std::max(j, 1), hiJ), j1 = std::min(std::max(j + 1, 1), hiJ);
    for (int i = 0; i < g.nx; i++) {
      int i0 = std::min(std::max(i, 1), hiI), i1 = std::min(std::max(i + 1, 1), hiI);
      out[idxP(g.nx, i, j)] = T(0.25) * (curlAtCorner(g, u, v, i0, j0) + curlAtCorner(g, u, v, i1, j0) +
                                         curlAtCorner(g, u, v, i0, j1) + curlAtCorner(g, u, v, i1, j1));
    }
  }
}

// NEW — vorticity confinement (Fedkiw, Stam & Jensen 2001, eqs. 9-11):
//   w = curl u at centres (computeVorticity above), a = |w|,
//   grad a by centred differences (one-sided at the walls),
//   N = grad a / (|grad a| + 1e-20),  f = eps*h * (N x w) = eps*h*(N_y w, -N_x w)
// at cell centres (zero in solid cells), averaged onto faces and added as
// u += dt * 0.5*(f_x[i-1,j] + f_x[i,j]) on the faces stir and buoyancy may
// write (interior, not touching an in-domain solid).
template <class T>
void confinementForce(const Grid<T>& g, const T* u, const T* v, const uint8_t* label, T eps, T* fx, T* fy) {
  const long n = (long)g.nx * g.ny;
  std::vector<T> w(n), a(n);
  computeVorticity(g, u, v, w.data());
  for (long k = 0; k < n; k++) a[k] = std::fabs(w[k]);
  const T epsh = eps * g.h;
  for (int j = 0; j < g.ny; j++)
    for (int i = 0; i < g.nx; i++) {
      long k = idxP(g.nx, i, j);
      if (label[k] == SOLID) {
        fx[k] = 0;
        fy[k] = 0;
        continue;
      }
      int ie = std::min(i + 1, g.nx - 1), iw = std::max(i - 1, 0);
      int jn = std::min(j + 1, g.ny - 1), js = std::max(j - 1, 0);
      T gx = (a[idxP(g.nx, ie, j)] - a[idxP(g.nx, iw, j)]) / (T(ie - iw) * g.h);
      T gy = (a[idxP(g.nx, i, jn)] - a[idxP(g.nx, i, js)]) / (T(jn - js) * g.h);
      T mag = std::sqrt(gx * gx + gy * gy) + T(1e-20);
      T Nx = gx / mag, Ny = gy / mag;
      fx[k] = epsh * (Ny * w[k]);
      fy[k] = epsh * (-(Nx * w[k]));
    }
}

template <class T>
void applyConfinement(const Grid<T>& g, T* u, T* v, const uint8_t* label, const T* fx, const T* fy, T dt) {
  const T half = T(0.5) * dt;
  for (int j = 0; j < g.ny; j++)
    for (int i = 1; i < g.nx; i++) {
      if (solidCell(g, label, i - 1, j) || solidCell(g, label, i, j)) continue;
      u[idxU(g.nx, i, j)] += half * (fx[idxP(g.nx, i - 1, j)] + fx[idxP(g.nx, i, j)]);
    }
  for (int j = 1; j < g.ny; j++)
    for (int i = 0; i < g.nx; i++) {
      if (solidCell(g, label, i, j - 1) || solidCell(g, label, i, j)) continue;
      v[idxV(g.nx, i, j)] += half * (fy[idxP(g.nx, i, j - 1)] + fy[idxP(g.nx, i, j)]);
    }
}

// stir.ts:49-83
template <class T>
void applyStir(const Grid<T>& g, T* u, T* v, const uint8_t* label, T sx, T sy, T sr, T sdx, T sdy) {
  const T invR2 = T(1) / (sr * sr);
  const T reach = T(3) * sr;
  const int c0 = (int)std::floor((sx - reach) / g.h), c1 = (int)std::ceil((sx + reach) / g.h);
  const int r0 = (int)std::floor((sy - reach) / g.h), r1 = (int)std::ceil((sy + reach) / g.h);
  auto clampi = [](int a, int lo, int hi) { return std::min(std::max(a, lo), hi); };
  for (int j = clampi(r0, 0, g.ny - 1); j <= clampi(r1, 0, g.ny - 1); j++) {
    T dy = (T(j) + T(0.5)) * g.h - sy;
    for (int i = clampi(c0, 1, g.nx - 1); i <= clampi(c1, 1, g.nx - 1); i++) {
      if (solidCell(g, label, i - 1, j) || solidCell(g, label, i, j)) continue;
      T dx = T(i) * g.h - sx;
      u[idxU(g.nx, i, j)] += sdx * std::exp(-(dx * dx + dy * dy) * invR2);
    }
  }
  for (int j = clampi(r0, 1, g.ny - 1); j <= clampi(r1, 1, g.ny - 1); j++) {
    T dy = T(j) * g.h - sy;
    for (int i = clampi(c0, 0, g.nx - 1); i <= clampi(c1, 0, g.nx - 1); i++) {
      if (solidCell(g, label, i, j - 1) || solidCell(g, label, i, j)) continue;
      T dx = (T(i) + T(0.5)) * g.h - sx;
      v[idxV(g.nx, i, j)] += sdy * std::exp(-(dx * dx + dy * dy) * invR2);
    }
  }
}

// ------------------------------------------------------------------- dye

// dye.ts:158-175 — data = 3 value planes then 1 coverage plane, pnx*pny each.
template <class T>
void applyDyePatch(const Grid<T>& dg, T* const* dye, int pi0, int pj0, int pnx, int pny, const float* data) {
  const long cells = (long)pnx * pny;
  for (int j = 0; j < pny; j++) {
    int dj = pj0 + j;
    if (dj < 0 || dj >= dg.ny) continue;
    for (int i = 0; i < pnx; i++) {
      int di = pi0 + i;
      if (di < 0 || di >= dg.nx) continue;
      long s = i + (long)j * pnx;
      T cov = T(data[DYE_CHANNELS * cells + s]);
      if (cov == T(0)) continue;
      long k = idxP(dg.nx, di, dj);
      for (int c = 0; c < DYE_CHANNELS; c++) dye[c][k] += cov * (T(data[c * cells + s]) - dye[c][k]);
    }
  }
}

// simulation.ts:243-247
inline double dyeKeepFor(double decay, double dt) { return decay > 0 ? std::exp(-decay * dt) : 1.0; }

// ------------------------------------------------------------ the step

// simulation.ts:134-234, reduced to what the projection step reads, plus the
// NEW knobs (alpha, confinement, multigrid shape and cycle cap).
struct StepParams {
  double cflTarget = 2.0, dtMax = 1.0 / 30.0, rho = 1.0;
  int macCormack = 0;
  int solver = 0;  // 0 = red-black SOR, 1 = multigrid, 2 = lexicographic SOR
  int pressureIters = 100;
  double omega = 1.9, tol = 5e-3;
  double dyeDecay[3] = {0, 0, 0};
  double beta = 0, alpha = 0, confinement = 0;
  MgShape mg;
  int mgMaxCycles = 3;
  int mixed = 0;  // NEW: defect correction around the multigrid, 1: float64 pressure, 2: double-float (float32 only)
  int warmExtrapolate = 0;  // NEW: the multigrid starts from 2 p(n) - p(n-1) on fluid cells
  int residualEvery = 1;    // simulation.ts:193-206, 233
};

template <class T>
struct Simulation {
  Grid<T> g, dg;
  StepParams prm;
  std::vector<T> u, v, p, div, uNext, vNext, uHat, vHat, qHat, fx, fy;
  // the post-step divergence (simulation.ts:539-540), kept apart from `div`
  // (the solve's input, which the reference reuses for it) so both can be
  // read; divPostStep is the index of the step that last computed it
  std::vector<T> divPost;
  long long steps = 0, divPostStep = -1;
  std::vector<double> p64;  // the pressure when prm.mixed
  std::vector<double> pPrev64;  // the previous step's pressure (warmExtrapolate, mixed)
  std::vector<T> pPrev;         // the previous step's pressure (warmExtrapolate)
  std::vector<float> pdf, pPrevDF;  // the double-float pressure and its previous value (mixed = 2, float32)
  std::vector<uint8_t> label;
  std::vector<T> dye[DYE_CHANNELS], dyeNext[DYE_CHANNELS];
  std::vector<float> patch;
  int pi0 = 0, pj0 = 0, pnx = 0, pny = 0;
  Multigrid<T> mg;
  double time = 0;
  T dt = 0;
  int iters = 0;
  double lastRelRes = -1;
  // simulation.ts:468-472, 504: a one-shot stir taken by the next step
  bool stirPending = false;
  T stir[5] = {0, 0, 0, 0, 0};

  Simulation(int nx, int ny, int dyeScale, const StepParams& p_) : prm(p_) {
    g = {nx, ny, T(1.0 / ny)};  // simulation.ts:365, h = 1/ny
    int s = std::max(1, dyeScale);
    dg = s == 1 ? g : Grid<T>{nx * s, ny * s, T(1.0 / (double)(ny * s))};
    long n = (long)nx * ny, nu = (long)(nx + 1) * ny, nv = (long)nx * (ny + 1), nd = (long)dg.nx * dg.ny;
    u.assign(nu, 0); v.assign(nv, 0); p.assign(n, 0); div.assign(n, 0); divPost.assign(n, 0);
    uNext.assign(nu, 0); vNext.assign(nv, 0); uHat.assign(nu, 0); vHat.assign(nv, 0);
    qHat.assign(nd, 0); fx.assign(n, 0); fy.assign(n, 0);
    label.assign(n, FLUID);
    p64.assign(n, 0.0);
    pPrev64.assign(n, 0.0);
    pPrev.assign(n, 0);
    pdf.assign(2 * n, 0.0f);
    pPrevDF.assign(2 * n, 0.0f);
    for (int c = 0; c < DYE_CHANNELS; c++) { dye[c].assign(nd, 0); dyeNext[c].assign(nd, 0); }
    mg.shape = prm.mg;
  }

  // mixed = 2 keeps the pressure as float pairs; the float64 instantiation
  // (the precision oracle) runs every mixed mode as float64.
  bool useDF() const { return prm.mixed == 2 && std::is_same<T, float>::value; }

  // The refined pressure (p64 / pdf) from the float pressure p, as an upload
  // of p sets it.
  void seedRefined() {
    for (size_t k = 0; k < p.size(); k++) {
      p64[k] = (double)p[k];
      pdf[2 * k] = (float)p[k];
      pdf[2 * k + 1] = 0.0f;
    }
    pPrev64 = p64;
    pPrevDF = pdf;
  }

  // simulation.ts:451-459
  T maxFaceSpeed() const {
    T m = 0;
    for (T x : u) m = std::max(m, std::fabs(x));
    for (T x : v) m = std::max(m, std::fabs(x));
    return m;
  }

  // simulation.ts:467-587 (CPU phase-wise path), with the NEW confinement and
  // alpha terms at the body-force seam. Returns pressure iterations used.
  int step() {
    const T uMax = maxFaceSpeed();
    const T cfl = T(prm.cflTarget), dtMax = T(prm.dtMax), rho = T(prm.rho);
    dt = uMax > T(1e-9) ? std::min(dtMax, (cfl * g.h) / uMax) : dtMax;
    const T scale = (rho * g.h * g.h) / dt;
    const T gradScale = dt / (rho * g.h);

    if (prm.macCormack)
      advectVelocityMacCormack(g, u.data(), v.data(), uHat.data(), vHat.data(), uNext.data(), vNext.data(),
                               label.data(), dt);
    else
      advectVelocity(g, u.data(), v.data(), uNext.data(), vNext.data(), label.data(), dt);
    std::swap(u, uNext);
    std::swap(v, vNext);
    // simulation.ts:504 — between advection and the body forces
    if (stirPending) {
      applyStir(g, u.data(), v.data(), label.data(), stir[0], stir[1], stir[2], stir[3], stir[4]);
      stirPending = false;
    }

    // Body forces: confinement is evaluated on the advected velocity, before
    // buoyancy changes it, then both are added (buoyancy first).
    if (prm.confinement != 0) confinementForce(g, u.data(), v.data(), label.data(), T(prm.confinement), fx.data(), fy.data());
    applyBuoyancy(g, dg, v.data(), dye[0].data(), dye[1].data(), label.data(), T(prm.beta), T(prm.alpha), dt);
    if (prm.confinement != 0) applyConfinement(g, u.data(), v.data(), label.data(), fx.data(), fy.data(), dt);

    computeDivergence(g, u.data(), v.data(), div.data());
    lastRelRes = -1;
    // NEW: second-order warm start p(n) + (p(n) - p(n-1)) on fluid cells
    if (prm.warmExtrapolate && prm.solver == 1) {
      const long n = (long)g.nx * g.ny;
      for (long k = 0; k < n; k++) {
        if (label[k] != FLUID) continue;
        if (useDF()) {
          if constexpr (std::is_same<T, float>::value) {
            const df::F2 t = df::at(pdf.data(), k);
            df::put(pdf.data(), k, df::add(t, df::add(t, df::neg(df::at(pPrevDF.data(), k)))));
            df::put(pPrevDF.data(), k, t);
          }
        } else if (prm.mixed) {
          const double t = p64[k];
          p64[k] = t + (t - pPrev64[k]);
          pPrev64[k] = t;
        } else {
          const T t = p[k];
          p[k] = t + (t - pPrev[k]);
          pPrev[k] = t;
        }
      }
    }
    if (prm.solver == 1 && useDF()) {
      if constexpr (std::is_same<T, float>::value) {
        iters = solveMixedDF(mg, g, pdf.data(), div.data(), label.data(), scale, prm.mgMaxCycles, prm.tol,
                             &lastRelRes);
        for (size_t k = 0; k < p.size(); k++) p[k] = df::round(df::at(pdf.data(), (long)k));
      }
    } else if (prm.solver == 1 && prm.mixed) {
      iters = solveMixed(mg, g, p64.data(), div.data(), label.data(), scale, prm.mgMaxCycles, prm.tol, &lastRelRes);
      for (size_t k = 0; k < p.size(); k++) p[k] = (T)p64[k];
    } else if (prm.solver == 1) {
      iters = mg.solve(g, p.data(), div.data(), label.data(), scale, prm.mgMaxCycles, prm.tol, &lastRelRes);
    } else if (prm.solver == 0) {
      iters = solvePressureRedBlack(g, p.data(), div.data(), label.data(), scale, prm.pressureIters, T(prm.omega), prm.tol);
    } else {
      iters = solvePressure(g, p.data(), div.data(), label.data(), scale, prm.pressureIters, T(prm.omega), prm.tol);
    }
    if (prm.solver == 1 && useDF()) {
      if constexpr (std::is_same<T, float>::value)
        subtractGradientDF(g, pdf.data(), u.data(), v.data(), label.data(), gradScale);
    } else if (prm.solver == 1 && prm.mixed)
      subtractGradient64(g, p64.data(), u.data(), v.data(), label.data(), gradScale);
    else
      subtractGradient(g, p.data(), u.data(), v.data(), label.data(), gradScale);
    applyOutflow(g, u.data(), v.data(), label.data());
    // simulation.ts:539-540 — the residual diagnostic; `steps` counts every
    // step taken (simulation.ts:324-326, 586)
    if (prm.residualEvery > 0 && steps % prm.residualEvery == 0) {
      computeDivergence(g, u.data(), v.data(), divPost.data());
      divPostStep = steps;
    }

    for (int c = 0; c < DYE_CHANNELS; c++) {
      if (prm.macCormack)
        advectScalarMacCormack(g, u.data(), v.data(), dye[c].data(), qHat.data(), dyeNext[c].data(), label.data(), dt, dg);
      else
        advectScalar(g, u.data(), v.data(), dye[c].data(), dyeNext[c].data(), label.data(), dt, dg);
      std::swap(dye[c], dyeNext[c]);
    }
    // simulation.ts:569-576 — decay after advection, per channel.
    for (int c = 0; c < DYE_CHANNELS; c++) {
      T keep = T(dyeKeepFor(prm.dyeDecay[c], (double)dt));
      if (keep == T(1)) continue;
      for (T& q : dye[c]) q *= keep;
    }
    if (pnx > 0 && pny > 0) {
      T* planes[3] = {dye[0].data(), dye[1].data(), dye[2].data()};
      applyDyePatch(dg, planes, pi0, pj0, pnx, pny, patch.data());
    }
    time += (double)dt;
    steps++;
    return iters;
  }
};

}  // namespace orc
