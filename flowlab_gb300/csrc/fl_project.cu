// The projection's glue passes (src/core/divergence.ts, subtractGradient.ts,
// boundaries.ts, buoyancy.ts, stir.ts, dye.ts, vorticity.ts; WGSL twin
// src/gpu/project.wgsl) plus the NEW vorticity confinement and the device-
// side CFL reduction that sets the next step's dt.
#include <algorithm>
#include <cmath>

#include "fl_internal.h"

namespace fl {

// vorticity.ts:9-14
__device__ __forceinline__ float curl_at_corner(const float* __restrict__ u, const float* __restrict__ v, int nx,
                                                const Spacing& h, int i, int j) {
  return over(v[i + j * nx] - v[(i - 1) + j * nx], h) -
         over(u[i + j * (nx + 1)] - u[i + (j - 1) * (nx + 1)], h);
}

// vorticity.ts:24-42 — corner curls averaged to the centre, clamped at walls.
__global__ void k_vorticity(int nx, int ny, Spacing h, const float* __restrict__ u, const float* __restrict__ v,
                            float* __restrict__ w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const int hiI = nx - 1, hiJ = ny - 1;
  const int j0 = min(max(j, 1), hiJ), j1 = min(max(j + 1, 1), hiJ);
  const int i0 = min(max(i, 1), hiI), i1 = min(max(i + 1, 1), hiI);
  w[i + j * nx] = 0.25f * (curl_at_corner(u, v, nx, h, i0, j0) + curl_at_corner(u, v, nx, h, i1, j0) +
                                 curl_at_corner(u, v, nx, h, i0, j1) + curl_at_corner(u, v, nx, h, i1, j1));
}

// NEW — vorticity confinement force at cell centres (Fedkiw, Stam & Jensen
// 2001): N = grad|w| / (|grad|w|| + 1e-20), f = eps*h * (N_y w, -N_x w),
// zero in solid cells. Centred differences, one-sided at the walls.
__global__ void k_confinement_force(int nx, int ny, Spacing h1, Spacing h2, const float* __restrict__ w,
                                    const uint8_t* __restrict__ label, float epsh, float* __restrict__ fx,
                                    float* __restrict__ fy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const int k = i + j * nx;
  if (label[k] == SOLID) {
    fx[k] = 0.0f;
    fy[k] = 0.0f;
    return;
  }
  const int ie = min(i + 1, nx - 1), iw = max(i - 1, 0);
  const int jn = min(j + 1, ny - 1), js = max(j - 1, 0);
  // (ie-iw)*h is h or 2h: both powers of two when h is one
  const float gx = over(fabsf(w[ie + j * nx]) - fabsf(w[iw + j * nx]), ie - iw == 2 ? h2 : h1);
  const float gy = over(fabsf(w[i + jn * nx]) - fabsf(w[i + js * nx]), jn - js == 2 ? h2 : h1);
  const float mag = sqrtf(gx * gx + gy * gy) + 1e-20f;
  const float Nx = gx / mag, Ny = gy / mag;
  const float wk = w[k];
  fx[k] = epsh * (Ny * wk);
  fy[k] = epsh * (-(Nx * wk));
}

// k_vorticity and k_confinement_force in one pass: a 32 x 8 tile of cells
// computes the vorticity of its cells and a one-cell ring into shared
// memory (the same corner-curl formula and clamping), then the confinement
// force of its own cells from it. u and v are only read here; the forces
// are applied by k_forces afterwards.
__global__ void __launch_bounds__(256) k_vort_confine(int nx, int ny, Spacing h, Spacing h1, Spacing h2,
                                                      const float* __restrict__ u, const float* __restrict__ v,
                                                      const uint8_t* __restrict__ label, float epsh,
                                                      float* __restrict__ fx, float* __restrict__ fy) {
  constexpr int TX = 32, TY = 8;
  __shared__ float ws[TY + 2][TX + 2];
  const int X0 = blockIdx.x * TX, Y0 = blockIdx.y * TY;
  const int t = threadIdx.x + TX * threadIdx.y;
  const int hiI = nx - 1, hiJ = ny - 1;
  for (int e = t; e < (TX + 2) * (TY + 2); e += TX * TY) {
    const int lx = e % (TX + 2), ly = e / (TX + 2);
    const int i = X0 - 1 + lx, j = Y0 - 1 + ly;
    float wv = 0.0f;
    if (i >= 0 && j >= 0 && i < nx && j < ny) {
      const int j0 = min(max(j, 1), hiJ), j1 = min(max(j + 1, 1), hiJ);
      const int i0 = min(max(i, 1), hiI), i1 = min(max(i + 1, 1), hiI);
      wv = 0.25f * (curl_at_corner(u, v, nx, h, i0, j0) + curl_at_corner(u, v, nx, h, i1, j0) +
                    curl_at_corner(u, v, nx, h, i0, j1) + curl_at_corner(u, v, nx, h, i1, j1));
    }
    ws[ly][lx] = wv;
  }
  __syncthreads();
  const int i = X0 + threadIdx.x, j = Y0 + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const int k = i + j * nx;
  if (label[k] == SOLID) {
    fx[k] = 0.0f;
    fy[k] = 0.0f;
    return;
  }
  const int ie = min(i + 1, nx - 1), iw = max(i - 1, 0);
  const int jn = min(j + 1, ny - 1), js = max(j - 1, 0);
  const int lx = threadIdx.x + 1, ly = threadIdx.y + 1;
  const float gx = over(fabsf(ws[ly][lx + (ie - i)]) - fabsf(ws[ly][lx - (i - iw)]), ie - iw == 2 ? h2 : h1);
  const float gy = over(fabsf(ws[ly + (jn - j)][lx]) - fabsf(ws[ly - (j - js)][lx]), jn - js == 2 ? h2 : h1);
  const float mag = sqrtf(gx * gx + gy * gy) + 1e-20f;
  const float Nx = gx / mag, Ny = gy / mag;
  const float wk = ws[ly][lx];
  fx[k] = epsh * (Ny * wk);
  fy[k] = epsh * (-(Nx * wk));
}

// Body forces on the faces they may write (buoyancy.ts:70-88 bounds for v,
// stir.ts:49-83 bounds for u): v += (beta*dt)*T + (-alpha*dt)*s, then the
// confinement face average. One thread per (u face, v face) pair, in place:
// every write depends only on the thread's own face.
__global__ void __launch_bounds__(256) k_forces(int nx, int ny, float h, int dnx, int dny, Spacing dh,
                                                float* __restrict__ u, float* __restrict__ v,
                                                const float* __restrict__ dye, const uint8_t* __restrict__ label,
                                                int beta_on, int alpha_on, int conf_on,
                                                const float* __restrict__ fx, const float* __restrict__ fy,
                                                const StepScalars* __restrict__ sc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (conf_on && i >= 1 && i < nx && j < ny) {
    if (!(solid_cell(label, nx, ny, i - 1, j) || solid_cell(label, nx, ny, i, j))) {
      const int k = i + j * (nx + 1);
      u[k] += sc->half_dt * (fx[(i - 1) + j * nx] + fx[i + j * nx]);
    }
  }
  if (i < nx && j >= 1 && j < ny) {
    if (!(solid_cell(label, nx, ny, i, j - 1) || solid_cell(label, nx, ny, i, j))) {
      const int k = i + j * nx;
      const float x = ((float)i + 0.5f) * h;
      const float y = (float)j * h;
      const int dcells = dnx * dny;
      float vk = v[k];
      if (beta_on) vk += sc->gain_beta * sample_p(dye, dnx, dny, dh, x, y);
      if (alpha_on) vk += sc->gain_alpha * sample_p(dye + dcells, dnx, dny, dh, x, y);
      if (conf_on) vk += sc->half_dt * (fy[i + (j - 1) * nx] + fy[i + j * nx]);
      v[k] = vk;
    }
  }
}

// divergence.ts:17-25. as_rhs: write b = (-scale)*div (pressureMultigrid.ts:
// 311) instead of div. Also accumulates the sum of squares of what it writes
// and the count over FLUID cells (pressure.ts:177-186's fluidDivRms).
__global__ void __launch_bounds__(256) k_divergence(int nx, int ny, float h, const float* __restrict__ u,
                                                    const float* __restrict__ v, float* __restrict__ out, int as_rhs,
                                                    const uint8_t* __restrict__ label,
                                                    const StepScalars* __restrict__ sc, StepAccum* acc,
                                                    float* __restrict__ out_lo) {
  __shared__ double red[32];
  __shared__ unsigned long long redn[32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float2 sq = make_float2(0.0f, 0.0f);
  unsigned long long n = 0;
  const float coef = 1.0f / h;
  const float ns = as_rhs ? sc->neg_scale : 0.0f;
  // rows strided over a bounded grid, so that few blocks feed the atomics
  // unrolled so that several rows' loads are in flight per thread
#pragma unroll 4
  for (int j = blockIdx.y * blockDim.y + threadIdx.y; j < ny; j += gridDim.y * blockDim.y) {
    if (i >= nx) break;
    const int k = i + j * nx;
    const float d = coef * (u[(i + 1) + j * (nx + 1)] - u[i + j * (nx + 1)] + v[i + (j + 1) * nx] -
                            v[i + j * nx]);
    const float o = as_rhs ? ns * d : d;
    out[k] = o;
    // the rounding error of b = (-scale) * div, exactly (an FMA of the
    // product against its rounded value): b + b_lo is the exact product
    if (out_lo) out_lo[k] = as_rhs ? __fmaf_rn(ns, d, -o) : 0.0f;
    if (label != nullptr && label[k] == FLUID) {
      // the square as an exact pair (product + FMA error) added to a
      // double-float sum: float32 work per cell, one widening per thread
      const float q = __fmul_rn(o, o);
      sq = df_add(sq, make_float2(q, __fmaf_rn(o, o, -q)));
      n += 1;
    }
  }
  if (acc == nullptr) return;
  double bs = block_sum_df(sq, reinterpret_cast<float2*>(red));
  unsigned long long bn = block_sum_u64(n, redn);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    atomicAdd(&acc->b_sq, bs);
    atomicAdd(&acc->n_fluid, bn);
  }
}

// subtractGradient.ts:40-61 then applyOutflow (boundaries.ts:115-143). Thread
// (i,j) owns u face (i,j) and v face (i,j). Outflow's writes land on the
// faces of the edge rows/columns; each is owned by the thread that computes
// the value it copies, so every face has exactly one writer:
//   u(1,j) and u(0,j): thread (1,j); u(nx-1,j) and u(nx,j): thread (nx-1,j).
// With nx == 2 both edges meet at face 1, handled left then right as the
// reference's loop order does.
// Pressure difference between two cells: float32, or with a float64
// pressure the difference formed in double and rounded once (the rounding
// on the integer pipe: d2f_rn equals the conversion instruction), or with
// the double-float pressure (`df`) the pairs' difference rounded once.
__device__ __forceinline__ float pdiff(const float* __restrict__ p, const double* __restrict__ p64, bool df, int a,
                                       int b) {
  if (p64 && df) {
    const float2* q = reinterpret_cast<const float2*>(p64);
    return df_diff(q[a], q[b]);
  }
  return p64 ? d2f_rn(p64[a] - p64[b]) : p[a] - p[b];
}

__device__ __forceinline__ float projected_u(const float* __restrict__ p, const double* __restrict__ p64, bool df,
                                             const float* __restrict__ u, const uint8_t* __restrict__ label, int nx,
                                             int ny, int i, int j, float gs, bool subtract) {
  float val = u[i + j * (nx + 1)];
  if (subtract && i >= 1 && i < nx) {
    if (!(solid_or_outside(label, nx, ny, i - 1, j) || solid_or_outside(label, nx, ny, i, j)))
      val -= gs * pdiff(p, p64, df, i + j * nx, (i - 1) + j * nx);
  }
  return val;
}
__device__ __forceinline__ float projected_v(const float* __restrict__ p, const double* __restrict__ p64, bool df,
                                             const float* __restrict__ v, const uint8_t* __restrict__ label, int nx,
                                             int ny, int i, int j, float gs, bool subtract) {
  float val = v[i + j * nx];
  if (subtract && j >= 1 && j < ny) {
    if (!(solid_or_outside(label, nx, ny, i, j - 1) || solid_or_outside(label, nx, ny, i, j)))
      val -= gs * pdiff(p, p64, df, i + j * nx, i + (j - 1) * nx);
  }
  return val;
}

__global__ void __launch_bounds__(256) k_subtract_outflow(int nx, int ny, const float* __restrict__ p,
                                                          const double* __restrict__ p64a,
                                                          const double* __restrict__ p64b,
                                                          const SolveCtl* __restrict__ ctl, float* __restrict__ u,
                                                          float* __restrict__ v, const uint8_t* __restrict__ label,
                                                          const StepScalars* __restrict__ sc, int subtract,
                                                          int outflow, int df, float* __restrict__ p32_out) {
  // the float64 pressure, when there is one, is the buffer ctl->par names
  const double* p64 = p64a ? (ctl->par ? p64b : p64a) : nullptr;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  // the refined pressure rounded to float (as k_select_p64 rounds it), for
  // a readback that then needs no kernel of its own
  if (p32_out != nullptr && p64 != nullptr && i < nx && j < ny) {
    const int k = i + j * nx;
    // (d2f_rn: the float64 rounding on the integer pipe, so that the
    // double-float case carries no predicated float64 conversion)
    p32_out[k] = df ? df_round(reinterpret_cast<const float2*>(p64)[k]) : d2f_rn(p64[k]);
  }
  const float gs = subtract ? sc->grad_scale : 0.0f;
  // u faces: threads 1..nx-1 write; faces 0 and nx are written only by outflow.
  if (j < ny && i >= 1 && i < nx) {
    float val = projected_u(p, p64, df, u, label, nx, ny, i, j, gs, subtract);
    if (outflow) {
      if (i == 1 && label[0 + j * nx] == AIR) {
        val = smin(val, 0.0f);
        u[0 + j * (nx + 1)] = val;
      }
      if (i == nx - 1 && label[(nx - 1) + j * nx] == AIR) {
        val = smax(val, 0.0f);
        u[nx + j * (nx + 1)] = val;
      }
    }
    u[i + j * (nx + 1)] = val;
  }
  if (i < nx && j >= 1 && j < ny) {
    float val = projected_v(p, p64, df, v, label, nx, ny, i, j, gs, subtract);
    if (outflow) {
      if (j == 1 && label[i] == AIR) {
        val = smin(val, 0.0f);
        v[i] = val;
      }
      if (j == ny - 1 && label[i + (ny - 1) * nx] == AIR) {
        val = smax(val, 0.0f);
        v[i + ny * nx] = val;
      }
    }
    v[i + j * nx] = val;
  }
}

// max |u|, |v| over every face (simulation.ts:451-459). The last block to
// finish turns it into the next step's scalars (simulation.ts:474-479,
// 243-247) and adds this step's dt to the device clock — no host round trip.
// The next step's scalars from the max face speed: simulation.ts:477-479,
// evaluated in float32 in the reference's order, and the per-channel keep
// factors of the dye decay (simulation.ts:243-247).
__device__ StepScalars cfl_scalars(float umax, float h, float cfl, float dt_max, float rho, double d0, double d1,
                                   double d2, float beta, float alpha) {
  const float dt = umax > 1e-9f ? smin(dt_max, (cfl * h) / umax) : dt_max;
  StepScalars s;
  s.dt = dt;
  s.scale = (rho * h * h) / dt;
  s.grad_scale = dt / (rho * h);
  const double dd = (double)dt;
  s.keep[0] = d0 > 0 ? (float)exp(-d0 * dd) : 1.0f;
  s.keep[1] = d1 > 0 ? (float)exp(-d1 * dd) : 1.0f;
  s.keep[2] = d2 > 0 ? (float)exp(-d2 * dd) : 1.0f;
  s.gain_beta = beta * dt;
  s.gain_alpha = -alpha * dt;
  s.half_dt = 0.5f * dt;
  s.neg_scale = -s.scale;
  for (int q = 0; q < 6; q++) s.pad[q] = 0;
  return s;
}

__global__ void __launch_bounds__(256) k_max_speed(long nu, long nv, const float* __restrict__ u,
                                                   const float* __restrict__ v, StepAccum* acc,
                                                   StepScalars* sc_next, double* time_dev, float h, float cfl,
                                                   float dt_max, float rho, double d0, double d1, double d2,
                                                   float beta, float alpha, int write_scalars, int add_time) {
  __shared__ float red[32];
  float m = 0.0f;
  const long stride = (long)gridDim.x * blockDim.x;
  const long t0 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  // 16-byte loads over the aligned body of each array (the max does not
  // depend on the order), the few trailing faces one by one
  const float4* u4 = reinterpret_cast<const float4*>(u);
  const float4* v4 = reinterpret_cast<const float4*>(v);
  for (long k = t0; k < nu / 4; k += stride) {
    const float4 q = u4[k];
    m = smax(m, smax(smax(fabsf(q.x), fabsf(q.y)), smax(fabsf(q.z), fabsf(q.w))));
  }
  for (long k = t0; k < nv / 4; k += stride) {
    const float4 q = v4[k];
    m = smax(m, smax(smax(fabsf(q.x), fabsf(q.y)), smax(fabsf(q.z), fabsf(q.w))));
  }
  for (long k = 4 * (nu / 4) + t0; k < nu; k += stride) m = smax(m, fabsf(u[k]));
  for (long k = 4 * (nv / 4) + t0; k < nv; k += stride) m = smax(m, fabsf(v[k]));
  float bm = block_max(m, red);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    atomicMax(&acc->max_speed_bits, __float_as_uint(bm));
    __threadfence();
    unsigned int done = atomicAdd(&acc->blocks_done, 1u);
    last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  const float umax = __uint_as_float(atomicExch(&acc->max_speed_bits, 0u));
  acc->blocks_done = 0u;
  acc->last_max_bits = __float_as_uint(umax);
  // The step that just finished ran with the current scalars: its dt joins
  // the clock before the scalars are replaced (simulation.ts:585).
  if (add_time && time_dev) *time_dev += (double)sc_next->dt;
  if (!write_scalars) return;
  *sc_next = cfl_scalars(umax, h, cfl, dt_max, rho, d0, d1, d2, beta, alpha);
}

// b = (-scale) * div with the fluid sum of squares (pressureMultigrid.ts:311,
// pressure.ts:177-186), for solves handed a divergence field.
__global__ void __launch_bounds__(256) k_scale_rhs(long n, const float* __restrict__ div, float* __restrict__ b,
                                                   float neg_scale, const uint8_t* __restrict__ label,
                                                   StepAccum* acc, float* __restrict__ b_lo) {
  __shared__ double red[32];
  __shared__ unsigned long long redn[32];
  float2 sq = make_float2(0.0f, 0.0f);
  unsigned long long cnt = 0;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    const float o = b ? neg_scale * div[k] : div[k];
    if (b) b[k] = o;
    if (b && b_lo) b_lo[k] = __fmaf_rn(neg_scale, div[k], -o);
    if (label[k] == FLUID) {
      const float q = __fmul_rn(o, o);
      sq = df_add(sq, make_float2(q, __fmaf_rn(o, o, -q)));
      cnt += 1;
    }
  }
  const double bs = block_sum_df(sq, reinterpret_cast<float2*>(red));
  const unsigned long long bn = block_sum_u64(cnt, redn);
  if (threadIdx.x == 0) {
    atomicAdd(&acc->b_sq, bs);
    atomicAdd(&acc->n_fluid, bn);
  }
}

// boundaries.ts:45-64 on the device (project.wgsl:155-165 for the faces),
// extended to p and dye as the host version does.
__global__ void k_commit_labels(int nx, int ny, const uint8_t* __restrict__ label, float* __restrict__ p,
                                float* __restrict__ u, float* __restrict__ v, float* __restrict__ dye,
                                long dye_cells, double* __restrict__ p64a, double* __restrict__ p64b,
                                const SolveCtl* __restrict__ ctl) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i < nx && j < ny) {
    const int k = i + j * nx;
    const uint8_t l = label[k];
    if (l != FLUID) {
      if (p) p[k] = 0.0f;
      // the float64 pressure of the defect correction keeps the same rule
      if (p64a) (ctl->par ? p64b : p64a)[k] = 0.0;
      if (l == SOLID && dye && k < dye_cells)
        for (int c = 0; c < DYE_CHANNELS; c++) dye[k + c * dye_cells] = 0.0f;
    }
  }
  if (i <= nx && j < ny) {
    if (solid_cell(label, nx, ny, i - 1, j) || solid_cell(label, nx, ny, i, j)) u[i + j * (nx + 1)] = 0.0f;
  }
  if (i < nx && j <= ny) {
    if (solid_cell(label, nx, ny, i, j - 1) || solid_cell(label, nx, ny, i, j)) v[i + j * nx] = 0.0f;
  }
}

// stir.ts:49-83 — every interior face (the WGSL version's whole-grid sweep,
// project.wgsl:180-207); faces beyond three radii get exp() of a large
// negative number, which the host version skips by its bounding box. The
// host's box is replicated here so both write exactly the same faces.
__global__ void k_stir(int nx, int ny, float h, float* __restrict__ u, float* __restrict__ v,
                       const uint8_t* __restrict__ label, float sx, float sy, float sr, float sdx, float sdy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const float invR2 = 1.0f / (sr * sr);
  const float reach = 3.0f * sr;
  const int c0 = (int)floorf((sx - reach) / h), c1 = (int)ceilf((sx + reach) / h);
  const int r0 = (int)floorf((sy - reach) / h), r1 = (int)ceilf((sy + reach) / h);
  if (j >= min(max(r0, 0), ny - 1) && j <= min(max(r1, 0), ny - 1) && i >= min(max(c0, 1), nx - 1) &&
      i <= min(max(c1, 1), nx - 1) && i <= nx && j < ny) {
    if (!(solid_cell(label, nx, ny, i - 1, j) || solid_cell(label, nx, ny, i, j))) {
      const float dy = ((float)j + 0.5f) * h - sy;
      const float dx = (float)i * h - sx;
      u[i + j * (nx + 1)] += sdx * expf(-(dx * dx + dy * dy) * invR2);
    }
  }
  if (j >= min(max(r0, 1), ny - 1) && j <= min(max(r1, 1), ny - 1) && i >= min(max(c0, 0), nx - 1) &&
      i <= min(max(c1, 0), nx - 1) && i < nx && j <= ny) {
    if (!(solid_cell(label, nx, ny, i, j - 1) || solid_cell(label, nx, ny, i, j))) {
      const float dy = (float)j * h - sy;
      const float dx = ((float)i + 0.5f) * h - sx;
      v[i + j * nx] += sdy * expf(-(dx * dx + dy * dy) * invR2);
    }
  }
}

// dye.ts:158-175 (project.wgsl:363-379)
__global__ void k_dye_patch(int dnx, int dny, float* __restrict__ dye, const float* __restrict__ patch, int pi0,
                            int pj0, int pnx, int pny) {
  const int pi = blockIdx.x * blockDim.x + threadIdx.x;
  const int pj = blockIdx.y * blockDim.y + threadIdx.y;
  if (pi >= pnx || pj >= pny) return;
  const int di = pi0 + pi, dj = pj0 + pj;
  if (di < 0 || dj < 0 || di >= dnx || dj >= dny) return;
  const long pc = (long)pnx * pny;  // 64-bit: the planes together may exceed 2^31 values
  const int s = pi + pj * pnx;
  const float cov = patch[DYE_CHANNELS * pc + s];
  if (cov == 0.0f) return;
  const long cells = (long)dnx * dny;
  const int k = di + dj * dnx;
  for (int c = 0; c < DYE_CHANNELS; c++) dye[k + c * cells] += cov * (patch[c * pc + s] - dye[k + c * cells]);
}

__global__ void k_convert_f64_f32(const double* __restrict__ a, float* __restrict__ b, long n) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    b[k] = (float)a[k];
}
__global__ void k_convert_f32_f64(const float* __restrict__ a, double* __restrict__ b, long n) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    b[k] = (double)a[k];
}
// to the double-float pressure: (p, 0) from float32, the rounded double and
// its remainder from float64
__global__ void k_convert_f32_df(const float* __restrict__ a, float2* __restrict__ b, long n) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    b[k] = make_float2(a[k], 0.0f);
}
__global__ void k_convert_f64_df(const double* __restrict__ a, float2* __restrict__ b, long n) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    b[k] = df_from_double(a[k]);
}

// ------------------------------------------------------------- launchers

static dim3 grid2(int w, int h, dim3 b) { return dim3((w + b.x - 1) / b.x, (h + b.y - 1) / b.y); }

void launch_vorticity(cudaStream_t s, int nx, int ny, float h, const float* u, const float* v, float* w) {
  dim3 b(32, 8);
  k_vorticity<<<grid2(nx, ny, b), b, 0, s>>>(nx, ny, make_spacing(h), u, v, w);
}

void launch_confinement_force(cudaStream_t s, int nx, int ny, float h, const float* w, const uint8_t* label,
                              float eps, float* fx, float* fy) {
  dim3 b(32, 8);
  k_confinement_force<<<grid2(nx, ny, b), b, 0, s>>>(nx, ny, make_spacing(1.0f * h), make_spacing(2.0f * h), w,
                                                     label, eps * h, fx, fy);
}

void launch_vort_confine(cudaStream_t s, int nx, int ny, float h, const float* u, const float* v,
                         const uint8_t* label, float eps, float* fx, float* fy) {
  dim3 b(32, 8);
  k_vort_confine<<<grid2(nx, ny, b), b, 0, s>>>(nx, ny, make_spacing(h), make_spacing(1.0f * h),
                                                make_spacing(2.0f * h), u, v, label, eps * h, fx, fy);
}

void launch_forces(cudaStream_t s, int nx, int ny, float h, int dnx, int dny, float dh, float* u, float* v,
                   const float* dye, const uint8_t* label, bool beta_on, bool alpha_on, bool conf_on,
                   const float* fx, const float* fy, const StepScalars* sc) {
  dim3 b(32, 8);
  k_forces<<<grid2(nx + 1, ny + 1, b), b, 0, s>>>(nx, ny, h, dnx, dny, make_spacing(dh), u, v, dye, label, beta_on, alpha_on,
                                                  conf_on, fx, fy, sc);
}

void launch_divergence(cudaStream_t s, int nx, int ny, float h, const float* u, const float* v, float* out,
                       bool as_rhs, const uint8_t* label, const StepScalars* sc, StepAccum* acc, float* out_lo) {
  dim3 b(32, 8);
  dim3 g = grid2(nx, ny, b);
  // about four blocks per SM, rows strided: every block ends in same-word
  // atomics, which serialise
  g.y = std::min(g.y, std::max(1u, 608u / g.x));
  k_divergence<<<g, b, 0, s>>>(nx, ny, h, u, v, out, as_rhs, label, sc, acc, out_lo);
}

void launch_subtract_outflow(cudaStream_t s, int nx, int ny, const float* p, float* u, float* v,
                             const uint8_t* label, const StepScalars* sc, bool subtract, bool outflow,
                             const double* p64a, const double* p64b, const SolveCtl* ctl, bool df,
                             float* p32_out) {
  dim3 b(32, 8);
  k_subtract_outflow<<<grid2(nx + 1, ny + 1, b), b, 0, s>>>(nx, ny, p, p64a, p64b, ctl, u, v, label, sc, subtract,
                                                            outflow, df, p32_out);
}

void launch_scale_rhs(cudaStream_t s, long n, const float* div, float* b, float neg_scale, const uint8_t* label,
                      StepAccum* acc, float* b_lo) {
  long blocks = (n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  k_scale_rhs<<<(unsigned)blocks, 256, 0, s>>>(n, div, b, neg_scale, label, acc, b_lo);
}

// The end-of-step scan with the residual diagnostic folded in: each thread
// owns a cell and reads its four faces once, which covers every face, for
// the max face speed of the next step's CFL dt (as k_max_speed); on the
// steps the diagnostic runs (simulation.ts:539: residualEvery > 0 &&
// steps % residualEvery === 0, `steps` counting every step taken) it also
// writes the post-step divergence (divergence.ts:17-25) of every cell and
// sums its square and max over FLUID cells (viz/fieldView.ts:44-60). The
// last block finishes the CFL scalars, publishes the diagnostic's sums and
// counts the step.
__global__ void __launch_bounds__(256) k_cfl_residual(int nx, int ny, float h, const float* __restrict__ u,
                                                      const float* __restrict__ v, float* __restrict__ div_out,
                                                      const uint8_t* __restrict__ label, int every, DiagAccum* d,
                                                      StepAccum* acc, StepScalars* sc_next, double* time_dev,
                                                      float cfl, float dt_max, float rho, double d0, double d1,
                                                      double d2, float beta, float alpha, int write_scalars,
                                                      int add_time) {
  __shared__ double red[32];
  __shared__ unsigned long long redn[32];
  __shared__ float redm[32];
  __shared__ bool last;
  const unsigned long long step = d->counter;  // advanced only by the last block, after every block read it
  const bool on = every > 0 && step % (unsigned long long)every == 0;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float m = 0.0f, mx = 0.0f;
  float2 sq = make_float2(0.0f, 0.0f);
  unsigned long long n = 0;
  const float coef = 1.0f / h;
  // unrolled so that several rows' loads are in flight per thread
#pragma unroll 4
  for (int j = blockIdx.y * blockDim.y + threadIdx.y; j < ny; j += gridDim.y * blockDim.y) {
    if (i >= nx) break;
    const int ku = i + j * (nx + 1), kv = i + j * nx;
    const float u0 = u[ku], u1 = u[ku + 1], v0 = v[kv], v1 = v[kv + nx];
    m = smax(m, smax(smax(fabsf(u0), fabsf(u1)), smax(fabsf(v0), fabsf(v1))));
    if (on) {
      const float dv = coef * (u1 - u0 + v1 - v0);
      div_out[kv] = dv;
      if (label[kv] == FLUID) {
        const float q = __fmul_rn(dv, dv);
        sq = df_add(sq, make_float2(q, __fmaf_rn(dv, dv, -q)));
        mx = fmaxf(mx, fabsf(dv));
        n += 1;
      }
    }
  }
  const float bm = block_max(m, redm);
  double bs = 0.0;
  unsigned long long bn = 0;
  float bx = 0.0f;
  if (on) {  // the same for the whole block
    bs = block_sum_df(sq, reinterpret_cast<float2*>(red));
    bn = block_sum_u64(n, redn);
    __syncthreads();
    bx = block_max(mx, redm);
  }
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  const unsigned nblocks = gridDim.x * gridDim.y;
  if (tid == 0) {
    atomicMax(&acc->max_speed_bits, __float_as_uint(bm));
    if (on) {
      atomicAdd(&d->div_sq, bs);
      atomicAdd(&d->n_fluid, bn);
      // non-negative floats order as their bits
      atomicMax(&d->div_max_bits, __float_as_uint(bx));
    }
    __threadfence();
    const unsigned done = atomicAdd(&acc->blocks_done, 1u);
    last = done == nblocks - 1;
  }
  __syncthreads();
  if (!last || tid != 0) return;
  __threadfence();
  if (on) {
    d->last_sq = d->div_sq;
    d->last_n = d->n_fluid;
    d->last_max_bits = d->div_max_bits;
    d->last_step = (long long)step;
    d->div_sq = 0.0;
    d->n_fluid = 0ull;
    d->div_max_bits = 0u;
  }
  d->counter = step + 1;
  const float umax = __uint_as_float(atomicExch(&acc->max_speed_bits, 0u));
  acc->blocks_done = 0u;
  acc->last_max_bits = __float_as_uint(umax);
  // the step that just finished ran with the current scalars: its dt joins
  // the clock before the scalars are replaced (simulation.ts:585)
  if (add_time && time_dev) *time_dev += (double)sc_next->dt;
  if (write_scalars) sc_next[0] = cfl_scalars(umax, h, cfl, dt_max, rho, d0, d1, d2, beta, alpha);
}

void launch_cfl_residual(cudaStream_t s, int nx, int ny, float h, const float* u, const float* v, float* div_out,
                         const uint8_t* label, int every, DiagAccum* d, StepAccum* acc, StepScalars* sc_next,
                         double* time_dev, const fl_params* prm, bool write_scalars, bool add_time) {
  dim3 b(32, 8);
  dim3 g = grid2(nx, ny, b);
  // about four blocks per SM, rows strided: every block ends in same-word
  // atomics, which serialise
  g.y = std::min(g.y, std::max(1u, 608u / g.x));
  k_cfl_residual<<<g, b, 0, s>>>(nx, ny, h, u, v, div_out, label, every, d, acc, sc_next, time_dev,
                                 (float)prm->cfl_target, (float)prm->dt_max, (float)prm->rho, prm->dye_decay[0],
                                 prm->dye_decay[1], prm->dye_decay[2], (float)prm->beta, (float)prm->alpha,
                                 write_scalars, add_time);
}

// Fills and device-to-device copies inside the step and upload graphs run as
// kernels: as memset or memcpy nodes they would queue on the copy engine
// behind the host transfers of fl_step_host (measured: the upload graph took
// 64 us behind the dye upload, 43 us without it).
__global__ void __launch_bounds__(256) k_fill32(uint32_t* __restrict__ p, long n, uint32_t v) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) p[k] = v;
}

__global__ void __launch_bounds__(256) k_copy32(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, long n) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) dst[k] = src[k];
}

void launch_fill32(cudaStream_t s, void* p, long words, uint32_t v) {
  const long blocks = std::max(1L, std::min((words + 255) / 256, 152L * 8));
  k_fill32<<<(unsigned)blocks, 256, 0, s>>>(static_cast<uint32_t*>(p), words, v);
}

void launch_copy32(cudaStream_t s, const void* src, void* dst, long words) {
  const long blocks = std::max(1L, std::min((words + 255) / 256, 152L * 8));
  k_copy32<<<(unsigned)blocks, 256, 0, s>>>(static_cast<const uint32_t*>(src), static_cast<uint32_t*>(dst), words);
}

void launch_max_speed(cudaStream_t s, int nx, int ny, const float* u, const float* v, StepAccum* acc,
                      StepScalars* sc_next, double* time_dev, const fl_params* prm, float h, bool write_scalars,
                      bool add_time) {
  long nu = (long)(nx + 1) * ny, nv = (long)nx * (ny + 1);
  // few blocks, several 16-byte loads per thread: every block ends in two
  // atomics on the same words, which serialise
  long blocks = (nu / 4 + 255) / 256;
  if (blocks > 152 * 2) blocks = 152 * 2;
  if (blocks < 1) blocks = 1;
  k_max_speed<<<(unsigned)blocks, 256, 0, s>>>(nu, nv, u, v, acc, sc_next, time_dev, h, (float)prm->cfl_target,
                                              (float)prm->dt_max, (float)prm->rho, prm->dye_decay[0],
                                              prm->dye_decay[1], prm->dye_decay[2], (float)prm->beta,
                                              (float)prm->alpha, write_scalars, add_time);
}

void launch_commit_labels(cudaStream_t s, int nx, int ny, const uint8_t* label, float* p, float* u, float* v,
                          float* dye, long dye_cells, double* p64a, double* p64b, const SolveCtl* ctl) {
  dim3 b(32, 8);
  k_commit_labels<<<grid2(nx + 1, ny + 1, b), b, 0, s>>>(nx, ny, label, p, u, v, dye, dye_cells, p64a, p64b, ctl);
}

void launch_stir(cudaStream_t s, int nx, int ny, float h, float* u, float* v, const uint8_t* label,
                 const float* st) {
  dim3 b(32, 8);
  k_stir<<<grid2(nx + 1, ny + 1, b), b, 0, s>>>(nx, ny, h, u, v, label, st[0], st[1], st[2], st[3], st[4]);
}

void launch_dye_patch(cudaStream_t s, int dnx, int dny, float* dye, const float* patch, int pi0, int pj0, int pnx,
                      int pny) {
  if (!patch || pnx <= 0 || pny <= 0) return;
  dim3 b(32, 8);
  k_dye_patch<<<grid2(pnx, pny, b), b, 0, s>>>(dnx, dny, dye, patch, pi0, pj0, pnx, pny);
}

void launch_convert(cudaStream_t s, const void* src, int src_dtype, void* dst, int dst_dtype, long n) {
  long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  if (blocks < 1) blocks = 1;
  if (src_dtype == FL_F64 && dst_dtype == FL_F32)
    k_convert_f64_f32<<<(unsigned)blocks, 256, 0, s>>>((const double*)src, (float*)dst, n);
  else if (src_dtype == FL_F32 && dst_dtype == FL_F64)
    k_convert_f32_f64<<<(unsigned)blocks, 256, 0, s>>>((const float*)src, (double*)dst, n);
  else if (src_dtype == FL_F32 && dst_dtype == DT_DF)
    k_convert_f32_df<<<(unsigned)blocks, 256, 0, s>>>((const float*)src, (float2*)dst, n);
  else if (src_dtype == FL_F64 && dst_dtype == DT_DF)
    k_convert_f64_df<<<(unsigned)blocks, 256, 0, s>>>((const double*)src, (float2*)dst, n);
}

// A fixed-duration single-thread kernel (about 40 us, bounded by its loop
// count) queued ahead of each profiled phase, so that the phase's launches
// are submitted before the device reaches its start event.
__global__ void k_hold() {
  for (int k = 0; k < 40; k++) __nanosleep(1000);
}

void launch_hold(cudaStream_t s) { k_hold<<<1, 1, 0, s>>>(); }

// Second-order warm start (no reference counterpart): on fluid cells
// p = p + (p - p_prev) and p_prev = the old p, in float (the plain
// multigrid's pressure), float64 or double-float (`df`; the defect
// correction's current buffer, chosen by the device parity).
__global__ void k_extrapolate(long n, const uint8_t* __restrict__ label, float* __restrict__ p32,
                              float* __restrict__ pp32, double* __restrict__ p64a, double* __restrict__ p64b,
                              double* __restrict__ pp64, const SolveCtl* __restrict__ ctl, int df) {
  double* p64 = p64a ? (ctl->par ? p64b : p64a) : nullptr;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    if (label[k] != FLUID) continue;
    if (p64 && df) {
      float2* q = reinterpret_cast<float2*>(p64);
      float2* qq = reinterpret_cast<float2*>(pp64);
      const float2 t = q[k];
      q[k] = df_add(t, df_add(t, df_neg(qq[k])));
      qq[k] = t;
    } else if (p64) {
      const double t = p64[k];
      p64[k] = t + (t - pp64[k]);
      pp64[k] = t;
    } else {
      const float t = p32[k];
      p32[k] = t + (t - pp32[k]);
      pp32[k] = t;
    }
  }
}

void launch_extrapolate(cudaStream_t s, long n, const uint8_t* label, float* p32, float* pp32, double* p64a,
                        double* p64b, double* pp64, const SolveCtl* ctl, bool df) {
  long blocks = std::min((n + 255) / 256, 152L * 8);
  k_extrapolate<<<(unsigned)std::max(1L, blocks), 256, 0, s>>>(n, label, p32, pp32, p64a, p64b, pp64, ctl, df);
}

// out = p64[ctl->par] as float64 or rounded to float32 (the double-float
// pressure: hi + lo in double, or the pair rounded to float).
__global__ void k_select_p64(const SolveCtl* __restrict__ ctl, const double* __restrict__ p64a,
                             const double* __restrict__ p64b, void* __restrict__ out, int as_f64, long n, int df) {
  const double* src = ctl->par ? p64b : p64a;
  const float2* src2 = reinterpret_cast<const float2*>(src);
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    if (df && as_f64)
      static_cast<double*>(out)[k] = df_to_double(src2[k]);
    else if (df)
      static_cast<float*>(out)[k] = df_round(src2[k]);
    else if (as_f64)
      static_cast<double*>(out)[k] = src[k];
    else
      static_cast<float*>(out)[k] = (float)src[k];
  }
}

void launch_select_p64(cudaStream_t s, const SolveCtl* ctl, const double* p64a, const double* p64b, void* out,
                       bool as_f64, long n, bool df) {
  long blocks = std::min((n + 255) / 256, 152L * 8);
  k_select_p64<<<(unsigned)std::max(1L, blocks), 256, 0, s>>>(ctl, p64a, p64b, out, as_f64, n, df);
}

}  // namespace fl
