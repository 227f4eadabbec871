// Semi-Lagrangian / MacCormack advection of the MAC velocity and the dye
// (src/core/advect.ts:41-312; the reference's WGSL twin is
// src/gpu/advect.wgsl:225-356).
//
// Velocity: one launch over (nx+1) x (ny+1) threads covers both face grids —
// thread (i,j) owns u-face (i,j) where it exists and v-face (i,j) where it
// exists. MacCormack is two launches: the forward pass writes uHat, the
// correction fuses the reverse pass (read only at its own face) with the
// clamp, as the reverse pass's value is needed nowhere else.
//
// Dye: one backtrace per dye cell serves all three channels. The correction
// launch (or the forward launch for semi-Lagrangian) also applies the step's
// per-channel decay and the dye inlet patch, in that order (simulation.ts:
// 569-581), so the dye is touched once per step after advection.
//
// All reads of the carrier and source fields are gathers through the
// read-only cache; at the 1024^2 working set they are served from L2.
#include "fl_internal.h"

namespace fl {

// advect.ts:41-55
__device__ __forceinline__ void backtrace(const float* __restrict__ uc, const float* __restrict__ vc, int nx, int ny,
                                          const Spacing& h, float x, float y, float u0, float v0, float dt, float& bx,
                                          float& by) {
  float midX = x - 0.5f * dt * u0;
  float midY = y - 0.5f * dt * v0;
  bx = x - dt * sample_u(uc, nx, ny, h, midX, midY);
  by = y - dt * sample_v(vc, nx, ny, h, midX, midY);
}

// MODE 0: forward pass (advectFaces with src = carrier), writes `out`.
// MODE 1: MacCormack correction: `hat` is the forward result, `out` receives
//         clamp(hat + 0.5*(in - reverse(hat))) (advect.ts:177-210).
template <int MODE>
__global__ void __launch_bounds__(256) k_advect_velocity(int nx, int ny, Spacing h, const float* __restrict__ u_in,
                                                         const float* __restrict__ v_in,
                                                         const float* __restrict__ u_hat,
                                                         const float* __restrict__ v_hat, float* __restrict__ u_out,
                                                         float* __restrict__ v_out,
                                                         const uint8_t* __restrict__ label,
                                                         const StepScalars* __restrict__ sc, float2* __restrict__ bt_u,
                                                         float2* __restrict__ bt_v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const float dt = sc->dt;
  if (i <= nx && j < ny) {
    const int k = i + j * (nx + 1);
    if (solid_or_outside(label, nx, ny, i - 1, j) || solid_or_outside(label, nx, ny, i, j)) {
      u_out[k] = u_in[k];
    } else {
      const float x = (float)i * h.h;
      const float y = ((float)j + 0.5f) * h.h;
      const float u0 = u_in[k];
      const float v0 = sample_v(v_in, nx, ny, h, x, y);
      float bx, by;
      if (MODE == 0) {
        backtrace(u_in, v_in, nx, ny, h, x, y, u0, v0, dt, bx, by);
        if (bt_u != nullptr) bt_u[k] = make_float2(bx, by);
        u_out[k] = sample_u(u_in, nx, ny, h, bx, by);
      } else {
        backtrace(u_in, v_in, nx, ny, h, x, y, u0, v0, -dt, bx, by);
        const float ubar = sample_u(u_hat, nx, ny, h, bx, by);
        const float corrected = u_hat[k] + 0.5f * (u_in[k] - ubar);
        if (bt_u != nullptr) {
          const float2 b = bt_u[k];
          bx = b.x;
          by = b.y;
        } else {
          backtrace(u_in, v_in, nx, ny, h, x, y, u0, v0, dt, bx, by);
        }
        u_out[k] = clamp_stencil_u(u_in, nx, ny, h, bx, by, corrected);
      }
    }
  }
  if (i < nx && j <= ny) {
    const int k = i + j * nx;
    if (solid_or_outside(label, nx, ny, i, j - 1) || solid_or_outside(label, nx, ny, i, j)) {
      v_out[k] = v_in[k];
    } else {
      const float x = ((float)i + 0.5f) * h.h;
      const float y = (float)j * h.h;
      const float u0 = sample_u(u_in, nx, ny, h, x, y);
      const float v0 = v_in[k];
      float bx, by;
      if (MODE == 0) {
        backtrace(u_in, v_in, nx, ny, h, x, y, u0, v0, dt, bx, by);
        if (bt_v != nullptr) bt_v[k] = make_float2(bx, by);
        v_out[k] = sample_v(v_in, nx, ny, h, bx, by);
      } else {
        backtrace(u_in, v_in, nx, ny, h, x, y, u0, v0, -dt, bx, by);
        const float vbar = sample_v(v_hat, nx, ny, h, bx, by);
        const float corrected = v_hat[k] + 0.5f * (v_in[k] - vbar);
        if (bt_v != nullptr) {
          const float2 b = bt_v[k];
          bx = b.x;
          by = b.y;
        } else {
          backtrace(u_in, v_in, nx, ny, h, x, y, u0, v0, dt, bx, by);
        }
        v_out[k] = clamp_stencil_v(v_in, nx, ny, h, bx, by, corrected);
      }
    }
  }
}

// Dye. MODE 0 forward (advect.ts:241-270), MODE 1 correction (advect.ts:
// 294-311). TAIL applies decay then the inlet patch (simulation.ts:569-581,
// dye.ts:158-175) to the value this thread writes.
template <int MODE, bool TAIL>
__global__ void __launch_bounds__(256) k_advect_dye(int nx, int ny, Spacing h, int dnx, int dny, Spacing dh,
                                                    const float* __restrict__ u, const float* __restrict__ v,
                                                    const float* __restrict__ q_in, const float* __restrict__ q_hat,
                                                    float* __restrict__ q_out, const uint8_t* __restrict__ label,
                                                    const StepScalars* __restrict__ sc,
                                                    const float* __restrict__ patch, int pi0, int pj0, int pnx,
                                                    int pny, float2* __restrict__ bt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= dnx || j >= dny) return;
  // 64-bit: the three planes together may hold more than 2^31 values
  const long cells = (long)dnx * dny;
  const int k = i + j * dnx;
  const float dt = sc->dt;
  const float ratio = dh.h / h.h;
  const int lj = (int)floorf(((float)j + 0.5f) * ratio);
  const int li = (int)floorf(((float)i + 0.5f) * ratio);
  float q[DYE_CHANNELS];
  if (solid_or_outside(label, nx, ny, li, lj)) {
#pragma unroll
    for (int c = 0; c < DYE_CHANNELS; c++) q[c] = q_in[k + c * cells];
  } else {
    const float x = ((float)i + 0.5f) * dh.h;
    const float y = ((float)j + 0.5f) * dh.h;
    const float u0 = sample_u(u, nx, ny, h, x, y);
    const float v0 = sample_v(v, nx, ny, h, x, y);
    float bx, by;
    if (MODE == 0) {
      backtrace(u, v, nx, ny, h, x, y, u0, v0, dt, bx, by);
      if (bt != nullptr) bt[k] = make_float2(bx, by);
#pragma unroll
      for (int c = 0; c < DYE_CHANNELS; c++) q[c] = sample_p(q_in + c * cells, dnx, dny, dh, bx, by);
    } else {
      float rbx, rby;
      backtrace(u, v, nx, ny, h, x, y, u0, v0, -dt, rbx, rby);
      if (bt != nullptr) {
        const float2 b = bt[k];
        bx = b.x;
        by = b.y;
      } else {
        backtrace(u, v, nx, ny, h, x, y, u0, v0, dt, bx, by);
      }
#pragma unroll
      for (int c = 0; c < DYE_CHANNELS; c++) {
        const float qbar = sample_p(q_hat + c * cells, dnx, dny, dh, rbx, rby);
        const float corrected = q_hat[k + c * cells] + 0.5f * (q_in[k + c * cells] - qbar);
        q[c] = clamp_stencil_p(q_in + c * cells, dnx, dny, dh, bx, by, corrected);
      }
    }
  }
  if (TAIL) {
#pragma unroll
    for (int c = 0; c < DYE_CHANNELS; c++) {
      const float keep = sc->keep[c];
      if (keep != 1.0f) q[c] *= keep;
    }
    if (patch != nullptr) {
      const int pi = i - pi0, pj = j - pj0;
      if (pi >= 0 && pj >= 0 && pi < pnx && pj < pny) {
        const long pc = (long)pnx * pny;  // 64-bit: five planes
        const int s = pi + pj * pnx;
        const float cov = patch[DYE_CHANNELS * pc + s];
        if (cov != 0.0f) {
#pragma unroll
          for (int c = 0; c < DYE_CHANNELS; c++) q[c] += cov * (patch[c * pc + s] - q[c]);
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < DYE_CHANNELS; c++) q_out[k + c * cells] = q[c];
}

void launch_advect_velocity(cudaStream_t s, int nx, int ny, float h, int mac, const float* u_in, const float* v_in,
                            float* u_hat, float* v_hat, float* u_out, float* v_out, const uint8_t* label,
                            const StepScalars* sc, float2* bt_u, float2* bt_v) {
  const Spacing hs = make_spacing(h);
  dim3 blk(32, 8);
  dim3 grd((nx + 1 + blk.x - 1) / blk.x, (ny + 1 + blk.y - 1) / blk.y);
  if (mac) {
    // the correction reuses the forward pass's backtrace positions when
    // there is room for them (bt_u, bt_v; identical to recomputing them)
    k_advect_velocity<0><<<grd, blk, 0, s>>>(nx, ny, hs, u_in, v_in, nullptr, nullptr, u_hat, v_hat, label, sc, bt_u,
                                             bt_v);
    k_advect_velocity<1><<<grd, blk, 0, s>>>(nx, ny, hs, u_in, v_in, u_hat, v_hat, u_out, v_out, label, sc, bt_u,
                                             bt_v);
  } else {
    k_advect_velocity<0><<<grd, blk, 0, s>>>(nx, ny, hs, u_in, v_in, nullptr, nullptr, u_out, v_out, label, sc,
                                             nullptr, nullptr);
  }
}

cudaError_t preload_advect_kernels() {
  cudaFuncAttributes a;
  cudaError_t err = cudaFuncGetAttributes(&a, k_advect_velocity<0>);
  if (err == cudaSuccess) err = cudaFuncGetAttributes(&a, k_advect_velocity<1>);
  return err;
}

void launch_advect_dye(cudaStream_t s, int nx, int ny, float h, int dnx, int dny, float dh, int mac, const float* u,
                       const float* v, const float* q_in, float* q_hat, float* q_out, const uint8_t* label,
                       const StepScalars* sc, bool tail, const float* patch, int pi0, int pj0, int pnx, int pny,
                       float2* bt) {
  const Spacing hs = make_spacing(h), ds = make_spacing(dh);
  dim3 blk(32, 8);
  dim3 grd((dnx + blk.x - 1) / blk.x, (dny + blk.y - 1) / blk.y);
  if (mac) {
    k_advect_dye<0, false><<<grd, blk, 0, s>>>(nx, ny, hs, dnx, dny, ds, u, v, q_in, nullptr, q_hat, label, sc, nullptr,
                                               0, 0, 0, 0, bt);
    if (tail)
      k_advect_dye<1, true><<<grd, blk, 0, s>>>(nx, ny, hs, dnx, dny, ds, u, v, q_in, q_hat, q_out, label, sc, patch,
                                                pi0, pj0, pnx, pny, bt);
    else
      k_advect_dye<1, false><<<grd, blk, 0, s>>>(nx, ny, hs, dnx, dny, ds, u, v, q_in, q_hat, q_out, label, sc,
                                                 nullptr, 0, 0, 0, 0, bt);
  } else {
    if (tail)
      k_advect_dye<0, true><<<grd, blk, 0, s>>>(nx, ny, hs, dnx, dny, ds, u, v, q_in, nullptr, q_out, label, sc, patch,
                                                pi0, pj0, pnx, pny, nullptr);
    else
      k_advect_dye<0, false><<<grd, blk, 0, s>>>(nx, ny, hs, dnx, dny, ds, u, v, q_in, nullptr, q_out, label, sc,
                                                 nullptr, 0, 0, 0, 0, nullptr);
  }
}

}  // namespace fl
