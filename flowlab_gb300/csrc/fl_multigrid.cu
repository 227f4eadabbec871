// Red-black SOR and the geometric-multigrid V-cycle (src/core/
// pressureRedBlack.ts:32-113, pressureMultigrid.ts:47-320; WGSL twins
// src/gpu/redBlack.wgsl and src/gpu/multigrid.wgsl).
//
// GB300 shape of the V-cycle:
//   * Fine levels: ONE launch per level on the way down and one on the way up.
//     Each CTA loads its tile plus a halo into shared memory and runs all of
//     the level's red-black half-sweeps there (temporal blocking: half-sweep s
//     is valid on the region shrunk by s+1 cells, so a halo of 2*pairs+1
//     leaves the tile and a one-cell ring valid after the last sweep). The
//     down kernel then forms the residual and restricts it to the coarse rhs;
//     the up kernel first adds the prolonged coarse correction. Every cell
//     sees exactly the operations, in exactly the order, of the reference's
//     sequence of separate passes, so the result is identical to it.
//     x is double-buffered per level: a tile reads its halo's pre-sweep values
//     while neighbouring tiles write.
//   * Coarse levels (from the first level with <= coarse_cells cells): ONE
//     single-CTA launch runs the rest of the V-cycle entirely in shared
//     memory, including the coarsest-level sweeps.
//   * Labels become one byte per cell of stencil links (fl_common.cuh), built
//     per level when labels change (pressureMultigrid.ts:302-310 rebuilt them
//     every solve; stepGpu.ts:498 only on change, as here).
#include <algorithm>
#include <cstdio>

#include "fl_internal.h"

namespace fl {

constexpr int MODE_PLAIN = 0, MODE_PRE = 1, MODE_POST = 2;
constexpr int MAX_LEVELS = 24;
constexpr int SMOOTH_THREADS_X = 32, SMOOTH_THREADS_Y = 8;

// ------------------------------------------------------------ label codes

__global__ void k_build_codes(int nx, int ny, const uint8_t* __restrict__ label, uint8_t* __restrict__ code) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const long k = i + (long)j * nx;
  uint8_t c = label[k] & 3u;
  if (i + 1 < nx && label[k + 1] != SOLID) c |= LINK_XP;
  if (i > 0 && label[k - 1] != SOLID) c |= LINK_XM;
  if (j + 1 < ny && label[k + nx] != SOLID) c |= LINK_YP;
  if (j > 0 && label[k - nx] != SOLID) c |= LINK_YM;
  code[k] = c;
}

// pressureMultigrid.ts:92-110 (multigrid.wgsl:259-286): Air > Fluid > Solid.
__global__ void k_coarsen_labels(int fnx, int fny, const uint8_t* __restrict__ fine, int cnx, int cny,
                                 uint8_t* __restrict__ coarse) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  if (I >= cnx || J >= cny) return;
  bool air = false, fluid = false;
  for (int dj = 0; dj < 2; dj++)
    for (int di = 0; di < 2; di++) {
      const int i = 2 * I + di, j = 2 * J + dj;
      if (i >= fnx || j >= fny) continue;
      const uint8_t l = fine[i + (long)j * fnx];
      air = air || l == AIR;
      fluid = fluid || l == FLUID;
    }
  coarse[I + (long)J * cnx] = air ? AIR : (fluid ? FLUID : SOLID);
}

// The red-black update of one cell from shared memory (pressureRedBlack.ts:
// 52-66 with sum order +x, -x, +y, -y).
__device__ __forceinline__ void rb_update(float* xs, const float* bs, uint8_t c, int s, int sw, float scale,
                                          float omega) {
  if ((c & 3u) != FLUID) return;
  const int cnt = code_count(c);
  if (cnt == 0) return;
  float sum = 0.0f;
  if (c & LINK_XP) sum += xs[s + 1];
  if (c & LINK_XM) sum += xs[s - 1];
  if (c & LINK_YP) sum += xs[s + sw];
  if (c & LINK_YM) sum += xs[s - sw];
  const float pgs = (sum - scale * bs[s]) / (float)cnt;
  xs[s] = (1.0f - omega) * xs[s] + omega * pgs;
}

// r = b - (count*x - sum), 0 off-fluid (pressureMultigrid.ts:117-151).
__device__ __forceinline__ float residual_at(const float* xs, const float* bs, uint8_t c, int s, int sw, bool& counted) {
  counted = false;
  if ((c & 3u) != FLUID) return 0.0f;
  const int cnt = code_count(c);
  if (cnt == 0) return 0.0f;
  float sum = 0.0f;
  if (c & LINK_XP) sum += xs[s + 1];
  if (c & LINK_XM) sum += xs[s - 1];
  if (c & LINK_YP) sum += xs[s + sw];
  if (c & LINK_YM) sum += xs[s - sw];
  counted = true;
  return bs[s] - ((float)cnt * xs[s] - sum);
}

struct SmoothArgs {
  int nx, ny;
  const float* xin;
  float* xout;
  const float* b;
  const uint8_t* code;
  float scale, omega;
  float* bc;  // PRE: coarse rhs target
  int cnx, cny;
  const float* ec;  // POST: coarse correction
  StepAccum* acc;   // POST: residual norm accumulation (may be null)
  int x_is_zero;    // PRE on a coarse level: x starts at zero (pressureMultigrid.ts:175)
};

template <int TW, int TH, int P, int MODE>
struct SmoothGeom {
  static constexpr int H = (MODE == MODE_PLAIN) ? 2 * P : 2 * P + 1;
  static constexpr int SW = TW + 2 * H, SH = TH + 2 * H;
  // Coarse footprint of the region for prolongation: indices (GX>>1)-1 ..
  // ((GX+SW-1)>>1)+1 with GX = X0-H and X0 even, i.e. TW/2 + H + 3 values.
  static constexpr int CW = TW / 2 + H + 3, CH = TH / 2 + H + 3;
  static constexpr size_t bytes() {
    return sizeof(float) * (2 * SW * SH + (MODE == MODE_POST ? CW * CH : 0)) + ((SW * SH + 15) / 16) * 16;
  }
};

template <int TW, int TH, int P, int MODE>
__global__ void __launch_bounds__(SMOOTH_THREADS_X* SMOOTH_THREADS_Y) k_smooth(SmoothArgs a) {
  using G = SmoothGeom<TW, TH, P, MODE>;
  constexpr int H = G::H, SW = G::SW, SH = G::SH, CW = G::CW, CH = G::CH;
  extern __shared__ __align__(16) unsigned char smem[];
  float* xs = reinterpret_cast<float*>(smem);
  float* bs = xs + SW * SH;
  float* es = bs + SW * SH;
  uint8_t* cs = reinterpret_cast<uint8_t*>(es + (MODE == MODE_POST ? CW * CH : 0));
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int X0 = blockIdx.x * TW, Y0 = blockIdx.y * TH;
  const int GX = X0 - H, GY = Y0 - H;
  const int nx = a.nx, ny = a.ny;

  for (int lj = ty; lj < SH; lj += SMOOTH_THREADS_Y) {
    const int gj = GY + lj;
    for (int li = tx; li < SW; li += SMOOTH_THREADS_X) {
      const int gi = GX + li;
      const int s = li + lj * SW;
      if (gi >= 0 && gj >= 0 && gi < nx && gj < ny) {
        const long k = gi + (long)gj * nx;
        xs[s] = a.x_is_zero ? 0.0f : a.xin[k];
        bs[s] = a.b[k];
        cs[s] = a.code[k];
      } else {
        xs[s] = 0.0f;
        bs[s] = 0.0f;
        cs[s] = CODE_OUTSIDE;
      }
    }
  }

  if (MODE == MODE_POST) {
    // pressureMultigrid.ts:192-207 — x += 9/16, 3/16, 3/16, 1/16 of e.
    const int cI0 = (GX >> 1) - 1, cJ0 = (GY >> 1) - 1;
    for (int cj = ty; cj < CH; cj += SMOOTH_THREADS_Y)
      for (int ci = tx; ci < CW; ci += SMOOTH_THREADS_X) {
        const int I = cI0 + ci, J = cJ0 + cj;
        es[ci + cj * CW] = (I >= 0 && J >= 0 && I < a.cnx && J < a.cny) ? a.ec[I + (long)J * a.cnx] : 0.0f;
      }
    __syncthreads();
    for (int lj = ty; lj < SH; lj += SMOOTH_THREADS_Y) {
      const int gj = GY + lj;
      if (gj < 0 || gj >= ny) continue;
      const int J = gj >> 1;
      const int J2 = (gj & 1) ? min(J + 1, a.cny - 1) : max(J - 1, 0);
      for (int li = tx; li < SW; li += SMOOTH_THREADS_X) {
        const int gi = GX + li;
        if (gi < 0 || gi >= nx) continue;
        const int s = li + lj * SW;
        if ((cs[s] & 3u) != FLUID) continue;
        const int I = gi >> 1;
        const int I2 = (gi & 1) ? min(I + 1, a.cnx - 1) : max(I - 1, 0);
        const float e00 = es[(I - cI0) + (J - cJ0) * CW];
        const float e20 = es[(I2 - cI0) + (J - cJ0) * CW];
        const float e02 = es[(I - cI0) + (J2 - cJ0) * CW];
        const float e22 = es[(I2 - cI0) + (J2 - cJ0) * CW];
        xs[s] += 0.5625f * e00 + 0.1875f * (e20 + e02) + 0.0625f * e22;
      }
    }
  }
  __syncthreads();

#pragma unroll 1
  for (int hs = 0; hs < 2 * P; hs++) {
    const int color = hs & 1;
    const int sh = hs + 1;
    for (int lj = sh + ty; lj < SH - sh; lj += SMOOTH_THREADS_Y) {
      const int gj = GY + lj;
      const int first = sh + ((GX + sh + gj + color) & 1);
      for (int li = first + 2 * tx; li < SW - sh; li += 2 * SMOOTH_THREADS_X) {
        const int s = li + lj * SW;
        rb_update(xs, bs, cs[s], s, SW, a.scale, a.omega);
      }
    }
    __syncthreads();
  }

  if (MODE == MODE_PRE || (MODE == MODE_POST && a.acc != nullptr)) {
    double rsq = 0.0;
    unsigned long long rn = 0;
    for (int lj = H + ty; lj < H + TH; lj += SMOOTH_THREADS_Y)
      for (int li = H + tx; li < H + TW; li += SMOOTH_THREADS_X) {
        const int s = li + lj * SW;
        bool counted;
        const float r = residual_at(xs, bs, cs[s], s, SW, counted);
        if (MODE == MODE_PRE) {
          // Each cell's b is read by that cell alone, so the residual can
          // replace it in place for the restriction below.
          bs[s] = r;
        } else if (counted) {
          rsq += (double)r * (double)r;
          rn += 1;
        }
      }
    if (MODE == MODE_PRE) {
      __syncthreads();
      // pressureMultigrid.ts:156-178: coarse b = sum of the (up to) four
      // children's residuals. Tiles are even-aligned, so every child of this
      // tile's coarse cells is one of its own cells.
      for (int cj = ty; cj < TH / 2; cj += SMOOTH_THREADS_Y)
        for (int ci = tx; ci < TW / 2; ci += SMOOTH_THREADS_X) {
          const int I = (X0 >> 1) + ci, J = (Y0 >> 1) + cj;
          if (I >= a.cnx || J >= a.cny) continue;
          float sum = 0.0f;
          for (int dj = 0; dj < 2; dj++)
            for (int di = 0; di < 2; di++) {
              const int i = 2 * I + di, j = 2 * J + dj;
              if (i < nx && j < ny) sum += bs[(i - GX) + (j - GY) * SW];
            }
          a.bc[I + (long)J * a.cnx] = sum;
        }
    } else {
      __shared__ double red[32];
      __shared__ unsigned long long redn[32];
      const double bsum = block_sum(rsq, red);
      const unsigned long long bn = block_sum_u64(rn, redn);
      if (tx == 0 && ty == 0) {
        atomicAdd(&a.acc->res_sq, bsum);
        atomicAdd(&a.acc->n_res, bn);
      }
    }
  }

  for (int lj = H + ty; lj < H + TH; lj += SMOOTH_THREADS_Y) {
    const int gj = GY + lj;
    if (gj >= ny) break;
    for (int li = H + tx; li < H + TW; li += SMOOTH_THREADS_X) {
      const int gi = GX + li;
      if (gi < nx) a.xout[gi + (long)gj * nx] = xs[li + lj * SW];
    }
  }
}

// ----------------------------------------------------- single-CTA coarse tail

struct CoarseLevel {
  int nx, ny;
  const uint8_t* code;
  int off_x, off_b, off_c;  // shared-memory offsets: floats, floats, bytes
};

struct CoarseArgs {
  int nlev;
  CoarseLevel lv[MAX_LEVELS];
  const float* b_top;
  float* x_top;
  int x_is_zero;
  int pre, post, coarse_sweeps;
  float omega;
  StepAccum* acc;
  int code_bytes_off;  // byte offset of the code region
};

constexpr int COARSE_THREADS = 1024;
constexpr int SMALL_LEVEL = 512;  // levels at or below this many cells run on one warp

__device__ void coarse_smooth(float* x, const float* b, const uint8_t* c, int nx, int ny, int pairs, float omega) {
  const int n = nx * ny;
  const int tid = threadIdx.x;
  if (n <= SMALL_LEVEL) {
    if (tid < 32) {
      for (int hs = 0; hs < 2 * pairs; hs++) {
        const int color = hs & 1;
        for (int k = tid; k < n; k += 32) {
          const int j = k / nx, i = k - j * nx;
          if (((i + j) & 1) != color) continue;
          rb_update(x, b, c[k], k, nx, -1.0f, omega);
        }
        __syncwarp();
      }
    }
    __syncthreads();
  } else {
    for (int hs = 0; hs < 2 * pairs; hs++) {
      const int color = hs & 1;
      for (int k = tid; k < n; k += COARSE_THREADS) {
        const int j = k / nx, i = k - j * nx;
        if (((i + j) & 1) != color) continue;
        rb_update(x, b, c[k], k, nx, -1.0f, omega);
      }
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(COARSE_THREADS) k_mg_coarse(CoarseArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* fs = reinterpret_cast<float*>(smem);
  const int tid = threadIdx.x;
  for (int l = 0; l < a.nlev; l++) {
    const CoarseLevel& L = a.lv[l];
    const int n = L.nx * L.ny;
    uint8_t* c = smem + L.off_c;
    for (int k = tid; k < n; k += COARSE_THREADS) c[k] = L.code[k];
  }
  {
    const CoarseLevel& L = a.lv[0];
    const int n = L.nx * L.ny;
    for (int k = tid; k < n; k += COARSE_THREADS) {
      fs[L.off_b + k] = a.b_top[k];
      fs[L.off_x + k] = a.x_is_zero ? 0.0f : a.x_top[k];
    }
  }
  __syncthreads();

  // down: pre-smooth, residual + restriction (x_coarse = 0)
  for (int l = 0; l < a.nlev - 1; l++) {
    const CoarseLevel& L = a.lv[l];
    const CoarseLevel& C = a.lv[l + 1];
    float* x = fs + L.off_x;
    float* b = fs + L.off_b;
    const uint8_t* c = smem + L.off_c;
    coarse_smooth(x, b, c, L.nx, L.ny, a.pre, a.omega);
    const int cn = C.nx * C.ny;
    for (int K = tid; K < cn; K += COARSE_THREADS) {
      const int J = K / C.nx, I = K - J * C.nx;
      float sum = 0.0f;
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
          const int i = 2 * I + di, j = 2 * J + dj;
          if (i < L.nx && j < L.ny) {
            bool counted;
            const int s = i + j * L.nx;
            sum += residual_at(x, b, c[s], s, L.nx, counted);
          }
        }
      fs[C.off_b + K] = sum;
      fs[C.off_x + K] = 0.0f;
    }
    __syncthreads();
  }
  {
    const CoarseLevel& L = a.lv[a.nlev - 1];
    coarse_smooth(fs + L.off_x, fs + L.off_b, smem + L.off_c, L.nx, L.ny, a.coarse_sweeps, a.omega);
  }
  // up: prolong + post-smooth
  for (int l = a.nlev - 2; l >= 0; l--) {
    const CoarseLevel& L = a.lv[l];
    const CoarseLevel& C = a.lv[l + 1];
    float* x = fs + L.off_x;
    const float* e = fs + C.off_x;
    const uint8_t* c = smem + L.off_c;
    const int n = L.nx * L.ny;
    for (int k = tid; k < n; k += COARSE_THREADS) {
      if ((c[k] & 3u) != FLUID) continue;
      const int j = k / L.nx, i = k - j * L.nx;
      const int J = j >> 1, I = i >> 1;
      const int J2 = (j & 1) ? min(J + 1, C.ny - 1) : max(J - 1, 0);
      const int I2 = (i & 1) ? min(I + 1, C.nx - 1) : max(I - 1, 0);
      x[k] += 0.5625f * e[I + J * C.nx] + 0.1875f * (e[I2 + J * C.nx] + e[I + J2 * C.nx]) + 0.0625f * e[I2 + J2 * C.nx];
    }
    __syncthreads();
    coarse_smooth(x, fs + L.off_b, c, L.nx, L.ny, a.post, a.omega);
  }

  const CoarseLevel& T = a.lv[0];
  const int n = T.nx * T.ny;
  if (a.acc != nullptr) {
    double rsq = 0.0;
    unsigned long long rn = 0;
    for (int k = tid; k < n; k += COARSE_THREADS) {
      bool counted;
      const float r = residual_at(fs + T.off_x, fs + T.off_b, smem[T.off_c + k], k, T.nx, counted);
      if (counted) {
        rsq += (double)r * (double)r;
        rn += 1;
      }
    }
    __shared__ double red[32];
    __shared__ unsigned long long redn[32];
    const double bsum = block_sum(rsq, red);
    const unsigned long long bn = block_sum_u64(rn, redn);
    if (tid == 0) {
      atomicAdd(&a.acc->res_sq, bsum);
      atomicAdd(&a.acc->n_res, bn);
    }
  }
  for (int k = tid; k < n; k += COARSE_THREADS) a.x_top[k] = fs[T.off_x + k];
}

// Float64 defect correction (oracle: solveMixed). p_out = p_in + e (e may be
// null: no update), then r = b - A p_out in double with the neighbour sum in
// the order +x, -x, +y, -y; r is stored as float (the next V-cycle's rhs) and
// its square summed over fluid cells with links. Each thread also forms its
// four neighbours' updated values (the same additions their own threads
// make), so the kernel needs no halo exchange; p_out must not alias p_in.
__global__ void __launch_bounds__(256) k_update_resid64(int nx, int ny, const double* __restrict__ p_in,
                                                        const float* __restrict__ e, const float* __restrict__ b,
                                                        const uint8_t* __restrict__ code, double* __restrict__ p_out,
                                                        float* __restrict__ r32, StepAccum* acc) {
  __shared__ double red[32];
  __shared__ unsigned long long redn[32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  double sq = 0.0;
  unsigned long long n = 0;
  if (i < nx && j < ny) {
    const long k = i + (long)j * nx;
    auto P = [&](long q) { return e ? p_in[q] + (double)e[q] : p_in[q]; };
    const double pk = P(k);
    if (p_out) p_out[k] = pk;
    const uint8_t c = code[k];
    float r = 0.0f;
    if ((c & 3u) == FLUID) {
      const int cnt = code_count(c);
      if (cnt > 0) {
        double sum = 0.0;
        if (c & LINK_XP) sum += P(k + 1);
        if (c & LINK_XM) sum += P(k - 1);
        if (c & LINK_YP) sum += P(k + nx);
        if (c & LINK_YM) sum += P(k - nx);
        const double rd = (double)b[k] - ((double)cnt * pk - sum);
        r = (float)rd;
        sq = rd * rd;
        n = 1;
      }
    }
    r32[k] = r;
  }
  const double bs = block_sum(sq, red);
  const unsigned long long bn = block_sum_u64(n, redn);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    atomicAdd(&acc->res_sq, bs);
    atomicAdd(&acc->n_res, bn);
  }
}

// Remaining divergence of the red-black solver's stopping test (pressure.ts:
// 127-167): neighbour sum in the lexicographic order +x, +y, -x, -y, the
// residual formed in double.
__global__ void __launch_bounds__(256) k_rms_remaining(int nx, int ny, const float* __restrict__ p,
                                                       const float* __restrict__ div,
                                                       const uint8_t* __restrict__ code, float scale,
                                                       StepAccum* acc) {
  __shared__ double red[32];
  __shared__ unsigned long long redn[32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  double sq = 0.0;
  unsigned long long n = 0;
  if (i < nx && j < ny) {
    const long k = i + (long)j * nx;
    const uint8_t c = code[k];
    if ((c & 3u) == FLUID && code_count(c) > 0) {
      float sum = 0.0f;
      if (c & LINK_XP) sum += p[k + 1];
      if (c & LINK_YP) sum += p[k + nx];
      if (c & LINK_XM) sum += p[k - 1];
      if (c & LINK_YM) sum += p[k - nx];
      const double r =
          (double)div[k] + ((double)(float)code_count(c) * (double)p[k] - (double)sum) / (double)scale;
      sq = r * r;
      n = 1;
    }
  }
  const double bs = block_sum(sq, red);
  const unsigned long long bn = block_sum_u64(n, redn);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    atomicAdd(&acc->res_sq, bs);
    atomicAdd(&acc->n_res, bn);
  }
}

// One plain red-black half-sweep (redBlack.wgsl:67-115), for the per-pass
// entry point.
__global__ void k_rb_halfsweep(int nx, int ny, float* __restrict__ p, const float* __restrict__ b,
                               const uint8_t* __restrict__ code, float scale, float omega, int color) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny || ((i + j) & 1) != color) return;
  const long k = i + (long)j * nx;
  const uint8_t c = code[k];
  if ((c & 3u) != FLUID) return;
  const int cnt = code_count(c);
  if (cnt == 0) return;
  float sum = 0.0f;
  if (c & LINK_XP) sum += p[k + 1];
  if (c & LINK_XM) sum += p[k - 1];
  if (c & LINK_YP) sum += p[k + nx];
  if (c & LINK_YM) sum += p[k - nx];
  const float pgs = (sum - scale * b[k]) / (float)cnt;
  p[k] = (1.0f - omega) * p[k] + omega * pgs;
}

// ------------------------------------------------------------- host side

template <int TW, int TH, int P, int MODE>
static void launch_smooth_t(cudaStream_t s, const SmoothArgs& a) {
  using G = SmoothGeom<TW, TH, P, MODE>;
  static bool configured = false;  // per-instantiation attribute, set once per process
  const size_t bytes = G::bytes();
  if (!configured) {
    cudaFuncSetAttribute(k_smooth<TW, TH, P, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    configured = true;
  }
  dim3 blk(SMOOTH_THREADS_X, SMOOTH_THREADS_Y);
  dim3 grd((a.nx + TW - 1) / TW, (a.ny + TH - 1) / TH);
  k_smooth<TW, TH, P, MODE><<<grd, blk, bytes, s>>>(a);
}

template <int TW, int TH, int MODE>
static bool launch_smooth_p(cudaStream_t s, const SmoothArgs& a, int pairs) {
  switch (pairs) {
    case 0: if (MODE != MODE_PLAIN) { launch_smooth_t<TW, TH, 0, MODE>(s, a); return true; } return false;
    case 1: launch_smooth_t<TW, TH, 1, MODE>(s, a); return true;
    case 2: launch_smooth_t<TW, TH, 2, MODE>(s, a); return true;
    case 3: launch_smooth_t<TW, TH, 3, MODE>(s, a); return true;
    case 4: launch_smooth_t<TW, TH, 4, MODE>(s, a); return true;
    default: return false;
  }
}

// Tile choice: large tiles where there are enough of them to fill 152 SMs,
// smaller ones on coarser levels.
static bool launch_smooth(cudaStream_t s, const SmoothArgs& a, int pairs, int mode) {
  const bool big = (long)a.nx * a.ny >= 512L * 1024L;
  if (big) {
    if (mode == MODE_PLAIN) return launch_smooth_p<64, 32, MODE_PLAIN>(s, a, pairs);
    if (mode == MODE_PRE) return launch_smooth_p<64, 32, MODE_PRE>(s, a, pairs);
    return launch_smooth_p<64, 32, MODE_POST>(s, a, pairs);
  }
  if (mode == MODE_PLAIN) return launch_smooth_p<32, 16, MODE_PLAIN>(s, a, pairs);
  if (mode == MODE_PRE) return launch_smooth_p<32, 16, MODE_PRE>(s, a, pairs);
  return launch_smooth_p<32, 16, MODE_POST>(s, a, pairs);
}

void launch_build_codes(cudaStream_t s, int nx, int ny, const uint8_t* label, uint8_t* code) {
  dim3 b(32, 8), g((nx + 31) / 32, (ny + 7) / 8);
  k_build_codes<<<g, b, 0, s>>>(nx, ny, label, code);
}

void launch_rb_halfsweep(cudaStream_t s, int nx, int ny, float* p, const float* b, const uint8_t* code,
                         float scale, float omega, int color) {
  dim3 bl(32, 8), g((nx + 31) / 32, (ny + 7) / 8);
  k_rb_halfsweep<<<g, bl, 0, s>>>(nx, ny, p, b, code, scale, omega, color);
}

void launch_rb_sweeps(cudaStream_t s, int nx, int ny, const float* x_in, float* x_out, const float* b,
                      const uint8_t* code, float scale, float omega, int pairs) {
  SmoothArgs a{};
  a.nx = nx;
  a.ny = ny;
  a.xin = x_in;
  a.xout = x_out;
  a.b = b;
  a.code = code;
  a.scale = scale;
  a.omega = omega;
  launch_smooth(s, a, pairs, MODE_PLAIN);
}

void launch_update_resid64(cudaStream_t s, int nx, int ny, const double* p_in, const float* e, const float* b,
                           const uint8_t* code, double* p_out, float* r32, StepAccum* acc) {
  dim3 bl(32, 8), g((nx + 31) / 32, (ny + 7) / 8);
  k_update_resid64<<<g, bl, 0, s>>>(nx, ny, p_in, e, b, code, p_out, r32, acc);
}

void launch_rms_remaining(cudaStream_t s, int nx, int ny, const float* p, const float* div, const uint8_t* code,
                          float scale, StepAccum* acc) {
  dim3 b(32, 8), g((nx + 31) / 32, (ny + 7) / 8);
  k_rms_remaining<<<g, b, 0, s>>>(nx, ny, p, div, code, scale, acc);
}

// Levels that the single-CTA tail holds in shared memory: from the first
// level at or below this many cells.
static long coarse_cells_limit() { return 64L * 64L; }

static size_t coarse_smem_bytes(const Engine& e, int from, int* off_x, int* off_b, int* off_c) {
  size_t floats = 0;
  for (int l = from; l < (int)e.levels.size(); l++) {
    const long n = (long)e.levels[l].nx * e.levels[l].ny;
    if (off_x) off_x[l - from] = (int)floats;
    floats += n;
    if (off_b) off_b[l - from] = (int)floats;
    floats += n;
  }
  size_t bytes = floats * sizeof(float);
  for (int l = from; l < (int)e.levels.size(); l++) {
    const long n = (long)e.levels[l].nx * e.levels[l].ny;
    if (off_c) off_c[l - from] = (int)bytes;
    bytes += (size_t)((n + 15) / 16) * 16;
  }
  return bytes;
}

void mg_free(Engine& e) {
  for (auto& L : e.levels) {
    cudaFree(L.x[0]);
    cudaFree(L.x[1]);
    cudaFree(L.b);
    if (&L != &e.levels[0]) cudaFree(L.label);
    cudaFree(L.code);
  }
  e.levels.clear();
}

void mg_setup(Engine& e) {
  mg_free(e);
  // pressureMultigrid.ts:71-78
  std::vector<std::pair<int, int>> sizes{{e.nx, e.ny}};
  const int coarsest = std::max(1, e.prm.mg_coarsest);
  while (sizes.back().first > coarsest || sizes.back().second > coarsest)
    sizes.push_back({(sizes.back().first + 1) / 2, (sizes.back().second + 1) / 2});
  for (auto& sz : sizes) {
    Level L;
    L.nx = sz.first;
    L.ny = sz.second;
    e.levels.push_back(L);
  }
  for (size_t l = 0; l < e.levels.size(); l++) {
    Level& L = e.levels[l];
    const size_t n = (size_t)L.nx * L.ny;
    cudaMalloc(&L.x[0], n * sizeof(float));
    cudaMalloc(&L.x[1], n * sizeof(float));
    cudaMalloc(&L.b, n * sizeof(float));
    if (l > 0) cudaMalloc(&L.label, n);
    cudaMalloc(&L.code, n);
    cudaMemsetAsync(L.x[0], 0, n * sizeof(float), e.stream);
    cudaMemsetAsync(L.x[1], 0, n * sizeof(float), e.stream);
    cudaMemsetAsync(L.b, 0, n * sizeof(float), e.stream);
  }
  int lc = (int)e.levels.size() - 1;
  for (int l = 0; l < (int)e.levels.size(); l++)
    if ((long)e.levels[l].nx * e.levels[l].ny <= coarse_cells_limit()) {
      lc = l;
      break;
    }
  // The tiled kernels need even-aligned tiles on the level they restrict
  // from; any level works. Keep the tail within shared memory.
  while (coarse_smem_bytes(e, lc, nullptr, nullptr, nullptr) > 200 * 1024 && lc < (int)e.levels.size() - 1) lc++;
  e.coarse_level = lc;
  e.coarse_smem = coarse_smem_bytes(e, lc, nullptr, nullptr, nullptr);
  cudaFuncSetAttribute(k_mg_coarse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e.coarse_smem);
  e.codes_valid = false;
}

void mg_build_codes(Engine& e) {
  cudaStream_t s = e.stream;
  for (size_t l = 1; l < e.levels.size(); l++) {
    const Level& F = e.levels[l - 1];
    const Level& C = e.levels[l];
    dim3 b(32, 8), g((C.nx + 31) / 32, (C.ny + 7) / 8);
    k_coarsen_labels<<<g, b, 0, s>>>(F.nx, F.ny, F.label, C.nx, C.ny, C.label);
  }
  for (const Level& L : e.levels) launch_build_codes(s, L.nx, L.ny, L.label, L.code);
  e.codes_valid = true;
}

// One V-cycle (pressureMultigrid.ts:253-275) on levels[0].b with the warm
// start in levels[0].x[0]; the result lands back in levels[0].x[0]. When
// `acc` is set, the finest level's residual sum of squares is accumulated
// into it for the tolerance test.
void mg_vcycle(Engine& e, StepAccum* acc) { mg_vcycle_on(e, e.levels[0].b, false, acc); }

// One V-cycle with level 0's rhs `b0`; with `zero_start` the level-0 unknown
// starts from 0 (the correction equation of the defect-correction loop)
// instead of the warm start in levels[0].x[0].
void mg_vcycle_on(Engine& e, const float* b0, bool zero_start, StepAccum* acc) {
  cudaStream_t s = e.stream;
  const int lc = e.coarse_level;
  const float omega = (float)e.prm.mg_omega;
  auto cells = [&](int l) { return (double)e.levels[l].nx * e.levels[l].ny; };
  for (int l = 0; l < lc; l++) {
    Level& L = e.levels[l];
    Level& C = e.levels[l + 1];
    // x (level 0 only: coarser levels start from zero), b, code, x out, coarse b
    const int tok = prof_begin(e, FL_PH_MG_DOWN);
    SmoothArgs a{};
    a.nx = L.nx;
    a.ny = L.ny;
    a.xin = L.x[0];
    a.xout = L.x[1];
    a.b = l == 0 ? b0 : L.b;
    a.code = L.code;
    a.scale = -1.0f;
    a.omega = omega;
    a.bc = C.b;
    a.cnx = C.nx;
    a.cny = C.ny;
    a.x_is_zero = l > 0 || zero_start;
    launch_smooth(s, a, e.prm.mg_pre, MODE_PRE);
    prof_end(e, tok, (l == 0 ? 13.0 : 9.0) * cells(l) + 4.0 * cells(l + 1), 1);
  }
  {
    const int tok = prof_begin(e, FL_PH_MG_COARSE);
    double bytes = (lc == 0 ? 4.0 : 0.0) * cells(lc) + 8.0 * cells(lc);
    for (int l = lc; l < (int)e.levels.size(); l++) bytes += cells(l);
    CoarseArgs a{};
    int ox[MAX_LEVELS], ob[MAX_LEVELS], oc[MAX_LEVELS];
    coarse_smem_bytes(e, lc, ox, ob, oc);
    a.nlev = (int)e.levels.size() - lc;
    for (int l = 0; l < a.nlev; l++) {
      const Level& L = e.levels[lc + l];
      a.lv[l] = CoarseLevel{L.nx, L.ny, L.code, ox[l], ob[l], oc[l]};
    }
    a.b_top = lc == 0 ? b0 : e.levels[lc].b;
    a.x_top = e.levels[lc].x[0];
    a.x_is_zero = lc > 0 || zero_start;
    a.pre = e.prm.mg_pre;
    a.post = e.prm.mg_post;
    a.coarse_sweeps = e.prm.mg_coarse_sweeps;
    a.omega = omega;
    a.acc = lc == 0 ? acc : nullptr;
    k_mg_coarse<<<1, COARSE_THREADS, e.coarse_smem, s>>>(a);
    prof_end(e, tok, bytes, 1);
  }
  for (int l = lc - 1; l >= 0; l--) {
    Level& L = e.levels[l];
    Level& C = e.levels[l + 1];
    // x in, b, code, coarse e, x out
    const int tok = prof_begin(e, FL_PH_MG_UP);
    SmoothArgs a{};
    a.nx = L.nx;
    a.ny = L.ny;
    a.xin = L.x[1];
    a.xout = L.x[0];
    a.b = l == 0 ? b0 : L.b;
    a.code = L.code;
    a.scale = -1.0f;
    a.omega = omega;
    a.ec = C.x[0];
    a.cnx = C.nx;
    a.cny = C.ny;
    a.acc = l == 0 ? acc : nullptr;
    launch_smooth(s, a, e.prm.mg_post, MODE_POST);
    prof_end(e, tok, 13.0 * cells(l) + 4.0 * cells(l + 1), 1);
  }
}

}  // namespace fl
