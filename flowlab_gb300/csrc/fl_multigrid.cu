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
#include <mutex>
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include "fl_internal.h"

namespace fl {

constexpr int MODE_PLAIN = 0, MODE_PRE = 1, MODE_POST = 2;
constexpr int MAX_LEVELS = 24;

// ------------------------------------------------------------ label codes

// only_if (when set): the kernel does nothing unless *only_if is nonzero
__global__ void k_build_codes(int nx, int ny, const uint8_t* __restrict__ label, uint8_t* __restrict__ code,
                              const int* only_if) {
  if (only_if != nullptr && *only_if == 0) return;
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

// The uploaded labels against the current ones: copies the cells that
// differ and raises *flag if there were any (16 bytes per thread step; the
// buffers come from cudaMalloc, so the 16-byte body is aligned).
__global__ void __launch_bounds__(256) k_label_sync(const uint8_t* __restrict__ in, uint8_t* __restrict__ cur, long n,
                                                    int* flag) {
  bool changed = false;
  const long stride = (long)gridDim.x * blockDim.x;
  const long t0 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const uint4* in4 = reinterpret_cast<const uint4*>(in);
  uint4* cur4 = reinterpret_cast<uint4*>(cur);
  for (long k = t0; k < n / 16; k += stride) {
    const uint4 a = in4[k], b = cur4[k];
    if (a.x != b.x || a.y != b.y || a.z != b.z || a.w != b.w) {
      cur4[k] = a;
      changed = true;
    }
  }
  for (long k = 16 * (n / 16) + t0; k < n; k += stride)
    if (in[k] != cur[k]) {
      cur[k] = in[k];
      changed = true;
    }
  if (__syncthreads_or(changed) && threadIdx.x == 0) atomicOr(flag, 1);
}

__global__ void k_label_cond(int* flag, cudaGraphConditionalHandle h) {
  cudaGraphSetConditional(h, *flag != 0 ? 1u : 0u);
  *flag = 0;
}

void launch_label_sync(cudaStream_t s, const uint8_t* in, uint8_t* cur, long n, int* flag) {
  const long blocks = std::min(std::max(1L, (n / 16 + 255) / 256), 152L * 4);
  k_label_sync<<<(unsigned)blocks, 256, 0, s>>>(in, cur, n, flag);
}

void launch_label_cond(cudaStream_t s, int* flag, cudaGraphConditionalHandle h) { k_label_cond<<<1, 1, 0, s>>>(flag, h); }

// pressureMultigrid.ts:92-110 (multigrid.wgsl:259-286): Air > Fluid > Solid.
__global__ void k_coarsen_labels(int fnx, int fny, const uint8_t* __restrict__ fine, int cnx, int cny,
                                 uint8_t* __restrict__ coarse, const int* only_if) {
  if (only_if != nullptr && *only_if == 0) return;
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
  const float* scale_dev;  // PLAIN: when set, the scale is read here (the step's scalars)
  float* bc;  // PRE: coarse rhs target
  int cnx, cny;
  const float* ec;  // POST: coarse correction
  StepAccum* acc;   // POST: residual norm accumulation (may be null)
  int x_is_zero;    // PRE on a coarse level: x starts at zero (pressureMultigrid.ts:175)
};

// (sum - scale*b) / count with count in 1..4: a multiply by the exact
// reciprocal for 1, 2 and 4 (the same float as the division, since scaling by
// a power of two is exact) and a true division for 3.
//
// The division by 3 is the correctly rounded quotient formed with two FMAs
// (the correction step for a divisor known in advance: Markstein; Brisebarre,
// Muller and Raina, IEEE Trans. Computers 2004): q0 = RN(s * RN(1/3)),
// r = s - 3 q0 (exact), q = RN(q0 + r * RN(1/3)); zero and infinities take
// q0. It equals IEEE s / 3 for every float (checked exhaustively), at a
// fraction of the division's latency.
__device__ __forceinline__ float div3(float s) {
  const float y = 0x1.555556p-2f;  // RN(1/3)
  const float q0 = __fmul_rn(s, y);
  const float r = __fmaf_rn(-3.0f, q0, s);
  const float q1 = __fmaf_rn(r, y, q0);
  return (s == 0.0f || fabsf(s) == __int_as_float(0x7f800000)) ? q0 : q1;
}

__device__ __forceinline__ float over_count(float s, int cnt) {
  const float third = div3(s);
  return cnt == 3 ? third : s * (cnt == 4 ? 0.25f : (cnt == 2 ? 0.5f : 1.0f));
}

// Temporally blocked red-black smoother. One 1024-thread CTA owns a 64x64
// region: its tile plus a halo of H = 2*pairs (+1 when a residual follows).
// Thread (tx, ty) owns the cells (2tx, ty), (2tx+1, ty), (2tx, ty+32),
// (2tx+1, ty+32) — one of each colour per row — and keeps their stencil
// code, rhs and value in registers for the whole launch. Neighbour values go
// through shared memory split by local parity, xs[(li+lj)&1][lj][li>>1], so
// a warp's reads and writes are unit-stride. Every half-sweep updates every
// region cell of its colour except the region's outer ring: half-sweep s is
// correct on the region shrunk by s+1 cells, so after 2*pairs half-sweeps the
// tile (and, with the +1, a ring around it) holds exactly the values the
// sequential sweeps produce; outer cells hold finite values nobody uses.
// The region side R is 64 (1024 threads) on large levels and 32 (256
// threads, more CTAs for levels too small to fill the GPU with 64^2 regions).
template <int P, int MODE, int R>
struct Tile {
  static constexpr int H = (MODE == MODE_PLAIN) ? 2 * P : 2 * P + 1;
  static constexpr int T = R - 2 * H;  // tile side, even
};

// Loads of data an earlier phase of the same launch may have written (the
// persistent solve): through L2 only, so that no stale L1 line is read.
// Otherwise plain loads, and the read-only path for the coarse correction.
template <bool COH>
__device__ __forceinline__ float ld_coherent(const float* p) {
  if constexpr (COH) return __ldcg(p);
  return *p;
}
template <bool COH>
__device__ __forceinline__ float ld_ro(const float* p) {
  if constexpr (COH) return __ldcg(p);
  return __ldg(p);
}

// One region of the temporally blocked smoother, region (bx, by) of the
// level; called by one whole block (every thread, in step).
template <int P, int MODE, int R, bool COH>
__device__ __forceinline__ void smooth_tile(const SmoothArgs& a, int bx, int by) {
  constexpr int RGN = R;
  constexpr int RGN_T = R / 2;
  constexpr int H = Tile<P, MODE, R>::H;
  constexpr int T = Tile<P, MODE, R>::T;
  static_assert(T % 2 == 0 && T > 0, "tile must be even");
  __shared__ float xs[2][RGN][RGN / 2];
  __shared__ float rs[MODE == MODE_PRE ? RGN : 1][MODE == MODE_PRE ? RGN : 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int X0 = bx * T, Y0 = by * T;
  const int GX = X0 - H, GY = Y0 - H;
  const int nx = a.nx, ny = a.ny;

  uint8_t cd[2][2];
  float bb[2][2], xx[2][2];
#pragma unroll
  for (int r = 0; r < 2; r++) {
    const int lj = ty + RGN_T * r;
    const int gj = GY + lj;
#pragma unroll
    for (int o = 0; o < 2; o++) {
      const int li = 2 * tx + o;
      const int gi = GX + li;
      if ((unsigned)gi < (unsigned)nx && (unsigned)gj < (unsigned)ny) {
        // 32-bit offsets: a level holds fewer than 2^31 cells (the engine's
        // grid limits)
        const int k = gi + gj * nx;
        cd[r][o] = a.code[k];
        bb[r][o] = ld_coherent<COH>(a.b + k);
        xx[r][o] = a.x_is_zero ? 0.0f : ld_coherent<COH>(a.xin + k);
      } else {
        cd[r][o] = CODE_OUTSIDE;
        bb[r][o] = 0.0f;
        xx[r][o] = 0.0f;
      }
    }
    if constexpr (MODE == MODE_POST) {
      // pressureMultigrid.ts:192-207 — a fluid cell's x += 9/16, 3/16, 3/16,
      // 1/16 of e at coarse columns (I, I2) and rows (J, J2), I = i >> 1, I2
      // = I + 1 (odd i, clamped) or I - 1 (even i, clamped). The row's two
      // cells are the odd column GX + 2tx (H is odd, T even) and the even one
      // after it, so both read coarse columns A = max(I, 0) and B = min(I +
      // 1, cnx - 1) of I = (GX + 2tx - 1) / 2: the odd cell as (I, I2) =
      // (A, B), the even one as (B, A). Four loads serve the two cells.
      // The loads do not wait for the codes: on rows inside the grid they
      // run for every pair, at columns clamped into the coarse level (the
      // clamps change nothing for a pair with a cell in the grid).
      static_assert(H % 2 == 1, "the prolongation pairs an odd column with the even one after it");
      if ((unsigned)gj < (unsigned)ny) {
        const int I = (GX + 2 * tx - 1) / 2;
        const int A = min(max(I, 0), a.cnx - 1), B = max(min(I + 1, a.cnx - 1), 0);
        const int J = gj >> 1;
        const int J2 = (gj & 1) ? min(J + 1, a.cny - 1) : max(J - 1, 0);
        const float* e = a.ec;
        const int cs = a.cnx;
        const float eAJ = ld_ro<COH>(e + A + J * cs), eBJ = ld_ro<COH>(e + B + J * cs);
        const float eAJ2 = ld_ro<COH>(e + A + J2 * cs), eBJ2 = ld_ro<COH>(e + B + J2 * cs);
        if ((cd[r][0] & 3u) == FLUID) xx[r][0] += 0.5625f * eAJ + 0.1875f * (eBJ + eAJ2) + 0.0625f * eBJ2;
        if ((cd[r][1] & 3u) == FLUID) xx[r][1] += 0.5625f * eBJ + 0.1875f * (eAJ + eBJ2) + 0.0625f * eAJ2;
      }
    }
#pragma unroll
    for (int o = 0; o < 2; o++) {
      // Solid cells (and cells outside the grid) are exactly the neighbours
      // no link points to; they hold +0.0 in shared memory (their own value
      // stays in xx), so that a sweep can add all four neighbours without a
      // test: an unlinked one adds +0.0, which leaves the sum's bits
      // unchanged (a sum that starts at +0.0 never becomes -0.0).
      xs[(2 * tx + o + lj) & 1][lj][tx] = (cd[r][o] & 3u) == SOLID ? 0.0f : xx[r][o];
    }
  }
  __syncthreads();

  const float scale = a.scale_dev ? *a.scale_dev : a.scale, omega = a.omega, keep = 1.0f - omega;
  {
    // Colour view of the thread's cells: in row r the colour-c cell is
    // column 2tx + oc[c] (the same for both rows), kept in registers with
    // what its updates need precomputed once: whether it is updated at all
    // (fluid, linked, off the region's outer ring), scale*b, the exact
    // reciprocal of its link count (0 marks a count of 3: true division).
    const int g = (GX + GY) & 1;
    int oc[2];
    oc[0] = (g + ty) & 1;
    oc[1] = 1 - oc[0];
    bool act[2][2];
    float sb[2][2], rc[2][2], xc[2][2];
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int c = 0; c < 2; c++) {
        const int o = oc[c];
        const int lj = ty + RGN_T * r, li = 2 * tx + o;
        const uint8_t code = o ? cd[r][1] : cd[r][0];
        const int cnt = code_count(code);
        act[r][c] = li != 0 && li != RGN - 1 && lj != 0 && lj != RGN - 1 && (code & 3u) == FLUID && cnt > 0;
        sb[r][c] = scale * (o ? bb[r][1] : bb[r][0]);
        rc[r][c] = cnt == 4 ? 0.25f : (cnt == 2 ? 0.5f : (cnt == 1 ? 1.0f : 0.0f));
        xc[r][c] = o ? xx[r][1] : xx[r][0];
      }
    // With omega = 1 (the multigrid's relaxation) the blend (1 - omega) x +
    // omega pGS is pGS for every finite x, up to the sign of an exact zero
    // (0 x + (-0) is +0), which compares equal: the sweeps then skip it.
    auto sweeps = [&](auto unit) {
      constexpr bool UNIT = decltype(unit)::value;
#pragma unroll
      for (int hs = 0; hs < 2 * P; hs++) {
        const int c = hs & 1;
        const int q = c ^ g;  // local parity plane of colour c
        const float(*xo)[RGN / 2] = xs[1 - q];
#pragma unroll
        for (int r = 0; r < 2; r++) {
          if (!act[r][c]) continue;
          const int lj = ty + RGN_T * r;
          const int o = oc[c];
          float sum = 0.0f;
          sum += xo[lj][tx + o];
          sum += xo[lj][tx + o - 1];
          sum += xo[lj + 1][tx];
          sum += xo[lj - 1][tx];
          const float d = sum - sb[r][c];
          const float third = div3(d);
          const float pgs = rc[r][c] != 0.0f ? d * rc[r][c] : third;
          const float nv = UNIT ? pgs : keep * xc[r][c] + omega * pgs;
          xc[r][c] = nv;
          xs[q][lj][tx] = nv;
        }
        __syncthreads();
      }
    };
    if (omega == 1.0f)
      sweeps(std::true_type{});
    else
      sweeps(std::false_type{});
#pragma unroll
    for (int r = 0; r < 2; r++) {
      xx[r][0] = oc[0] == 0 ? xc[r][0] : xc[r][1];
      xx[r][1] = oc[0] == 0 ? xc[r][1] : xc[r][0];
    }
  }

  if (MODE == MODE_PRE || (MODE == MODE_POST && a.acc != nullptr)) {
    double rsq = 0.0;
    unsigned long long rn = 0;
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const int lj = ty + RGN_T * r;
#pragma unroll
      for (int o = 0; o < 2; o++) {
        const int li = 2 * tx + o;
        if ((unsigned)(li - H) >= (unsigned)T || (unsigned)(lj - H) >= (unsigned)T) continue;
        const uint8_t c = cd[r][o];
        float res = 0.0f;
        if ((c & 3u) == FLUID) {
          const int cnt = code_count(c);
          if (cnt > 0) {
            // r = b - (count*x - sum), sum order +x, -x, +y, -y (pressureMultigrid.ts:117-151);
            // every neighbour read, an unlinked one being +0.0 (as in the sweeps)
            const float(*xq)[RGN / 2] = xs[1 - ((li + lj) & 1)];
            float sum = 0.0f;
            sum += xq[lj][tx + o];
            sum += xq[lj][tx + o - 1];
            sum += xq[lj + 1][tx];
            sum += xq[lj - 1][tx];
            res = bb[r][o] - ((float)cnt * xx[r][o] - sum);
            rsq = fma(f2d_exact(res), f2d_exact(res), rsq);
            rn += 1;
          }
        }
        if (MODE == MODE_PRE) rs[lj][li] = res;
      }
    }
    if (MODE == MODE_PRE) {
      __syncthreads();
      // pressureMultigrid.ts:156-178: coarse b = sum of the children's
      // residuals; tiles start at even coordinates, so all children of the
      // tile's coarse cells are tile cells.
      const int t = tx + RGN_T * ty;
      if (t < (T / 2) * (T / 2)) {
        const int cj = t / (T / 2), ci = t - cj * (T / 2);
        const int I = (X0 >> 1) + ci, J = (Y0 >> 1) + cj;
        if (I < a.cnx && J < a.cny) {
          float sum = 0.0f;
          for (int dj = 0; dj < 2; dj++)
            for (int di = 0; di < 2; di++) {
              const int i = 2 * I + di, j = 2 * J + dj;
              if (i < nx && j < ny) sum += rs[j - GY][i - GX];
            }
          a.bc[I + J * a.cnx] = sum;
        }
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

  if (a.xout != nullptr) {
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const int lj = ty + RGN_T * r;
      const int gj = GY + lj;
      if (lj < H || lj >= H + T || gj >= ny) continue;
#pragma unroll
      for (int o = 0; o < 2; o++) {
        const int li = 2 * tx + o;
        const int gi = GX + li;
        if (li < H || li >= H + T || gi >= nx) continue;
        a.xout[gi + gj * nx] = xx[r][o];
      }
    }
  }
}

template <int P, int MODE, int R>
__global__ void __launch_bounds__(R* R / 4, R == 64 ? 1 : 4) k_smooth(SmoothArgs a) {
  smooth_tile<P, MODE, R, false>(a, blockIdx.x, blockIdx.y);
}

// ----------------------------------------------------- single-CTA coarse tail

// The coarsest levels (both sides <= fl_params.mg_tail_side, 32 by default,
// at most 64) run in ONE 1024-thread CTA, entirely in shared memory (a zero
// word first, then per level x split by parity, xs[(i+j)&1][j][i>>1] with a
// power-of-two row stride, b and the stencil codes row-major). The CTA is bound by how
// many instructions its warps issue, so each level is owned by as few warps
// as hold its cells: a row of colour-c cells gets LPR = 2^lsh lanes (the
// power of two >= ceil(nx/2)), a warp covers 32/LPR rows, and only the first
// `nwarps` warps (at most 32; a 64-row level gives each of them two row
// groups) take part in that level's phases, synchronising on the level's own
// named barrier. Coarser levels are owned by a subset of the finer level's
// warps, so the barrier that ends a phase on a level also orders it before
// every coarser-level phase.
struct CoarseLevel {
  int nx, ny;
  const uint8_t* code;
  int off_x, off_b, off_c;  // shared-memory offsets: floats, floats, bytes
  int lsh;                  // log2 of the lanes per row
  int nwarps;               // owner warps
  int slots;                // row groups per warp: 2 when the level has more than 32 groups
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
};

// Default first level of the single-CTA tail (fl_params.mg_tail_side = 0):
// levels with both sides <= 32. Measured on the 1024^2 plume: 1641 steps/s
// from 32, 1570 from 64, 1636 from 16, 1626 from 8 (below 32 the extra
// launches cost more than the tail's shorter barrier chain saves).
constexpr int TAIL_SIDE_DEFAULT = 32;

struct CoarseView {
  float* xs;  // 2 * ny * rs floats
  float* bs;
  const uint8_t* cs;
  int nx, ny, rs;
  __device__ float& x(int i, int j) const { return xs[((i + j) & 1) * ny * rs + j * rs + (i >> 1)]; }
};

__device__ __forceinline__ CoarseView coarse_view(unsigned char* smem, const CoarseLevel& L) {
  float* fs = reinterpret_cast<float*>(smem);
  CoarseView v;
  v.xs = fs + L.off_x;
  v.bs = fs + L.off_b;
  v.cs = smem + L.off_c;
  v.nx = L.nx;
  v.ny = L.ny;
  v.rs = 1 << L.lsh;
  return v;
}

// The cell of colour c in row group w + 32 s owned by `lane`.
__device__ __forceinline__ void tail_cell(const CoarseLevel& L, int w, int lane, int s, int c, int& i, int& j) {
  j = ((w + 32 * s) << (5 - L.lsh)) + (lane >> L.lsh);
  i = 2 * (lane & ((1 << L.lsh) - 1)) + ((c + j) & 1);
}

// Named barrier `l + 1` over the owner warps of tail level l (a warp
// barrier when one warp owns the level).
__device__ __forceinline__ void tail_bar(int l, int nwarps) {
  if (nwarps == 1) {
    __syncwarp();
    return;
  }
  asm volatile("bar.sync %0, %1;" ::"r"(l + 1), "r"(nwarps * 32) : "memory");
}

// r = b - (count*x - sum), 0 off-fluid (pressureMultigrid.ts:117-151).
// Branch-free for the same reason as tail_smooth: every neighbour is read
// (an unlinked one at the cell itself) and an unlinked one adds +0.0.
__device__ __forceinline__ float coarse_residual(const CoarseView& v, int i, int j, bool& counted) {
  const int k = i + j * v.nx;
  const uint8_t c = v.cs[k];
  const int cnt = code_count(c);
  counted = (c & 3u) == FLUID && cnt > 0;
  const int pl = v.ny * v.rs;
  const int own = ((i + j) & 1) * pl + j * v.rs + (i >> 1);
  const int oth = (1 - ((i + j) & 1)) * pl + j * v.rs;
  const float x0 = v.xs[own];
  const float vxp = v.xs[(c & LINK_XP) ? oth + ((i + 1) >> 1) : own];
  const float vxm = v.xs[(c & LINK_XM) ? oth + ((i - 1) >> 1) : own];
  const float vyp = v.xs[(c & LINK_YP) ? oth + v.rs + (i >> 1) : own];
  const float vym = v.xs[(c & LINK_YM) ? oth - v.rs + (i >> 1) : own];
  float sum = 0.0f;
  sum += (c & LINK_XP) ? vxp : 0.0f;
  sum += (c & LINK_XM) ? vxm : 0.0f;
  sum += (c & LINK_YP) ? vyp : 0.0f;
  sum += (c & LINK_YM) ? vym : 0.0f;
  const float r = v.bs[k] - ((float)cnt * x0 - sum);
  return counted ? r : 0.0f;
}

// `pairs` red-black sweep pairs on tail level l by its owner warps; ends
// with the level's barrier (also when pairs is 0). Each thread keeps its
// cells' rhs, value, link mask and the shared-memory addresses of their
// four neighbours in registers. The update has no branches: on these small
// levels most warps hold boundary cells, and a lane-divergent branch around
// each neighbour load serialised the warp (measured: a one-warp half-sweep
// took ~630 cycles that way, ~270 with unconditional loads). An unlinked
// neighbour is read at the zero word that starts shared memory and adds
// +0.0, which leaves the sum's bits unchanged: a running sum that starts at
// +0.0 never becomes -0.0.
__device__ __forceinline__ float lds_f32(uint32_t addr) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ void sts_f32(uint32_t addr, float v) {
  asm volatile("st.shared.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}

__device__ void tail_smooth(unsigned char* smem, const CoarseLevel& L, int l, int pairs, float omega, int w,
                            int lane) {
  if (w >= L.nwarps) return;
  float* xs = reinterpret_cast<float*>(smem) + L.off_x;
  const uint32_t sm_sh = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  const float* bs = reinterpret_cast<const float*>(smem) + L.off_b;
  const uint8_t* cs = smem + L.off_c;
  // row stride: the lanes per row (a power of two), so that the rows a warp
  // covers fall in distinct shared-memory banks
  const int rs = 1 << L.lsh;
  const int plane = L.ny * rs;
  bool upd[2][2];  // the cell is updated
  int own[2][2], nb[2][2][4];
  float bq[2][2], xq[2][2], rc[2][2];
#pragma unroll
  for (int s = 0; s < 2; s++)
#pragma unroll
    for (int c = 0; c < 2; c++) {
      int i, j;
      tail_cell(L, w, lane, s, c, i, j);
      const bool ok = i < L.nx && j < L.ny;
      const uint8_t code = ok ? cs[i + j * L.nx] : (uint8_t)CODE_OUTSIDE;
      const int cnt = code_count(code);
      const bool act = ok && (code & 3u) == FLUID && cnt > 0;
      // float indices from the start of shared memory; an unlinked
      // neighbour (and every neighbour of a cell outside the level) is the
      // zero word at index 0
      const int ow = L.off_x + (ok ? c * plane + j * rs + (i >> 1) : 0);
      const int o = L.off_x + (1 - c) * plane + j * rs + (i >> 1), d = i & 1;
      own[s][c] = ow;
      nb[s][c][0] = (ok && (code & LINK_XP)) ? o + d : 0;
      nb[s][c][1] = (ok && (code & LINK_XM)) ? o + d - 1 : 0;
      nb[s][c][2] = (ok && (code & LINK_YP)) ? o + rs : 0;
      nb[s][c][3] = (ok && (code & LINK_YM)) ? o - rs : 0;
      upd[s][c] = act;
      rc[s][c] = cnt == 4 ? 0.25f : (cnt == 2 ? 0.5f : (cnt == 1 ? 1.0f : 0.0f));
      bq[s][c] = ok ? bs[i + j * L.nx] : 0.0f;
      xq[s][c] = ok ? xs[ow - L.off_x] : 0.0f;
    }
  // shared-space byte addresses (explicit ld/st.shared)
#pragma unroll
  for (int s = 0; s < 2; s++)
#pragma unroll
    for (int c = 0; c < 2; c++) {
      own[s][c] = (int)(sm_sh + 4u * (uint32_t)own[s][c]);
#pragma unroll
      for (int k = 0; k < 4; k++) nb[s][c][k] = (int)(sm_sh + 4u * (uint32_t)nb[s][c][k]);
    }
  const bool two = L.slots == 2;
  const float keep = 1.0f - omega;
  // omega = 1: pGS itself (see smooth_tile)
  auto sweeps = [&](auto unit) {
    constexpr bool UNIT = decltype(unit)::value;
#pragma unroll 1
    for (int hs = 0; hs < 2 * pairs; hs += 2) {
#pragma unroll
      for (int c = 0; c < 2; c++) {
#pragma unroll
        for (int s = 0; s < 2; s++) {
          if (s == 1 && !two) continue;  // warp-uniform: the level has one row group per warp
          const float v0 = lds_f32((uint32_t)nb[s][c][0]), v1 = lds_f32((uint32_t)nb[s][c][1]);
          const float v2 = lds_f32((uint32_t)nb[s][c][2]), v3 = lds_f32((uint32_t)nb[s][c][3]);
          float sum = 0.0f;
          sum += v0;
          sum += v1;
          sum += v2;
          sum += v3;
          const float dv = sum - (-1.0f) * bq[s][c];
          const float third = div3(dv);
          const float pgs = rc[s][c] != 0.0f ? dv * rc[s][c] : third;
          const float nv = UNIT ? pgs : keep * xq[s][c] + omega * pgs;
          if (upd[s][c]) {
            xq[s][c] = nv;
            sts_f32((uint32_t)own[s][c], nv);
          }
        }
        tail_bar(l, L.nwarps);
      }
    }
  };
  if (omega == 1.0f)
    sweeps(std::true_type{});
  else
    sweeps(std::false_type{});
  if (pairs <= 0) tail_bar(l, L.nwarps);
}

// The whole tail, run by one 1024-thread block over `smem` (the layout of
// coarse_smem_bytes).
__device__ __forceinline__ void mg_coarse_body(const CoarseArgs& a, unsigned char* smem) {
  const int tid = threadIdx.x + 32 * threadIdx.y;
  const int lane = tid & 31, w = tid >> 5;
  if (tid == 0) reinterpret_cast<float*>(smem)[0] = 0.0f;  // the zero word tail_smooth's unlinked neighbours read
  for (int l = 0; l < a.nlev; l++) {
    const CoarseLevel& L = a.lv[l];
    const int n = L.nx * L.ny;
    uint8_t* c = smem + L.off_c;
    for (int k = tid; k < n; k += 1024) c[k] = L.code[k];
  }
  const CoarseLevel& TL = a.lv[0];
  const CoarseView T = coarse_view(smem, TL);
  if (w < TL.nwarps) {
#pragma unroll
    for (int s = 0; s < 2; s++)
#pragma unroll
      for (int c = 0; c < 2; c++) {
        int i, j;
        tail_cell(TL, w, lane, s, c, i, j);
        if (i < T.nx && j < T.ny) {
          const int k = i + j * T.nx;
          T.bs[k] = a.b_top[k];
          T.x(i, j) = a.x_is_zero ? 0.0f : a.x_top[k];
        }
      }
  }
  __syncthreads();

  // down: pre-smooth, then residual + restriction (by the coarse level's
  // owners) with the coarse x set to 0
  for (int l = 0; l < a.nlev - 1; l++) {
    const CoarseLevel& FL = a.lv[l];
    const CoarseLevel& CL = a.lv[l + 1];
    tail_smooth(smem, FL, l, a.pre, a.omega, w, lane);
    if (w >= CL.nwarps) continue;
    const CoarseView F = coarse_view(smem, FL);
    const CoarseView C = coarse_view(smem, CL);
#pragma unroll
    for (int s = 0; s < 2; s++)
#pragma unroll
      for (int c = 0; c < 2; c++) {
        int I, J;
        tail_cell(CL, w, lane, s, c, I, J);
        if (I >= C.nx || J >= C.ny) continue;
        float sum = 0.0f;
        for (int dj = 0; dj < 2; dj++)
          for (int di = 0; di < 2; di++) {
            const int i = 2 * I + di, j = 2 * J + dj;
            if (i < F.nx && j < F.ny) {
              bool counted;
              sum += coarse_residual(F, i, j, counted);
            }
          }
        C.bs[I + J * C.nx] = sum;
        C.x(I, J) = 0.0f;
      }
    tail_bar(l + 1, CL.nwarps);
  }
  tail_smooth(smem, a.lv[a.nlev - 1], a.nlev - 1, a.coarse_sweeps, a.omega, w, lane);
  // up: prolongation (9/16, 3/16, 3/16, 1/16), then post-smooth
  for (int l = a.nlev - 2; l >= 0; l--) {
    const CoarseLevel& FL = a.lv[l];
    if (w >= FL.nwarps) continue;
    tail_bar(l, FL.nwarps);  // the coarse level's owners are done with it
    const CoarseView F = coarse_view(smem, FL);
    const CoarseView C = coarse_view(smem, a.lv[l + 1]);
#pragma unroll
    for (int s = 0; s < 2; s++)
#pragma unroll
      for (int c = 0; c < 2; c++) {
        int i, j;
        tail_cell(FL, w, lane, s, c, i, j);
        if (i >= F.nx || j >= F.ny) continue;
        if ((F.cs[i + j * F.nx] & 3u) != FLUID) continue;
        const int I = i >> 1, J = j >> 1;
        const int I2 = (i & 1) ? min(I + 1, C.nx - 1) : max(I - 1, 0);
        const int J2 = (j & 1) ? min(J + 1, C.ny - 1) : max(J - 1, 0);
        F.x(i, j) += 0.5625f * C.x(I, J) + 0.1875f * (C.x(I2, J) + C.x(I, J2)) + 0.0625f * C.x(I2, J2);
      }
    tail_bar(l, FL.nwarps);
    tail_smooth(smem, FL, l, a.post, a.omega, w, lane);
  }

  double rsq = 0.0;
  unsigned long long rn = 0;
  if (w < TL.nwarps) {
#pragma unroll
    for (int s = 0; s < 2; s++)
#pragma unroll
      for (int c = 0; c < 2; c++) {
        int i, j;
        tail_cell(TL, w, lane, s, c, i, j);
        if (i >= T.nx || j >= T.ny) continue;
        if (a.acc != nullptr) {
          bool counted;
          const float res = coarse_residual(T, i, j, counted);
          if (counted) {
            rsq = fma(f2d_exact(res), f2d_exact(res), rsq);
            rn += 1;
          }
        }
        a.x_top[i + j * T.nx] = T.x(i, j);
      }
  }
  if (a.acc != nullptr) {
    __shared__ double red[32];
    __shared__ unsigned long long redn[32];
    const double bsum = block_sum(rsq, red);
    const unsigned long long bn = block_sum_u64(rn, redn);
    if (tid == 0) {
      atomicAdd(&a.acc->res_sq, bsum);
      atomicAdd(&a.acc->n_res, bn);
    }
  }
}

__global__ void __launch_bounds__(1024, 1) k_mg_coarse(CoarseArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  mg_coarse_body(a, smem);
}

// The float64 defect-correction pass (iterative refinement, solveMixed):
// p64' = p64 + e (when `update`), then r = b - (count*p64' - sum) in double
// with the neighbour sum in the order +x, -x, +y, -y, r32 = float(r), and
// the squared norm of r accumulated. GB300 issues float64 arithmetic at about
// 1.6 lanes per clock per SM (measured; 32-bit integer adds: ~100), so this
// pass is bound by its float64 instructions, not by memory, and spends them
// only where the result needs them: each p64' is formed once and handed to
// its neighbours in registers (the rows above and below) and by warp
// shuffles (left and right); the exact float -> double widenings, the first
// addition to 0.0, the products by 2 and 4 and the rounding of r to float
// run on the integer pipe with identical results (fl_common.cuh), with their
// rare cases out of line and their bit casts opaque, so that the compiler
// neither predicates nor re-forms float64 instructions into every cell.
// A warp owns 30 interior columns (lanes 1..30; lanes 0 and 31 are the halo
// columns, formed redundantly) and walks UR_ROWS rows as a rolling window
// (row above, row, row below), the raw values of the row two below loaded one
// iteration ahead of their use.
// 16 rows per warp, 4 warps per block (measured at 1024^2, per step of 5
// passes: 128.5 us against 131.1 with 8 x 8 and 156 with 32-row warps, whose
// grid leaves too few warps to cover the float64 latency)
constexpr int UR_ROWS = 16;
constexpr int UR_WARPS = 4;

// One block's rows of the float64 pass: block (bx, by) of its grid.
template <bool UPDATE>
__device__ __forceinline__ void update_resid64_tile(int nx, int ny, double* __restrict__ p64a,
                                                    double* __restrict__ p64b, const SolveCtl* ctl,
                                                    const float* __restrict__ e, const float* __restrict__ b,
                                                    const float* __restrict__ b_lo,
                                                    const uint8_t* __restrict__ code, float* __restrict__ r32,
                                                    StepAccum* acc, int bx, int by) {
  __shared__ double red[32];
  __shared__ unsigned long long redn[32];
  const int par = ctl->par;
  const double* p_in = par ? p64b : p64a;
  double* p_out = par ? p64a : p64b;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int gx = bx * 30 - 1 + lane;
  const int y0 = (by * UR_WARPS + w) * UR_ROWS;
  const bool col = gx >= 0 && gx < nx;
  const bool own = col && lane != 0 && lane != 31;

  // raw p64 and e of row y (zero outside the grid), and p64' formed from them
  auto raw = [&](int y, double& rp, float& re) {
    rp = 0.0;
    re = 0.0f;
    if (col && y >= 0 && y < ny) {
      const int k = gx + y * nx;
      rp = p_in[k];
      if (UPDATE) re = e[k];
    }
  };
  auto form = [](double rp, float re) { return UPDATE ? rp + f2d_exact(re) : rp; };
  double rp, rp0;
  float re, re0;
  raw(y0 - 1, rp0, re0);
  raw(y0, rp, re);
  double pm = form(rp0, re0), pc = form(rp, re);
  raw(y0 + 1, rp, re);
  float bnext = 0.0f, blnext = 0.0f;
  uint8_t cnext = (uint8_t)CODE_OUTSIDE;
  if (own && y0 < ny) {
    const int k = gx + y0 * nx;
    bnext = b[k];
    blnext = b_lo[k];
    cnext = code[k];
  }

  double sq = 0.0;
  unsigned long long n = 0;
#pragma unroll 1
  for (int t = 0; t < UR_ROWS; t++) {
    const int gy = y0 + t;
    if (gy >= ny) break;  // the same for the whole warp
    const double pp = form(rp, re);
    raw(gy + 2, rp, re);
    const float bv = bnext, blv = blnext;
    const uint8_t c = cnext;
    if (own && gy + 1 < ny && t + 1 < UR_ROWS) {
      const int k = gx + (gy + 1) * nx;
      bnext = b[k];
      blnext = b_lo[k];
      cnext = code[k];
    }
    const double left = __shfl_up_sync(0xffffffffu, pc, 1);
    const double right = __shfl_down_sync(0xffffffffu, pc, 1);
    if (own) {
      const int k = gx + gy * nx;
      if (UPDATE) p_out[k] = pc;
      float r = 0.0f;
      const int cnt = code_count(c);
      if ((c & 3u) == FLUID && cnt > 0) {
        // the first linked term enters as 0.0 + term
        double sum;
        bool first = true;
        if (c & LINK_XP) {
          sum = zero_plus(right);
          first = false;
        }
        if (c & LINK_XM) {
          sum = first ? zero_plus(left) : sum + left;
          first = false;
        }
        if (c & LINK_YP) {
          sum = first ? zero_plus(pp) : sum + pp;
          first = false;
        }
        if (c & LINK_YM) sum = first ? zero_plus(pm) : sum + pm;
        const double cp = cnt == 4 ? scale_pow2(pc, 2)
                          : cnt == 2 ? scale_pow2(pc, 1)
                          : cnt == 1 ? pc
                                     : dmul_slow(pc, 3.0);
        // b + b_lo is exact in double (at most 49 significant bits)
        const double rd = (f2d_exact(bv) + f2d_exact(blv)) - (cp - sum);
        r = d2f_rn(rd);
        sq = fma(rd, rd, sq);
        n += 1;
      }
      r32[k] = r;
    }
    pm = pc;
    pc = pp;
  }
  const double bs = block_sum(sq, red);
  const unsigned long long bn = block_sum_u64(n, redn);
  if (threadIdx.x == 0) {
    atomicAdd(&acc->res_sq, bs);
    atomicAdd(&acc->n_res, bn);
  }
}

// The same pass with the double-float pressure (fl_params.mixed = 2): p' =
// p + e per cell (df_add_f), then r = b - (count*p' - sum) in double-float
// arithmetic, the neighbour sum in the order +x, -x, +y, -y starting from
// the first linked neighbour, r32 = the pair rounded to float. All of it is
// float32 arithmetic (~80 operations per cell), so unlike the float64 pass
// this one is bound by memory, not by a pipe: a warp owns 30 interior
// columns (lanes 1..30; lanes 0 and 31 load the halo columns) of DF_ROWS
// rows and issues every load of its rows (DF_ROWS + 2 rows of p and e,
// DF_ROWS of b and codes) before any arithmetic, so each warp waits for
// memory once. The residual norm sums r32^2: each square is an exact pair
// (the product and its FMA error), accumulated per thread as a double-float
// and widened to double once per thread for the block reduction.
// At 64 registers 8 blocks fit an SM, so a 1024^2 grid's 1120 blocks run
// in one wave (at 72 registers, 7 per SM, the last 56 blocks made a second).
constexpr int DF_ROWS = 8;
constexpr int DF_WARPS = 4;

// One block's rows of the double-float pass: block (bx, by) of its grid.
template <bool UPDATE>
__device__ __forceinline__ void update_resid_df_tile(int nx, int ny, float2* __restrict__ p2a,
                                                     float2* __restrict__ p2b, const SolveCtl* ctl,
                                                     const float* __restrict__ e, const float* __restrict__ b,
                                                     const float* __restrict__ b_lo,
                                                     const uint8_t* __restrict__ code, float* __restrict__ r32,
                                                     StepAccum* acc, int bx, int by) {
  __shared__ double red[32];
  __shared__ unsigned long long redn[32];
  const int par = ctl->par;
  const float2* p_in = par ? p2b : p2a;
  float2* p_out = par ? p2a : p2b;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int gx = bx * 30 - 1 + lane;
  const int y0 = (by * DF_WARPS + w) * DF_ROWS;
  const bool col = gx >= 0 && gx < nx;
  const bool own = col && lane != 0 && lane != 31;

  // rows y0-1 .. y0+DF_ROWS of p (and e), rows y0 .. y0+DF_ROWS-1 of b and
  // the codes; zero / outside where the grid ends
  float2 P[DF_ROWS + 2];
  float E[DF_ROWS + 2];
  float B[DF_ROWS], BL[DF_ROWS];
  uint8_t C[DF_ROWS];
#pragma unroll
  for (int r = 0; r < DF_ROWS + 2; r++) {
    const int y = y0 - 1 + r;
    P[r] = make_float2(0.0f, 0.0f);
    E[r] = 0.0f;
    if (col && y >= 0 && y < ny) {
      const int k = gx + y * nx;  // 32-bit offsets: a grid holds fewer than 2^31 cells
      P[r] = p_in[k];
      if (UPDATE) E[r] = e[k];
    }
  }
#pragma unroll
  for (int r = 0; r < DF_ROWS; r++) {
    const int y = y0 + r;
    B[r] = 0.0f;
    BL[r] = 0.0f;
    C[r] = (uint8_t)CODE_OUTSIDE;
    if (own && y < ny) {
      const int k = gx + y * nx;
      B[r] = b[k];
      BL[r] = b_lo[k];
      C[r] = code[k];
    }
  }
  if (UPDATE) {
#pragma unroll
    for (int r = 0; r < DF_ROWS + 2; r++) P[r] = df_add_f(P[r], E[r]);
  }

  float2 acc2 = make_float2(0.0f, 0.0f);
  unsigned long long n = 0;
#pragma unroll
  for (int t = 0; t < DF_ROWS; t++) {
    const int gy = y0 + t;
    const float2 pc = P[t + 1];
    const float2 left = make_float2(__shfl_up_sync(0xffffffffu, pc.x, 1), __shfl_up_sync(0xffffffffu, pc.y, 1));
    const float2 right =
        make_float2(__shfl_down_sync(0xffffffffu, pc.x, 1), __shfl_down_sync(0xffffffffu, pc.y, 1));
    if (own && gy < ny) {
      const int k = gx + gy * nx;
      if (UPDATE) p_out[k] = pc;
      const uint8_t c = C[t];
      float r = 0.0f;
      const int cnt = code_count(c);
      if ((c & 3u) == FLUID && cnt > 0) {
        const float2 pp = P[t + 2], pm = P[t];
        float2 sum = make_float2(0.0f, 0.0f);
        bool first = true;
        if (c & LINK_XP) {
          sum = right;
          first = false;
        }
        if (c & LINK_XM) {
          sum = first ? left : df_add(sum, left);
          first = false;
        }
        if (c & LINK_YP) {
          sum = first ? pp : df_add(sum, pp);
          first = false;
        }
        if (c & LINK_YM) sum = first ? pm : df_add(sum, pm);
        const float2 d = df_add(df_mul_count(pc, cnt), df_neg(sum));
        // (b + b_lo) - d: b_lo (the rhs's rounding error) joins the low parts
        const float2 s = df_two_sum(B[t], -d.x);
        r = __fadd_rn(s.x, __fadd_rn(s.y, __fsub_rn(BL[t], d.y)));
        const float q = __fmul_rn(r, r);
        acc2 = df_add(acc2, make_float2(q, __fmaf_rn(r, r, -q)));
        n += 1;
      }
      r32[k] = r;
    }
  }
  const double bs = block_sum_df(acc2, reinterpret_cast<float2*>(red));
  const unsigned long long bn = block_sum_u64(n, redn);
  if (threadIdx.x == 0) {
    atomicAdd(&acc->res_sq, bs);
    atomicAdd(&acc->n_res, bn);
  }
}

__device__ __forceinline__ double acc_rms(double sq, unsigned long long n) { return n ? sqrt(sq / (double)n) : 0.0; }

// Before the cycle loop (pressureMultigrid.ts:294-300, solveMixed): the rhs
// RMS; a vanishing rhs means p = 0 and no cycle; the float64 path also tests
// its initial residual, so a converged warm start costs no cycle.
__device__ int solve_begin_sums(StepAccum* acc, SolveCtl* ctl, double res_sq, unsigned long long n_res) {
  const double b_rms = acc_rms(acc->b_sq, acc->n_fluid);
  ctl->b_rms = b_rms;
  ctl->cycles = 0;
  ctl->zero_p = b_rms == 0.0;
  ctl->nonfinite = !isfinite(b_rms);
  int cont = 0;
  if (ctl->zero_p) {
    ctl->rel = 0.0;
  } else if (ctl->nonfinite) {
    ctl->rel = -1.0;
  } else if (ctl->mode == SOLVE_MIXED) {
    const double rel = acc_rms(res_sq, n_res) / b_rms;
    ctl->rel = rel;
    cont = ctl->max_cycles > 0 && !(rel <= ctl->tol);
  } else {
    ctl->rel = -1.0;
    cont = ctl->max_cycles > 0;
  }
  ctl->rel0 = ctl->rel;
  acc->res_sq = 0.0;
  acc->n_res = 0ull;
  ctl->cont = cont;
  return cont;
}

__device__ int solve_begin(StepAccum* acc, SolveCtl* ctl) { return solve_begin_sums(acc, ctl, acc->res_sq, acc->n_res); }

__global__ void k_solve_begin(StepAccum* acc, SolveCtl* ctl, int use_cond, cudaGraphConditionalHandle h) {
  const int cont = solve_begin(acc, ctl);
  if (use_cond) cudaGraphSetConditional(h, cont);
}

// After each cycle: count it, evaluate the relative residual the cycle's
// last kernel accumulated, and decide on another (pressureMultigrid.ts:
// 314-317 for float32, solveMixed for float64 defect correction).
__device__ int solve_check_sums(StepAccum* acc, SolveCtl* ctl, double res_sq, unsigned long long n_res) {
  ctl->cycles += 1;
  if (ctl->mode == SOLVE_MIXED) ctl->par = 1 - ctl->par;
  const double rel = acc_rms(res_sq, n_res) / ctl->b_rms;
  ctl->rel = rel;
  int cont = ctl->cycles < ctl->max_cycles;
  if (!isfinite(rel)) {
    ctl->nonfinite = 1;
    cont = 0;
  } else if (ctl->mode == SOLVE_MIXED) {
    cont = cont && !(rel <= ctl->tol);
  } else if (ctl->tol > 0) {
    cont = cont && !(rel <= ctl->tol);
  }
  acc->res_sq = 0.0;
  acc->n_res = 0ull;
  ctl->cont = cont;
  return cont;
}

__device__ int solve_check(StepAccum* acc, SolveCtl* ctl) { return solve_check_sums(acc, ctl, acc->res_sq, acc->n_res); }

// The begin test (test 1) or the cycle test (test 2) run by the last block
// of the defect pass that accumulated the residual, instead of a one-thread
// launch after it. Each block's thread 0 has added its sums (the tile's
// last statement) before it counts itself done; the last block reads the
// totals from L2 once every block has counted, and resets the counter.
__device__ __noinline__ void defect_pass_test_last(StepAccum* acc, SolveCtl* ctl, int test, int use_cond,
                                                   cudaGraphConditionalHandle h) {
  __threadfence();
  acc->test_done = 0u;
  const double sq = __ldcg(&acc->res_sq);
  const unsigned long long n = __ldcg(&acc->n_res);
  const int cont = test == 1 ? solve_begin_sums(acc, ctl, sq, n) : solve_check_sums(acc, ctl, sq, n);
  if (use_cond) cudaGraphSetConditional(h, cont);
}

__device__ __forceinline__ void defect_pass_test(StepAccum* acc, SolveCtl* ctl, int test, int use_cond,
                                                 cudaGraphConditionalHandle h) {
  // only the first thread, which added the block's sums, takes part: the
  // block's other threads are done
  if (test == 0 || threadIdx.x != 0) return;
  __threadfence();
  const unsigned int done = atomicAdd(&acc->test_done, 1u);
  if (done != gridDim.x * gridDim.y - 1) return;
  // out of line: the tests' float64 arithmetic stays out of the pass's
  // register budget (64 registers for 8 blocks per SM)
  defect_pass_test_last(acc, ctl, test, use_cond, h);
}

__global__ void k_solve_check(StepAccum* acc, SolveCtl* ctl, int use_cond, cudaGraphConditionalHandle h) {
  const int cont = solve_check(acc, ctl);
  if (use_cond) cudaGraphSetConditional(h, cont);
}

// After the loop: when the rhs vanished the answer is p = 0 (float32 field
// or the current float64 buffer).
__global__ void k_zero_if(const SolveCtl* __restrict__ ctl, float* __restrict__ p32, double* __restrict__ p64a,
                          double* __restrict__ p64b, long n) {
  if (!ctl->zero_p) return;
  double* p64 = p64a ? (ctl->par ? p64b : p64a) : nullptr;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    if (p32) p32[k] = 0.0f;
    if (p64) p64[k] = 0.0;
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
  double sq = 0.0;
  unsigned long long n = 0;
  for (int j = blockIdx.y * blockDim.y + threadIdx.y; j < ny; j += gridDim.y * blockDim.y) {
    if (i >= nx) break;
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
      sq += r * r;
      n += 1;
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

template <int P, int MODE, int R>
static void launch_smooth_r(cudaStream_t s, const SmoothArgs& a) {
  constexpr int T = Tile<P, MODE, R>::T;
  dim3 blk(R / 2, R / 2);
  dim3 grd((a.nx + T - 1) / T, (a.ny + T - 1) / T);
  k_smooth<P, MODE, R><<<grd, blk, 0, s>>>(a);
}

// 64^2 regions unless they would leave most SMs idle: below 64 such CTAs
// (levels of about 400^2 and smaller) the 32^2 regions' extra CTAs win over
// their larger halo share (measured: 256^2 and 128^2 faster, 512^2 slower).
template <int P, int MODE>
static void launch_smooth_t(cudaStream_t s, const SmoothArgs& a) {
  constexpr int T = Tile<P, MODE, 64>::T;
  const long blocks64 = (long)((a.nx + T - 1) / T) * ((a.ny + T - 1) / T);
  if (blocks64 < 64)
    launch_smooth_r<P, MODE, 32>(s, a);
  else
    launch_smooth_r<P, MODE, 64>(s, a);
}

template <int MODE>
static bool launch_smooth_p(cudaStream_t s, const SmoothArgs& a, int pairs) {
  switch (pairs) {
    case 0: if (MODE != MODE_PLAIN) { launch_smooth_t<0, MODE>(s, a); return true; } return false;
    case 1: launch_smooth_t<1, MODE>(s, a); return true;
    case 2: launch_smooth_t<2, MODE>(s, a); return true;
    case 3: launch_smooth_t<3, MODE>(s, a); return true;
    case 4: launch_smooth_t<4, MODE>(s, a); return true;
    default: return false;
  }
}

static bool launch_smooth(cudaStream_t s, const SmoothArgs& a, int pairs, int mode) {
  if (mode == MODE_PLAIN) return launch_smooth_p<MODE_PLAIN>(s, a, pairs);
  if (mode == MODE_PRE) return launch_smooth_p<MODE_PRE>(s, a, pairs);
  return launch_smooth_p<MODE_POST>(s, a, pairs);
}

void launch_build_codes(cudaStream_t s, int nx, int ny, const uint8_t* label, uint8_t* code, const int* only_if) {
  dim3 b(32, 8), g((nx + 31) / 32, (ny + 7) / 8);
  k_build_codes<<<g, b, 0, s>>>(nx, ny, label, code, only_if);
}

void launch_rb_halfsweep(cudaStream_t s, int nx, int ny, float* p, const float* b, const uint8_t* code,
                         float scale, float omega, int color) {
  dim3 bl(32, 8), g((nx + 31) / 32, (ny + 7) / 8);
  k_rb_halfsweep<<<g, bl, 0, s>>>(nx, ny, p, b, code, scale, omega, color);
}

void launch_rb_sweeps(cudaStream_t s, int nx, int ny, const float* x_in, float* x_out, const float* b,
                      const uint8_t* code, float scale, float omega, int pairs, const float* scale_dev) {
  SmoothArgs a{};
  a.scale_dev = scale_dev;
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

template <bool UPDATE>
__global__ void __launch_bounds__(32 * UR_WARPS) k_update_resid64(int nx, int ny, double* __restrict__ p64a,
                                                                double* __restrict__ p64b,
                                                                SolveCtl* ctl, const float* __restrict__ e,
                                                                const float* __restrict__ b,
                                                                const float* __restrict__ b_lo,
                                                                const uint8_t* __restrict__ code,
                                                                float* __restrict__ r32, StepAccum* acc, int test,
                                                                int use_cond, cudaGraphConditionalHandle h) {
  update_resid64_tile<UPDATE>(nx, ny, p64a, p64b, ctl, e, b, b_lo, code, r32, acc, blockIdx.x, blockIdx.y);
  defect_pass_test(acc, ctl, test, use_cond, h);
}

template <bool UPDATE>
__global__ void __launch_bounds__(32 * DF_WARPS, 8) k_update_resid_df(int nx, int ny, float2* __restrict__ p2a,
                                                                   float2* __restrict__ p2b,
                                                                   SolveCtl* ctl, const float* __restrict__ e,
                                                                   const float* __restrict__ b,
                                                                   const float* __restrict__ b_lo,
                                                                   const uint8_t* __restrict__ code,
                                                                   float* __restrict__ r32, StepAccum* acc,
                                                                   int test, int use_cond,
                                                                   cudaGraphConditionalHandle h) {
  update_resid_df_tile<UPDATE>(nx, ny, p2a, p2b, ctl, e, b, b_lo, code, r32, acc, blockIdx.x, blockIdx.y);
  defect_pass_test(acc, ctl, test, use_cond, h);
}

void launch_update_resid64(cudaStream_t s, int nx, int ny, double* p64a, double* p64b, SolveCtl* ctl,
                           const float* e, const float* b, const float* b_lo, const uint8_t* code, bool update,
                           float* r32, StepAccum* acc, bool df, int test, bool use_cond,
                           cudaGraphConditionalHandle h) {
  const int uc = use_cond ? 1 : 0;
  if (df) {
    float2* a = reinterpret_cast<float2*>(p64a);
    float2* bb = reinterpret_cast<float2*>(p64b);
    dim3 g((nx + 29) / 30, (ny + DF_WARPS * DF_ROWS - 1) / (DF_WARPS * DF_ROWS));
    if (update)
      k_update_resid_df<true><<<g, 32 * DF_WARPS, 0, s>>>(nx, ny, a, bb, ctl, e, b, b_lo, code, r32, acc, test, uc, h);
    else
      k_update_resid_df<false><<<g, 32 * DF_WARPS, 0, s>>>(nx, ny, a, bb, ctl, e, b, b_lo, code, r32, acc, test, uc,
                                                           h);
    return;
  }
  dim3 g((nx + 29) / 30, (ny + UR_WARPS * UR_ROWS - 1) / (UR_WARPS * UR_ROWS));
  if (update)
    k_update_resid64<true><<<g, 32 * UR_WARPS, 0, s>>>(nx, ny, p64a, p64b, ctl, e, b, b_lo, code, r32, acc, test, uc,
                                                       h);
  else
    k_update_resid64<false><<<g, 32 * UR_WARPS, 0, s>>>(nx, ny, p64a, p64b, ctl, e, b, b_lo, code, r32, acc, test,
                                                        uc, h);
}

void launch_solve_begin(cudaStream_t s, StepAccum* acc, SolveCtl* ctl, bool use_cond, cudaGraphConditionalHandle h) {
  k_solve_begin<<<1, 1, 0, s>>>(acc, ctl, use_cond, h);
}

void launch_solve_check(cudaStream_t s, StepAccum* acc, SolveCtl* ctl, bool use_cond, cudaGraphConditionalHandle h) {
  k_solve_check<<<1, 1, 0, s>>>(acc, ctl, use_cond, h);
}

void launch_zero_if(cudaStream_t s, const SolveCtl* ctl, float* p32, double* p64a, double* p64b, long n) {
  long blocks = std::min((n + 255) / 256, 152L * 4);
  k_zero_if<<<(unsigned)std::max(1L, blocks), 256, 0, s>>>(ctl, p32, p64a, p64b, n);
}

void launch_rms_remaining(cudaStream_t s, int nx, int ny, const float* p, const float* div, const uint8_t* code,
                          float scale, StepAccum* acc) {
  dim3 b(32, 8), g((nx + 31) / 32, (ny + 7) / 8);
  g.y = std::min(g.y, std::max(1u, 1024u / g.x));
  k_rms_remaining<<<g, b, 0, s>>>(nx, ny, p, div, code, scale, acc);
}

// Shared-memory layout of the single-CTA tail for levels from..end.
// log2 of the lanes a tail level gives one row of one colour: the power of
// two >= ceil(nx / 2); also the row stride of its parity planes.
static int tail_lsh(int nx) {
  int lpr = 1, lsh = 0;
  while (lpr < (nx + 1) / 2) {
    lpr <<= 1;
    lsh++;
  }
  return lsh;
}

static size_t coarse_smem_bytes(const Engine& e, int from, int* off_x, int* off_b, int* off_c) {
  size_t floats = 4;  // 16 bytes: the zero word
  for (int l = from; l < (int)e.levels.size(); l++) {
    const long n = (long)e.levels[l].nx * e.levels[l].ny;
    if (off_x) off_x[l - from] = (int)floats;
    floats += 2 * ((size_t)1 << tail_lsh(e.levels[l].nx)) * (size_t)e.levels[l].ny;
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

// The dynamic shared-memory limit of k_mg_coarse is a per-device property
// of the function, shared by every engine in the process: it only ever grows
// to the largest tail any engine on the device needs (an engine with a
// smaller tail must not lower it under another engine's launches).
static void raise_coarse_smem_limit(int device, size_t bytes) {
  static std::mutex mu;
  static size_t limit[256] = {};
  std::lock_guard<std::mutex> lock(mu);
  if (device < 0 || device >= 256 || bytes <= limit[device]) return;
  if (cudaFuncSetAttribute(k_mg_coarse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess)
    limit[device] = bytes;
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
  // the tail starts at the first level with both sides <= mg_tail_side (the
  // coarsest level at the latest)
  const int side = e.prm.mg_tail_side > 0 ? e.prm.mg_tail_side : TAIL_SIDE_DEFAULT;
  int lc = (int)e.levels.size() - 1;
  for (int l = 0; l < (int)e.levels.size(); l++)
    if (e.levels[l].nx <= side && e.levels[l].ny <= side) {
      lc = l;
      break;
    }
  e.coarse_level = lc;
  e.coarse_smem = coarse_smem_bytes(e, lc, nullptr, nullptr, nullptr);
  raise_coarse_smem_limit(e.device, e.coarse_smem);
  e.codes_valid = false;
}

void mg_build_codes(Engine& e) {
  cudaStream_t s = e.stream;
  for (size_t l = 1; l < e.levels.size(); l++) {
    const Level& F = e.levels[l - 1];
    const Level& C = e.levels[l];
    dim3 b(32, 8), g((C.nx + 31) / 32, (C.ny + 7) / 8);
    k_coarsen_labels<<<g, b, 0, s>>>(F.nx, F.ny, F.label, C.nx, C.ny, C.label, nullptr);
  }
  for (const Level& L : e.levels) launch_build_codes(s, L.nx, L.ny, L.label, L.code);
  e.codes_valid = true;
}

__global__ void k_clear_flag(int* flag) { *flag = 0; }

// The same rebuild on stream s as kernels that each return at once unless
// *flag is set (the label compare's result), then the flag cleared: a
// plain graph's worth of launches where an IF node would otherwise decide.
void mg_build_codes_if(Engine& e, cudaStream_t s, int* flag) {
  for (size_t l = 1; l < e.levels.size(); l++) {
    const Level& F = e.levels[l - 1];
    const Level& C = e.levels[l];
    dim3 b(32, 8), g((C.nx + 31) / 32, (C.ny + 7) / 8);
    k_coarsen_labels<<<g, b, 0, s>>>(F.nx, F.ny, F.label, C.nx, C.ny, C.label, flag);
  }
  for (const Level& L : e.levels) launch_build_codes(s, L.nx, L.ny, L.label, L.code, flag);
  k_clear_flag<<<1, 1, 0, s>>>(flag);
}

// One V-cycle (pressureMultigrid.ts:253-275) on levels[0].b with the warm
// start in levels[0].x[0]; the result lands back in levels[0].x[0]. When
// `acc` is set, the finest level's residual sum of squares is accumulated
// into it for the tolerance test.
void mg_vcycle(Engine& e, StepAccum* acc) { mg_vcycle_on(e, e.levels[0].b, false, acc); }

// One V-cycle with level 0's rhs `b0`; with `zero_start` the level-0 unknown
// starts from 0 (the correction equation of the defect-correction loop)
// instead of the warm start in levels[0].x[0].
// The single-CTA tail's arguments for a V-cycle on b0 (the finest level's
// rhs when the tail starts there), from zero when zero_start, accumulating
// the finest residual into acc when the tail holds the finest level.
static CoarseArgs coarse_args(const Engine& e, const float* b0, bool zero_start, StepAccum* acc) {
  const int lc = e.coarse_level;
  CoarseArgs a{};
  int ox[MAX_LEVELS], ob[MAX_LEVELS], oc[MAX_LEVELS];
  coarse_smem_bytes(e, lc, ox, ob, oc);
  a.nlev = (int)e.levels.size() - lc;
  for (int l = 0; l < a.nlev; l++) {
    const Level& L = e.levels[lc + l];
    const int lsh = tail_lsh(L.nx);
    const int rows_per_warp = 32 >> lsh;
    const int groups = (L.ny + rows_per_warp - 1) / rows_per_warp;
    a.lv[l] = CoarseLevel{L.nx, L.ny, L.code, ox[l], ob[l], oc[l], lsh, std::min(32, groups), groups > 32 ? 2 : 1};
  }
  a.b_top = lc == 0 ? b0 : e.levels[lc].b;
  a.x_top = e.levels[lc].x[0];
  a.x_is_zero = lc > 0 || zero_start;
  a.pre = e.prm.mg_pre;
  a.post = e.prm.mg_post;
  a.coarse_sweeps = e.prm.mg_coarse_sweeps;
  a.omega = (float)e.prm.mg_omega;
  a.acc = lc == 0 ? acc : nullptr;
  return a;
}

void mg_vcycle_on(Engine& e, const float* b0, bool zero_start, StepAccum* acc) {
  cudaStream_t s = e.stream;
  const int lc = e.coarse_level;
  const float omega = (float)e.prm.mg_omega;
  auto cells = [&](int l) { return (double)e.levels[l].nx * e.levels[l].ny; };
  for (int l = 0; l < lc; l++) {
    Level& L = e.levels[l];
    Level& C = e.levels[l + 1];
    // x (level 0 only: coarser levels start from zero), b, code, x out, coarse b
    const int tok = prof_begin(e, l == 0 ? FL_PH_MG_PRE_FINE : FL_PH_MG_PRE);
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
    const CoarseArgs a = coarse_args(e, b0, zero_start, acc);
    k_mg_coarse<<<1, dim3(32, 32), e.coarse_smem, s>>>(a);
    prof_end(e, tok, bytes, 1);
  }
  for (int l = lc - 1; l >= 0; l--) {
    Level& L = e.levels[l];
    Level& C = e.levels[l + 1];
    // x in, b, code, coarse e, x out
    const int tok = prof_begin(e, l == 0 ? FL_PH_MG_POST_FINE : FL_PH_MG_POST);
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


// ------------------------------------------------------------ batched solve
//
// The pressure solves of many engines advanced together (fl_batch): each
// V-cycle phase is ONE launch over a list of (scene, level, tile) items
// drawn from every scene of the batch, the scenes' tails aligned (a scene
// with fewer levels above its tail joins the descent later and leaves the
// ascent earlier), and the cycle loop is one device-side WHILE over "some
// scene still iterates". A scene that has converged (its control block's
// `cont` cleared by its own test) leaves its items at once, so every scene
// runs exactly the cycles it would run alone, through the same per-tile code
// (smooth_tile, mg_coarse_body, the defect-pass tiles, solve_begin /
// solve_check): its results are bit-identical to stepping it alone.

struct BatchLevel {
  int nx, ny;
  float* x0;
  float* x1;
  float* b;
  const uint8_t* code;
};

struct BatchScene {
  BatchLevel lv[MAX_LEVELS];
  CoarseArgs tail;
  double* p64a;
  double* p64b;
  float* r32;
  float* b_lo;
  SolveCtl* ctl;
  StepAccum* acc;
  long cells;
  int nlev, lc, mixed;
  float omega;
};

struct BatchItem {
  int scene, level, bx, by;
};

// The plan's device-side lists. Cycle phases ph: PRE at depth d (0..D-1),
// the tail (D), POST at depth d (D+1..2D), the defect pass (2D+1); items of
// scene k in phase ph are items[base[ph][k] .. + count[ph][k]). The begin and
// check kernels compact, per phase, the scenes still iterating: act_scene
// (in the plan's order, largest scenes first), act_pre (exclusive prefix of
// their item counts), act_n and act_total; a phase kernel's blocks walk
// 0 .. act_total by the grid's stride.
struct BatchPlan {
  const BatchScene* sc;
  const BatchItem* items;
  const int* base;
  const int* count;
  int* act_scene;
  int* act_pre;
  int* act_n;
  int* act_total;
  int n, nph;
};

struct BatchSolve {
  int device = 0;
  int n = 0, depth = 0, sms = 0;
  int pre = 0, post = 0;
  bool any_mixed = false;
  size_t tail_smem = 0;
  BatchScene* scenes = nullptr;  // device, largest scene first
  BatchItem* items = nullptr;    // device
  int* lists = nullptr;          // device: base, count, act_scene, act_pre, act_n, act_total
  BatchPlan plan{};
  std::vector<int> max_items;    // per cycle phase: all scenes' items (the grid's bound)
  std::pair<int, int> init_ph{0, 0}, zero_ph{0, 0};  // prologue defect pass, p = 0 fill: every scene
};

__device__ __forceinline__ bool batch_item(const BatchPlan& P, int ph, int i, BatchItem& it) {
  if (i >= P.act_total[ph]) return false;
  const int* pre = P.act_pre + (long)ph * (P.n + 1);
  int lo = 0, hi = P.act_n[ph] - 1;  // the last active scene whose prefix is <= i
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int k = P.act_scene[(long)ph * P.n + lo];
  it = P.items[P.base[(long)ph * P.n + k] + (i - pre[lo])];
  return true;
}

// Per phase, the items of the scenes whose control block says they iterate
// (one warp per phase, a warp-wide scan per 32 scenes). Called by a whole
// block after the scenes' tests, behind a barrier.
__device__ void batch_compact(const BatchPlan& P) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int ph = w; ph < P.nph; ph += nw) {
    int run = 0, nact = 0;
    for (int c = 0; c < P.n; c += 32) {
      const int k = c + lane;
      const int cnt = k < P.n && P.sc[k].ctl->cont ? P.count[(long)ph * P.n + k] : 0;
      int x = cnt;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      const unsigned on = __ballot_sync(0xffffffffu, cnt > 0);
      if (cnt > 0) {
        const int pos = nact + __popc(on & ((1u << lane) - 1u));
        P.act_scene[(long)ph * P.n + pos] = k;
        P.act_pre[(long)ph * (P.n + 1) + pos] = run + x - cnt;
      }
      run += __shfl_sync(0xffffffffu, x, 31);
      nact += __popc(on);
    }
    if (lane == 0) {
      P.act_total[ph] = run;
      P.act_n[ph] = nact;
      P.act_pre[(long)ph * (P.n + 1) + nact] = run;
    }
  }
}

template <int P, int MODE>
__global__ void __launch_bounds__(1024, 1) k_batch_smooth(BatchPlan plan, int ph) {
  for (int i = blockIdx.x;; i += gridDim.x) {
    BatchItem it;
    if (!batch_item(plan, ph, i, it)) return;  // the same for the whole block
    const BatchScene& S = plan.sc[it.scene];
    const int l = it.level;
    const BatchLevel& L = S.lv[l];
    const BatchLevel& C = S.lv[l + 1];
    // the arguments mg_vcycle_on gives this level (mixed: a V-cycle on the
    // defect pass's residual from zero; otherwise on b from the warm start)
    SmoothArgs a{};
    a.nx = L.nx;
    a.ny = L.ny;
    a.code = L.code;
    a.scale = -1.0f;
    a.omega = S.omega;
    a.cnx = C.nx;
    a.cny = C.ny;
    a.b = l == 0 && S.mixed ? S.r32 : L.b;
    if (MODE == MODE_PRE) {
      a.xin = L.x0;
      a.xout = L.x1;
      a.bc = C.b;
      a.x_is_zero = l > 0 || S.mixed;
    } else {
      a.xin = L.x1;
      a.xout = L.x0;
      a.ec = C.x0;
      a.acc = l == 0 && !S.mixed ? S.acc : nullptr;
    }
    smooth_tile<P, MODE, 64, false>(a, it.bx, it.by);
    __syncthreads();  // the next region reuses the shared tiles
  }
}

__global__ void __launch_bounds__(1024, 1) k_batch_tail(BatchPlan plan, int ph) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int i = blockIdx.x;; i += gridDim.x) {
    BatchItem it;
    if (!batch_item(plan, ph, i, it)) return;
    mg_coarse_body(plan.sc[it.scene].tail, smem);
    __syncthreads();
  }
}

template <bool UPDATE>
__device__ __forceinline__ void batch_defect_item(const BatchScene& S, const BatchItem& it) {
  const BatchLevel& L0 = S.lv[0];
  const float* e = UPDATE ? L0.x0 : nullptr;
  if (S.mixed == MIXED_DF)
    update_resid_df_tile<UPDATE>(L0.nx, L0.ny, reinterpret_cast<float2*>(S.p64a), reinterpret_cast<float2*>(S.p64b),
                                 S.ctl, e, L0.b, S.b_lo, L0.code, S.r32, S.acc, it.bx, it.by);
  else
    update_resid64_tile<UPDATE>(L0.nx, L0.ny, S.p64a, S.p64b, S.ctl, e, L0.b, S.b_lo, L0.code, S.r32, S.acc, it.bx,
                                it.by);
}

// The defect pass of the iterating scenes with a refined pressure: p += e
// and the new residual.
__global__ void __launch_bounds__(32 * UR_WARPS) k_batch_defect(BatchPlan plan, int ph) {
  for (int i = blockIdx.x;; i += gridDim.x) {
    BatchItem it;
    if (!batch_item(plan, ph, i, it)) return;
    batch_defect_item<true>(plan.sc[it.scene], it);
    __syncthreads();
  }
}

// The initial defect pass of every scene with a refined pressure (before
// the loop), one item per block.
__global__ void __launch_bounds__(32 * UR_WARPS) k_batch_defect_init(const BatchScene* __restrict__ sc,
                                                                    const BatchItem* __restrict__ items) {
  const BatchItem it = items[blockIdx.x];
  batch_defect_item<false>(sc[it.scene], it);
}

// Every scene's begin test, the compacted lists of the first cycle; the
// WHILE node runs while any scene iterates.
__global__ void __launch_bounds__(1024) k_batch_begin(BatchPlan plan, cudaGraphConditionalHandle h) {
  int any = 0;
  for (int k = threadIdx.x; k < plan.n; k += blockDim.x) any |= solve_begin(plan.sc[k].acc, plan.sc[k].ctl);
  any = __syncthreads_or(any);
  batch_compact(plan);
  if (threadIdx.x == 0) cudaGraphSetConditional(h, any ? 1u : 0u);
}

// Every iterating scene's cycle test (the others keep their state), the
// compacted lists of the next cycle.
__global__ void __launch_bounds__(1024) k_batch_check(BatchPlan plan, cudaGraphConditionalHandle h) {
  int any = 0;
  for (int k = threadIdx.x; k < plan.n; k += blockDim.x)
    if (plan.sc[k].ctl->cont) any |= solve_check(plan.sc[k].acc, plan.sc[k].ctl);
  any = __syncthreads_or(any);
  batch_compact(plan);
  if (threadIdx.x == 0) cudaGraphSetConditional(h, any ? 1u : 0u);
}

// k_zero_if per scene: item (scene, -, block, blocks of the scene).
__global__ void __launch_bounds__(256) k_batch_zero(const BatchScene* __restrict__ sc,
                                                    const BatchItem* __restrict__ items) {
  const BatchItem it = items[blockIdx.x];
  const BatchScene& S = sc[it.scene];
  if (!S.ctl->zero_p) return;
  float* p32 = S.mixed ? nullptr : S.lv[0].x0;
  double* p64 = S.mixed ? (S.ctl->par ? S.p64b : S.p64a) : nullptr;
  for (long k = it.bx * 256L + threadIdx.x; k < S.cells; k += (long)it.by * 256) {
    if (p32) p32[k] = 0.0f;
    if (p64) p64[k] = 0.0;
  }
}

BatchSolve* batch_solve_create(const std::vector<Engine*>& es_in, std::string& why) {
  if (es_in.empty()) {
    why = "no scenes";
    return nullptr;
  }
  const fl_params& p0 = es_in[0]->prm;
  for (const Engine* e : es_in) {
    if (e->prm.solver != FL_SOLVER_MG) why = "a scene solves with red-black SOR";
    else if (e->prm.mg_pre != p0.mg_pre || e->prm.mg_post != p0.mg_post)
      why = "the scenes' V-cycle shapes differ";
    else if (e->prm.mg_pre < 0 || e->prm.mg_pre > 4 || e->prm.mg_post < 0 || e->prm.mg_post > 4)
      why = "sweep pairs beyond 4";
    else if ((int)e->levels.size() > MAX_LEVELS || e->levels.empty())
      why = "too many levels";
    if (!why.empty()) return nullptr;
  }
  // the plan's scenes, largest first (blocks walk the items in this order)
  std::vector<const Engine*> es(es_in.begin(), es_in.end());
  std::stable_sort(es.begin(), es.end(), [](const Engine* x, const Engine* y) { return x->cells() > y->cells(); });
  BatchSolve* b = new BatchSolve();
  b->device = es[0]->device;
  b->n = (int)es.size();
  b->pre = p0.mg_pre;
  b->post = p0.mg_post;
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
  if (b->sms < 1) b->sms = 1;
  std::vector<BatchScene> hs(es.size());
  for (size_t k = 0; k < es.size(); k++) {
    const Engine& e = *es[k];
    BatchScene& S = hs[k];
    std::memset(&S, 0, sizeof S);
    S.nlev = (int)e.levels.size();
    S.lc = e.coarse_level;
    S.mixed = e.prm.mixed;
    S.omega = (float)e.prm.mg_omega;
    S.cells = e.cells();
    for (int l = 0; l < S.nlev; l++) {
      const Level& L = e.levels[l];
      S.lv[l] = BatchLevel{L.nx, L.ny, L.x[0], L.x[1], L.b, L.code};
    }
    const bool mixed = e.prm.mixed != 0;
    S.tail = coarse_args(e, mixed ? e.r32 : e.levels[0].b, mixed, mixed ? nullptr : e.acc);
    S.p64a = e.p64[0];
    S.p64b = e.p64[1];
    S.r32 = e.r32;
    S.b_lo = e.b_lo;
    S.ctl = e.ctl;
    S.acc = e.acc;
    b->any_mixed = b->any_mixed || mixed;
    b->tail_smem = std::max(b->tail_smem, e.coarse_smem);
    b->depth = std::max(b->depth, S.lc);
  }
  const int n = b->n, depth = b->depth, nph = 2 * depth + 2;
  std::vector<BatchItem> items;
  std::vector<int> base((size_t)nph * n, 0), count((size_t)nph * n, 0);
  b->max_items.assign(nph, 0);
  // scene k's items of phase ph, appended
  auto add = [&](int ph, int k, auto&& emit) {
    base[(size_t)ph * n + k] = (int)items.size();
    emit();
    count[(size_t)ph * n + k] = (int)items.size() - base[(size_t)ph * n + k];
    b->max_items[ph] += count[(size_t)ph * n + k];
  };
  auto smooth_items = [&](int k, int l, int halo) {
    const int T = 64 - 2 * halo;
    const BatchLevel& L = hs[k].lv[l];
    for (int by = 0; by < (L.ny + T - 1) / T; by++)
      for (int bx = 0; bx < (L.nx + T - 1) / T; bx++) items.push_back(BatchItem{k, l, bx, by});
  };
  auto defect_items = [&](int k) {
    const BatchLevel& L = hs[k].lv[0];
    const int rows = hs[k].mixed == MIXED_DF ? DF_WARPS * DF_ROWS : UR_WARPS * UR_ROWS;
    for (int by = 0; by < (L.ny + rows - 1) / rows; by++)
      for (int bx = 0; bx < (L.nx + 29) / 30; bx++) items.push_back(BatchItem{k, 0, bx, by});
  };
  for (int k = 0; k < n; k++) {
    // PRE: level lc_k - depth + d at phase d (the tails aligned); POST: level
    // lc_k - 1 - d at phase depth + 1 + d
    for (int d = 0; d < depth; d++) {
      const int l = hs[k].lc - depth + d;
      if (l >= 0) add(d, k, [&] { smooth_items(k, l, 2 * b->pre + 1); });
    }
    add(depth, k, [&] { items.push_back(BatchItem{k, hs[k].lc, 0, 0}); });
    for (int d = 0; d < depth; d++) {
      const int l = hs[k].lc - 1 - d;
      if (l >= 0) add(depth + 1 + d, k, [&] { smooth_items(k, l, 2 * b->post + 1); });
    }
    if (hs[k].mixed) add(2 * depth + 1, k, [&] { defect_items(k); });
  }
  b->init_ph.first = (int)items.size();
  for (int k = 0; k < n; k++)
    if (hs[k].mixed) defect_items(k);
  b->init_ph.second = (int)items.size() - b->init_ph.first;
  b->zero_ph.first = (int)items.size();
  for (int k = 0; k < n; k++) {
    const int blocks = (int)std::min<long>(64, std::max<long>(1, (hs[k].cells + 255) / 256));
    for (int q = 0; q < blocks; q++) items.push_back(BatchItem{k, 0, q, blocks});
  }
  b->zero_ph.second = (int)items.size() - b->zero_ph.first;
  // lists: base, count [nph*n]; act_scene [nph*n]; act_pre [nph*(n+1)]; act_n, act_total [nph]
  const size_t nl = 3 * (size_t)nph * n + (size_t)nph * (n + 1) + 2 * (size_t)nph;
  cudaError_t err = cudaMalloc(&b->scenes, hs.size() * sizeof(BatchScene));
  if (err == cudaSuccess) err = cudaMalloc(&b->items, items.size() * sizeof(BatchItem));
  if (err == cudaSuccess) err = cudaMalloc(&b->lists, nl * sizeof(int));
  if (err == cudaSuccess) err = cudaMemset(b->lists, 0, nl * sizeof(int));
  if (err == cudaSuccess)
    err = cudaMemcpy(b->scenes, hs.data(), hs.size() * sizeof(BatchScene), cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(b->items, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(b->lists, base.data(), base.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(b->lists + base.size(), count.data(), count.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (err == cudaSuccess && b->tail_smem > 48 * 1024)
    err = cudaFuncSetAttribute(k_batch_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->tail_smem);
  if (err != cudaSuccess) {
    why = cudaGetErrorString(err);
    batch_solve_destroy(b);
    return nullptr;
  }
  BatchPlan& P = b->plan;
  P.sc = b->scenes;
  P.items = b->items;
  P.base = b->lists;
  P.count = b->lists + (size_t)nph * n;
  P.act_scene = b->lists + 2 * (size_t)nph * n;
  P.act_pre = b->lists + 3 * (size_t)nph * n;
  P.act_n = P.act_pre + (size_t)nph * (n + 1);
  P.act_total = P.act_n + nph;
  P.n = n;
  P.nph = nph;
  return b;
}

void batch_solve_destroy(BatchSolve* b) {
  if (!b) return;
  cudaFree(b->scenes);
  cudaFree(b->items);
  cudaFree(b->lists);
  delete b;
}

// A cycle phase: a grid of at most `per_sm` blocks per SM (bounded by the
// phase's items over all scenes) walking the iterating scenes' items.
static unsigned phase_grid(const BatchSolve& b, int ph, int per_sm) {
  return (unsigned)std::max(1, std::min(b.max_items[ph], b.sms * per_sm));
}

template <int MODE>
static void launch_batch_smooth(cudaStream_t s, const BatchSolve& b, int pairs, int ph) {
  if (b.max_items[ph] == 0) return;
  const dim3 blk(32, 32), g(phase_grid(b, ph, 1));
  switch (pairs) {
    case 0: k_batch_smooth<0, MODE><<<g, blk, 0, s>>>(b.plan, ph); break;
    case 1: k_batch_smooth<1, MODE><<<g, blk, 0, s>>>(b.plan, ph); break;
    case 2: k_batch_smooth<2, MODE><<<g, blk, 0, s>>>(b.plan, ph); break;
    case 3: k_batch_smooth<3, MODE><<<g, blk, 0, s>>>(b.plan, ph); break;
    default: k_batch_smooth<4, MODE><<<g, blk, 0, s>>>(b.plan, ph); break;
  }
}

// The whole batched solve, enqueued on `s` while it is being captured: the
// initial defect pass and begin test, a WHILE node whose body (captured from
// `body`) is one V-cycle of every iterating scene plus the defect pass and
// the cycle tests, then the p = 0 fill of scenes whose rhs vanished.
cudaError_t batch_solve_enqueue(const BatchSolve& b, cudaStream_t s, cudaStream_t body) {
  if (b.init_ph.second > 0)
    k_batch_defect_init<<<b.init_ph.second, 32 * UR_WARPS, 0, s>>>(b.scenes, b.items + b.init_ph.first);
  cudaStreamCaptureStatus cst;
  cudaGraph_t cap = nullptr;
  cudaError_t err = cudaStreamGetCaptureInfo(s, &cst, nullptr, &cap, nullptr, nullptr, nullptr);
  cudaGraphConditionalHandle h = 0;
  if (err == cudaSuccess) err = cudaGraphConditionalHandleCreate(&h, cap, 0, cudaGraphCondAssignDefault);
  if (err != cudaSuccess) return err;
  k_batch_begin<<<1, 1024, 0, s>>>(b.plan, h);
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
  if (err == cudaSuccess)
    err = cudaStreamBeginCaptureToGraph(body, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal);
  if (err != cudaSuccess) return err;
  const int D = b.depth;
  for (int d = 0; d < D; d++) launch_batch_smooth<MODE_PRE>(body, b, b.pre, d);
  k_batch_tail<<<phase_grid(b, D, 1), dim3(32, 32), b.tail_smem, body>>>(b.plan, D);
  for (int d = 0; d < D; d++) launch_batch_smooth<MODE_POST>(body, b, b.post, D + 1 + d);
  if (b.max_items[2 * D + 1] > 0)
    k_batch_defect<<<phase_grid(b, 2 * D + 1, 8), 32 * UR_WARPS, 0, body>>>(b.plan, 2 * D + 1);
  k_batch_check<<<1, 1024, 0, body>>>(b.plan, h);
  cudaGraph_t done = nullptr;
  err = cudaStreamEndCapture(body, &done);
  if (err != cudaSuccess) return err;
  k_batch_zero<<<b.zero_ph.second, 256, 0, s>>>(b.scenes, b.items + b.zero_ph.first);
  return cudaGetLastError();
}

}  // namespace fl
