// Shared device-side definitions of the flowlab_gb300 engine.
//
// Numerics note: the library is compiled with -fmad=false and IEEE division /
// square root, and every formula below keeps the reference's operation order
// (src/core/*.ts), so each kernel performs the same float32 operations as the
// reference's arithmetic evaluated in float32.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fl {

// src/core/grid.ts:41-45
constexpr uint8_t FLUID = 0, AIR = 1, SOLID = 2;
constexpr int DYE_CHANNELS = 3;

// Per-cell stencil code, built once per label change: the label in bits 0-1
// and, for each neighbour in the pressure stencil's order, whether it is
// non-solid AND in the domain (the negation of grid.ts:159-161
// isSolidOrOutside). Cells outside the domain are coded SOLID with no links.
constexpr uint8_t LINK_XP = 1u << 2;  // (i+1, j)
constexpr uint8_t LINK_XM = 1u << 3;  // (i-1, j)
constexpr uint8_t LINK_YP = 1u << 4;  // (i, j+1)
constexpr uint8_t LINK_YM = 1u << 5;  // (i, j-1)
constexpr uint8_t CODE_OUTSIDE = SOLID;

__host__ __device__ inline uint8_t code_label(uint8_t c) { return c & 3u; }
// the number of links (bits 2..5)
__host__ __device__ inline int code_count(uint8_t c) {
#ifdef __CUDA_ARCH__
  return __popc((unsigned int)c & 0x3cu);
#else
  return ((c >> 2) & 1) + ((c >> 3) & 1) + ((c >> 4) & 1) + ((c >> 5) & 1);
#endif
}

// Scalars of one step, written on the device (from the CFL reduction) or by
// the host, and read by every kernel of the step through a pointer so that a
// captured graph needs no re-recording when dt changes.
struct StepScalars {
  float dt;          // simulation.ts:477
  float scale;       // rho*h^2/dt (simulation.ts:478)
  float grad_scale;  // dt/(rho*h) (simulation.ts:479)
  float keep[3];     // exp(-decay*dt) per channel (simulation.ts:243-247)
  float gain_beta;   // beta*dt (buoyancy.ts:80)
  float gain_alpha;  // -alpha*dt (soot term)
  float half_dt;     // 0.5*dt (confinement face average)
  float neg_scale;   // -scale: b = (-scale)*div (pressureMultigrid.ts:311)
  int pad[6];
};

// Double-precision accumulators of one step. The first four fields are
// cleared before every solve; the last four are managed by the kernels that
// use them (the CFL reduction clears its own running max and block counter).
struct StepAccum {
  double b_sq;                  // sum b^2 over fluid cells (fluidDivRms, pressure.ts:177-186)
  double res_sq;                // sum r^2 over fluid cells with links (pressure.ts:127-167)
  unsigned long long n_fluid;
  unsigned long long n_res;
  unsigned int max_speed_bits;  // running max |u|,|v| as float bits (non-negative floats order as ints)
  unsigned int blocks_done;     // last-block detection of the CFL reduction
  unsigned int last_max_bits;   // the finished max face speed, for the report
  unsigned int nonfinite;
  unsigned int test_done;       // last-block detection of the defect pass that runs the cycle test
  unsigned int pad0;
};

// The residual diagnostic (simulation.ts:539-540, SimulationParams.
// residualEvery): the post-step divergence of the projected velocity,
// recomputed on steps whose index is a multiple of residual_every, and its
// FLUID-cell statistics (viz/fieldView.ts:44-60).
struct DiagAccum {
  // sums of the step in progress (zeroed again once a step's are final)
  double div_sq;               // sum div^2 over fluid cells
  unsigned long long n_fluid;
  unsigned int div_max_bits;   // max |div| over fluid cells as float bits
  unsigned int blocks_done;    // last-block detection
  unsigned long long counter;  // steps finished since the engine was created
  // the last step that computed it
  double last_sq;
  unsigned long long last_n;
  long long last_step;         // its index (-1: none)
  unsigned int last_max_bits;
  int pad;
};

// Device-side state of one pressure solve, so that the cycle loop can run
// without the host: the begin/check kernels decide whether another cycle
// runs (a CUDA-graph WHILE condition, or a flag the host reads), count
// cycles, and keep the float64 pressure's buffer parity.
struct SolveCtl {
  double tol;        // relative-residual target (<= 0: run max_cycles)
  double b_rms;      // RMS of the rhs over fluid cells
  double rel;        // last relative residual (-1: not evaluated)
  int max_cycles;
  int mode;          // SOLVE_MG, SOLVE_MIXED, SOLVE_RB
  int cycles;        // cycles run in this solve
  int cont;          // 1: run another cycle
  int zero_p;        // the rhs vanished: p = 0 is the answer
  int nonfinite;     // a NaN/Inf showed up in the rhs or the residual
  int par;           // which float64 pressure buffer holds p
  int pad;
  double rel0;       // the relative residual of the warm start, before any cycle (-1: not evaluated)
};
constexpr int SOLVE_MG = 0, SOLVE_MIXED = 1, SOLVE_RB = 2;

// ------------------------------------------------------------ sampling

// A cell size with its reciprocal. When h is a power of two, x / h and
// x * (1/h) are the same float (both scale by an exact power of two), so the
// samplers multiply instead of dividing; otherwise they divide as the
// reference does.
struct Spacing {
  float h;
  float inv;
  int pow2;
};

__host__ inline Spacing make_spacing(float h) {
  int ex = 0;
  const float m = frexpf(h, &ex);
  Spacing s;
  s.h = h;
  s.inv = 1.0f / h;
  s.pow2 = (m == 0.5f) ? 1 : 0;
  return s;
}

__device__ __forceinline__ float over(float x, const Spacing& s) { return s.pow2 ? x * s.inv : x / s.h; }

struct AxisF {
  int i0;
  float f;
};

// min/max with the C++ standard library's semantics ((b < a) ? b : a), so
// that signed zeros and NaNs resolve exactly as in a host evaluation of the
// same formula.
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }

// grid.ts:173-177 clampedAxis: position clamped to [0, count-1], index to
// count-2.
__device__ __forceinline__ AxisF clamped_axis(float pos, int count) {
  float c = smin(smax(pos, 0.0f), (float)(count - 1));
  int i0 = min((int)floorf(c), count - 2);
  AxisF a;
  a.i0 = i0;
  a.f = c - (float)i0;
  return a;
}

// grid.ts:180-191
__device__ __forceinline__ float bilerp(float v00, float v10, float v01, float v11, float fx, float fy) {
  float lo = v00 + fx * (v10 - v00);
  float hi = v01 + fx * (v11 - v01);
  return lo + fy * (hi - lo);
}

__device__ __forceinline__ float ldg(const float* p) { return __ldg(p); }

// The samplers index with 32-bit offsets: a sampled field holds fewer than
// 2^31 values (the engine's grid and dye-grid limits guarantee it).

// grid.ts:197-208 sampleU: u[i,j] at (i*h, (j+0.5)*h), (nx+1) x ny values.
__device__ __forceinline__ float sample_u(const float* __restrict__ u, int nx, int ny, const Spacing& h, float x, float y) {
  AxisF a = clamped_axis(over(x, h), nx + 1);
  AxisF b = clamped_axis(over(y, h) - 0.5f, ny);
  const int s = nx + 1;
  const int k = a.i0 + b.i0 * s;
  return bilerp(ldg(u + k), ldg(u + k + 1), ldg(u + k + s), ldg(u + k + s + 1), a.f, b.f);
}

// grid.ts:214-225 sampleV: v[i,j] at ((i+0.5)*h, j*h), nx x (ny+1) values.
__device__ __forceinline__ float sample_v(const float* __restrict__ v, int nx, int ny, const Spacing& h, float x, float y) {
  AxisF a = clamped_axis(over(x, h) - 0.5f, nx);
  AxisF b = clamped_axis(over(y, h), ny + 1);
  const int s = nx;
  const int k = a.i0 + b.i0 * s;
  return bilerp(ldg(v + k), ldg(v + k + 1), ldg(v + k + s), ldg(v + k + s + 1), a.f, b.f);
}

// grid.ts:239-250 sampleP on a cell-centred field of nx x ny.
__device__ __forceinline__ float sample_p(const float* __restrict__ q, int nx, int ny, const Spacing& h, float x, float y) {
  AxisF a = clamped_axis(over(x, h) - 0.5f, nx);
  AxisF b = clamped_axis(over(y, h) - 0.5f, ny);
  const int s = nx;
  const int k = a.i0 + b.i0 * s;
  return bilerp(ldg(q + k), ldg(q + k + 1), ldg(q + k + s), ldg(q + k + s + 1), a.f, b.f);
}

// grid.ts:268-270
__device__ __forceinline__ float clamp_to_range(float q, float a, float b, float c, float d) {
  float lo = smin(smin(a, b), smin(c, d));
  float hi = smax(smax(a, b), smax(c, d));
  return smin(smax(q, lo), hi);
}

// grid.ts:273-315 clampToStencil{U,V,P}
__device__ __forceinline__ float clamp_stencil_u(const float* __restrict__ u, int nx, int ny, const Spacing& h, float x, float y,
                                                 float q) {
  int i0 = clamped_axis(over(x, h), nx + 1).i0;
  int j0 = clamped_axis(over(y, h) - 0.5f, ny).i0;
  const int s = nx + 1;
  const int k = i0 + j0 * s;
  return clamp_to_range(q, ldg(u + k), ldg(u + k + 1), ldg(u + k + s), ldg(u + k + s + 1));
}
__device__ __forceinline__ float clamp_stencil_v(const float* __restrict__ v, int nx, int ny, const Spacing& h, float x, float y,
                                                 float q) {
  int i0 = clamped_axis(over(x, h) - 0.5f, nx).i0;
  int j0 = clamped_axis(over(y, h), ny + 1).i0;
  const int s = nx;
  const int k = i0 + j0 * s;
  return clamp_to_range(q, ldg(v + k), ldg(v + k + 1), ldg(v + k + s), ldg(v + k + s + 1));
}
__device__ __forceinline__ float clamp_stencil_p(const float* __restrict__ q, int nx, int ny, const Spacing& h, float x, float y,
                                                 float val) {
  int i0 = clamped_axis(over(x, h) - 0.5f, nx).i0;
  int j0 = clamped_axis(over(y, h) - 0.5f, ny).i0;
  const int s = nx;
  const int k = i0 + j0 * s;
  return clamp_to_range(val, ldg(q + k), ldg(q + k + 1), ldg(q + k + s), ldg(q + k + s + 1));
}

// grid.ts:159-161 isSolidOrOutside on the velocity grid's labels.
__device__ __forceinline__ bool solid_or_outside(const uint8_t* __restrict__ label, int nx, int ny, int i, int j) {
  return (unsigned)i >= (unsigned)nx || (unsigned)j >= (unsigned)ny || __ldg(label + i + j * nx) == SOLID;
}
// boundaries.ts:23-25 isSolidCell
__device__ __forceinline__ bool solid_cell(const uint8_t* __restrict__ label, int nx, int ny, int i, int j) {
  return (unsigned)i < (unsigned)nx && (unsigned)j < (unsigned)ny && __ldg(label + i + j * nx) == SOLID;
}

// Block-wide reductions (thread count a multiple of 32, <= 1024); the result
// is valid in the block's first thread.
__device__ inline double block_sum(double v, double* shm32) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  int lane = tid & 31, w = tid >> 5;
  __syncthreads();
  if (lane == 0) shm32[w] = v;
  __syncthreads();
  double t = 0;
  if (w == 0) {
    int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
    t = lane < nw ? shm32[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;  // valid in thread 0
}

__device__ inline unsigned long long block_sum_u64(unsigned long long v, unsigned long long* shm32) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  int lane = tid & 31, w = tid >> 5;
  __syncthreads();
  if (lane == 0) shm32[w] = v;
  __syncthreads();
  unsigned long long t = 0;
  if (w == 0) {
    int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
    t = lane < nw ? shm32[lane] : 0ull;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;
}

__device__ inline float block_max(float v, float* shm32) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  int lane = tid & 31, w = tid >> 5;
  __syncthreads();
  if (lane == 0) shm32[w] = v;
  __syncthreads();
  float t = 0.0f;
  if (w == 0) {
    int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
    t = lane < nw ? shm32[lane] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_down_sync(0xffffffffu, t, o));
  }
  return t;
}

// Bit casts opaque to the compiler's optimiser: through the plain
// intrinsics it recognises sign-bit masks and flips on a double's bits as
// fabs / fneg / compares and emits them as float64 instructions, the very
// pipe these helpers exist to avoid.
__device__ __forceinline__ unsigned long long dbits_opaque(double x) {
  unsigned long long u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  return u;
}
__device__ __forceinline__ double dfrom_opaque(unsigned long long u) {
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(u));
  return x;
}

// The rare cases of the integer helpers below, out of line: inlined, the
// compiler predicates these instructions into the common path, where they
// would occupy GB300's slow float64 pipe on every call.
static __device__ __noinline__ double f2d_slow(float f) { return (double)f; }
static __device__ __noinline__ double dmul_slow(double x, double y) { return x * y; }
static __device__ __noinline__ float d2f_slow(double d) { return (float)d; }

// Exact float -> double by bit manipulation (integer pipe) for zero and
// normal floats; subnormals, infinities and NaN take the conversion
// instruction. The result equals (double)f in every case.
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  if (ex != 0u && ex != 0xffu) {
    const unsigned long long bits =
        sign | ((unsigned long long)(ex + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
    return dfrom_opaque(bits);
  }
  if ((u & 0x7fffffffu) == 0u) return dfrom_opaque(sign);
  return f2d_slow(f);
}

// x * 2^k (k = 1, 2) by an exponent increment when x is normal and the
// product stays normal; zero returns itself (as x * 2^k does); otherwise
// the multiply. Equal to x * 2^k in every case.
__device__ __forceinline__ double scale_pow2(double x, int k) {
  const long long bits = (long long)dbits_opaque(x);
  const long long ex = (bits >> 52) & 0x7ff;
  if (ex != 0 && ex < 0x7ff - k) return dfrom_opaque((unsigned long long)(bits + ((long long)k << 52)));
  if ((bits & 0x7fffffffffffffffll) == 0) return x;
  return dmul_slow(x, (double)(1 << k));
}

// Double -> float rounded to nearest even by integer operations when the
// result is a normal float (a round-up that carries into the next binade,
// or past the largest float to infinity, falls out of the addition); other
// cases (results that are zero or subnormal, overflowing exponents, NaN)
// take the conversion instruction. Equal to (float)d in every case.
__device__ __forceinline__ float d2f_rn(double d) {
  const unsigned long long b = dbits_opaque(d);
  const unsigned ex = (unsigned)(b >> 52) & 0x7ffu;
  if (ex >= 897u && ex <= 1150u) {  // float biased exponent 1..254
    const unsigned long long m = b & 0xfffffffffffffull;
    const unsigned long long rem = m & 0x1fffffffull;  // the 29 bits rounded away
    unsigned long long f = ((unsigned long long)(ex - 896u) << 23) | (m >> 29);
    f += (rem > 0x10000000ull || (rem == 0x10000000ull && (f & 1ull))) ? 1ull : 0ull;
    return __uint_as_float((unsigned)(b >> 63) << 31 | (unsigned)f);
  }
  return d2f_slow(d);
}

// ------------------------------------------------------ double-float pairs
//
// The double-float pressure of the defect correction (fl_params.mixed = 2):
// a value is the unevaluated sum hi + lo of two floats (float2 x = hi,
// y = lo; ~48 significand bits) and lives in the same 8-byte-per-cell
// buffers as the float64 pressure. The arithmetic is error-free float
// transformations on the float32 pipe: TwoSum (Knuth, TAOCP vol. 2, 4.2.2),
// FastTwoSum and Dekker's double-length addition (Numer. Math. 18, 1971),
// and the product by 3 through one exact FMA. Each helper is a fixed
// sequence of IEEE float operations (explicit _rn intrinsics: never
// contracted or reordered), so results are reproducible bit for bit.
__device__ __forceinline__ float2 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return make_float2(s, e);
}
// exact when |a| >= |b| or a == 0
__device__ __forceinline__ float2 df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return make_float2(s, e);
}
__device__ __forceinline__ float2 df_add(float2 x, float2 y) {
  const float2 s = df_two_sum(x.x, y.x);
  const float e = __fadd_rn(s.y, __fadd_rn(x.y, y.y));
  return df_fast_two_sum(s.x, e);
}
__device__ __forceinline__ float2 df_neg(float2 x) { return make_float2(-x.x, -x.y); }
__device__ __forceinline__ float2 df_add_f(float2 x, float f) {
  const float2 s = df_two_sum(x.x, f);
  const float e = __fadd_rn(s.y, x.y);
  return df_fast_two_sum(s.x, e);
}
// count * x for a link count 1..4 (2 and 4 scale exactly)
__device__ __forceinline__ float2 df_mul_count(float2 x, int count) {
  if (count == 4) return make_float2(__fmul_rn(4.0f, x.x), __fmul_rn(4.0f, x.y));
  if (count == 2) return make_float2(__fmul_rn(2.0f, x.x), __fmul_rn(2.0f, x.y));
  if (count == 1) return x;
  const float p = __fmul_rn(3.0f, x.x);
  float e = __fmaf_rn(3.0f, x.x, -p);
  e = __fmaf_rn(3.0f, x.y, e);
  return df_fast_two_sum(p, e);
}
__device__ __forceinline__ float df_round(float2 x) { return __fadd_rn(x.x, x.y); }
// a - b rounded to one float
__device__ __forceinline__ float df_diff(float2 a, float2 b) {
  const float2 s = df_two_sum(a.x, -b.x);
  const float e = __fadd_rn(s.y, __fsub_rn(a.y, b.y));
  return __fadd_rn(s.x, e);
}
__device__ __forceinline__ double df_to_double(float2 x) { return (double)x.x + (double)x.y; }

// Block-wide sum of double-float pairs on the float32 pipe (one df_add per
// shuffle step), widened to double once, in the block's first thread: the
// float64 pipe issues ~1.6 lanes per clock per SM, so a double-precision
// tree over every block costs more than the sums it reduces.
__device__ inline double block_sum_df(float2 v, float2* shm32) {
  for (int o = 16; o > 0; o >>= 1)
    v = df_add(v, make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o)));
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int lane = tid & 31, w = tid >> 5;
  __syncthreads();
  if (lane == 0) shm32[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
    float2 u = lane < nw ? shm32[lane] : make_float2(0.0f, 0.0f);
    for (int o = 16; o > 0; o >>= 1)
      u = df_add(u, make_float2(__shfl_down_sync(0xffffffffu, u.x, o), __shfl_down_sync(0xffffffffu, u.y, o)));
    t = df_to_double(u);
  }
  return t;  // valid in thread 0
}
__device__ __forceinline__ float2 df_from_double(double d) {
  const float hi = (float)d;
  return make_float2(hi, (float)(d - (double)hi));
}

// 0.0 + x: x itself except that -0.0 becomes +0.0.
__device__ __forceinline__ double zero_plus(double x) {
  const unsigned long long bits = dbits_opaque(x);
  return bits == 0x8000000000000000ull ? 0.0 : x;
}

}  // namespace fl
