// Tensor-core forward convolution of the warm-start U-Net on sm_103a:
// tcgen05.mma (kind::f16, bf16 operands, float32 accumulator in TMEM).
//
// Implicit GEMM: M = 128 consecutive pixels of one image (a CTA), N = all
// output channels (16..128, multiple of 16), K = 9 taps x input channels
// (a multiple of 32) in chunks of 32 channels of one tap. Each chunk's A
// tile (128 pixels x 32 channels, gathered from the shifted input with zero
// padding) and B tile (N x 32 channels of that tap's weights) are written to
// shared memory by the CTA's 128 threads in the canonical no-swizzle
// K-major layout (8-row x 16-byte core matrices, contiguous 128 bytes),
// double-buffered: while the tensor core runs chunk i, the threads load
// chunk i+1. One elected thread issues two 128xNx16 MMAs per chunk and
// commits them to the chunk buffer's mbarrier. The epilogue reads the
// accumulator back with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31,
// i.e. pixels), adds the bias, applies ReLU and stores bf16 NHWC.
//
// Every wait is bounded: on timeout the kernel records the failure in a
// device word (read by unet_tc_take_error), stops issuing, waits (bounded)
// for what it issued, frees its TMEM and returns.
#include <cstdint>

#include "fl_internal.h"
#include "fl_unet.h"

namespace fl {

namespace {

bool g_tc_on = true;

constexpr int TM = 128;      // pixels per CTA (the MMA's M)
constexpr int KC = 32;       // input channels per chunk
constexpr int STAGE_A = TM * KC * 2;        // bytes
constexpr int STAGE_B_MAX = 128 * KC * 2;   // bytes, N <= 128
constexpr int SMEM_TILES = 2 * STAGE_A + 2 * STAGE_B_MAX;  // 32 KB
// every offset the descriptors reach lies inside the tiles (checked on the
// host for every N); the barriers and the TMEM slot follow
constexpr int SLACK = 0;
constexpr int SMEM_BYTES = SMEM_TILES + SLACK + 64;
constexpr long WAIT_LIMIT = 1L << 22;

__device__ int g_tc_error = 0;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: no swizzle, K-major; lbo = byte stride
// between core matrices adjacent in K, sbo = between core matrices adjacent
// in M (or N); version 1 (bits 46-47).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: D float32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long k = 0; k < WAIT_LIMIT; k++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 16 consecutive float32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}

// Byte offset of row r, 16-byte group g within a K-major no-swizzle tile
// of `rows` rows: core matrix (r/8, g) at (g * rows/8 + r/8) * 128.
__device__ __forceinline__ uint32_t tile_off(int r, int g, int rows) {
  return (uint32_t)((g * (rows >> 3) + (r >> 3)) * 128 + (r & 7) * 16);
}

__global__ void __launch_bounds__(128) k_conv3_tc(const __nv_bfloat16* __restrict__ x, int H, int W, int Cin,
                                                  const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias,
                                                  int N, int ncols, __nv_bfloat16* __restrict__ y) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* tiles = smem;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + SMEM_TILES + SLACK);  // 2 mbarriers
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + SMEM_TILES + SLACK + 16);
  const int tid = threadIdx.x, warp = tid >> 5;
  const long HW = (long)H * W;
  const long img = (long)blockIdx.y * HW;
  const long p0 = (long)blockIdx.x * TM;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(smem_u32(&bars[0]), 1);
    mbar_init(smem_u32(&bars[1]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  // this thread's output pixel (row of A)
  const long p = p0 + tid;
  const bool pix_ok = p < HW;
  const int py = pix_ok ? (int)(p / W) : 0, px = pix_ok ? (int)(p % W) : 0;

  const int cchunks = Cin / KC;
  const int niter = 9 * cchunks;
  const uint32_t idesc = instr_desc(TM, N);
  const uint32_t lbo_a = (TM / 8) * 128, lbo_b = (uint32_t)(N / 8) * 128;
  bool failed = false;
  int issued = 0;  // chunks committed

  // chunk loads go through registers one chunk ahead: the global (L2)
  // latency of chunk it+1 overlaps the barrier and MMA issue of chunk it
  uint4 ra[KC / 8], rb[4];
  auto load_chunk = [&](int it) {
    const int tap = it / cchunks, c0 = (it % cchunks) * KC;
    const int ky = tap / 3, kx = tap % 3;
    const int yy = py + ky - 1, xx = px + kx - 1;
    const bool ok = pix_ok && yy >= 0 && yy < H && xx >= 0 && xx < W;
    const uint4* src = reinterpret_cast<const uint4*>(x + (img + (long)(ok ? yy : 0) * W + (ok ? xx : 0)) * Cin + c0);
#pragma unroll
    for (int g = 0; g < KC / 8; g++) ra[g] = ok ? src[g] : make_uint4(0, 0, 0, 0);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int e = tid + 128 * q;
      const int n = e / (KC / 8), g = e % (KC / 8);
      rb[q] = n < N ? *reinterpret_cast<const uint4*>(w + ((long)n * 9 + tap) * Cin + c0 + 8 * g)
                    : make_uint4(0, 0, 0, 0);
    }
  };
  load_chunk(0);
  for (int it = 0; it < niter; it++) {
    const int buf = it & 1;
    unsigned char* A = tiles + buf * STAGE_A;
    unsigned char* B = tiles + 2 * STAGE_A + buf * STAGE_B_MAX;
    if (it >= 2) {
      // the MMAs of chunk it-2 read this buffer
      if (!mbar_wait(smem_u32(&bars[buf]), (uint32_t)(((it - 2) >> 1) & 1))) failed = true;
    }
    if (__syncthreads_or(failed)) {
      failed = true;
      break;
    }
#pragma unroll
    for (int g = 0; g < KC / 8; g++) *reinterpret_cast<uint4*>(A + tile_off(tid, g, TM)) = ra[g];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int e = tid + 128 * q;
      const int n = e / (KC / 8), g = e % (KC / 8);
      if (n < N) *reinterpret_cast<uint4*>(B + tile_off(n, g, N)) = rb[q];
    }
    if (it + 1 < niter) load_chunk(it + 1);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
#pragma unroll
      for (int kk = 0; kk < KC / 16; kk++) {
        const uint64_t ad = smem_desc(a0 + kk * 2 * lbo_a, lbo_a, 128);
        const uint64_t bd = smem_desc(b0 + kk * 2 * lbo_b, lbo_b, 128);
        mma_bf16(tmem, ad, bd, idesc, (it > 0 || kk > 0) ? 1u : 0u);
      }
      mma_commit(smem_u32(&bars[buf]));
    }
    issued = it + 1;
  }

  // wait for the last committed chunk (its commit covers all earlier MMAs);
  // also on failure, so that nothing is in flight when TMEM is freed
  if (issued > 0) {
    const int last = issued - 1;
    if (!mbar_wait(smem_u32(&bars[last & 1]), (uint32_t)((last >> 1) & 1))) failed = true;
  }
  failed = __syncthreads_or(failed) != 0;
  tc_fence_after();
  if (failed) {
    if (tid == 0) atomicExch(&g_tc_error, 1);
  } else {
    // tcgen05.ld is warp-collective: every lane loads, lanes with a pixel store
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    __nv_bfloat16* out = y + (img + (pix_ok ? p : 0)) * N;
    for (int c = 0; c < N; c += 16) {
      float v[16];
      tmem_ld16(lane_base + (uint32_t)c, v);
      if (pix_ok) {
        __align__(16) __nv_bfloat16 o[16];
#pragma unroll
        for (int k = 0; k < 16; k++) o[k] = __float2bfloat16_rn(fmaxf(v[k] + bias[c + k], 0.0f));
        reinterpret_cast<uint4*>(out + c)[0] = reinterpret_cast<const uint4*>(o)[0];
        reinterpret_cast<uint4*>(out + c)[1] = reinterpret_cast<const uint4*>(o)[1];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
  }
}

bool g_attr_set = false;

}  // namespace

// Opts the kernel into its dynamic shared memory; called when a network is
// created (outside any stream capture).
void unet_tc_setup() {
  g_attr_set = cudaFuncSetAttribute(k_conv3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) == cudaSuccess;
  cudaGetLastError();
}

void unet_tc_enable(bool on) { g_tc_on = on; }
bool unet_tc_enabled() { return g_tc_on; }

int unet_tc_take_error() {
  int v = 0, z = 0;
  cudaMemcpyFromSymbol(&v, g_tc_error, sizeof v);
  cudaMemcpyToSymbol(g_tc_error, &z, sizeof z);
  return v;
}

bool unet_tc_conv_fwd(cudaStream_t s, const __nv_bfloat16* x, int B, int H, int W, int Cin, const __nv_bfloat16* w,
                      const float* bias, int Cout, __nv_bfloat16* y) {
  if (!g_tc_on) return false;
  if (Cin % KC != 0 || Cout % 16 != 0 || Cout < 16 || Cout > 128) return false;
  // 16-byte aligned rows of x, w and y
  if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(w) | reinterpret_cast<uintptr_t>(y)) & 15)
    return false;
  if (!g_attr_set) return false;  // unet_tc_setup not called on this device
  int ncols = 32;
  while (ncols < Cout) ncols <<= 1;
  const long HW = (long)H * W;
  dim3 grid((unsigned)((HW + TM - 1) / TM), (unsigned)B);
  k_conv3_tc<<<grid, 128, SMEM_BYTES, s>>>(x, H, W, Cin, w, bias, Cout, ncols, y);
  return true;
}

}  // namespace fl
