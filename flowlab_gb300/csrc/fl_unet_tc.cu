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
// for what it issued, frees its TMEM and returns. Two bounds: the waits that
// gate progress (a ring slot freed, a tile's data landed, an accumulator
// ready) give up after g_tc_wait_limit polls, a runtime value
// (fl_unet_set_wait_limit); the waits that drain what the CTA itself issued
// (its last copies, its MMAs' final commit) always allow WAIT_LIMIT polls,
// so that however early the progress waits give up, no copy or MMA is in
// flight when the TMEM is freed and the CTA ends.
#include <cstdint>

#include <cuda.h>  // CUtensorMap and its enums; the encoder is fetched through the runtime
#include <cudaTypedefs.h>

#include "fl_internal.h"
#include "fl_unet.h"

namespace fl {

namespace {

bool g_tc_on = true;
int g_tc_form = 1;  // 1: halo form where it applies, 0: always the chunked-gather form
int g_num_sms = 0;

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
__device__ long long g_tc_wait_limit = WAIT_LIMIT;

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
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit) {
  for (long long k = 0; k < limit; k++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// The drain bound (see the top of this file).
__device__ __forceinline__ bool mbar_drain(uint32_t bar, uint32_t parity) { return mbar_wait(bar, parity, WAIT_LIMIT); }

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

// 16 consecutive float32 columns of this thread's TMEM lane, without the
// wait (tmem_wait_ld completes every load issued before it).
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, float* v) {
  uint32_t* r = reinterpret_cast<uint32_t*>(v);
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

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
  const long long lim = g_tc_wait_limit;

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
      if (!mbar_wait(smem_u32(&bars[buf]), (uint32_t)(((it - 2) >> 1) & 1), lim)) failed = true;
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
    if (!mbar_drain(smem_u32(&bars[last & 1]), (uint32_t)((last >> 1) & 1))) failed = true;
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

// ---------------------------------------------------------------- halo form
//
// The main forward form. A tile is TR image rows x 128 columns of one image
// (TR accumulators of 128 pixels x N channels in TMEM). Per chunk of 32
// input channels the tile's (TR+2) x 130 pixel halo is loaded once, with
// four TMA tensor loads (one per 8-channel group; zero fill outside the
// image), into four "planes" [halo row][halo column][8 channels] of 16-byte
// rows, and the chunk's weights for all 9 taps with one bulk copy of a
// pre-arranged weight image. In a plane the pixels sit 16 bytes apart,
// which is the no-swizzle K-major layout with its 8-row groups 128 bytes
// apart; so the A operand of tap (ky, kx) for output row r is the same halo
// with the descriptor's start moved by ((r + ky) * 130 + kx) * 16 bytes. No
// tap is re-gathered: per chunk the tensor core runs 9 x TR x 2 MMAs
// (128 x N x 16) from one copy of the halo.
//
// The kernel is persistent and warp-specialised: one CTA per SM walks the
// tiles blockIdx.x, blockIdx.x + gridDim.x, ... Warp 0 (one lane) streams
// every tile's chunks through a 2-stage ring (waiting on a stage's "empty"
// barrier, which the MMAs' commit arrives on); warp 1 (one lane) issues the
// MMAs once a stage's "full" barrier (transaction bytes) completes, into one
// of two TMEM accumulator sets (tile i uses set i & 1), and commits
// "accumulator full"; warps 2-9 run the epilogue (bias, ReLU, bf16 NHWC) of
// tile i while the tensor core fills the other set with tile i+1, and
// release the set ("accumulator empty", one arrive per warp). Epilogue warp
// w reads TMEM lanes 32 (w % 4) .. +31, the lane quarter its rank in the
// warpgroup may access; the two warps of a quarter take alternate rows.
// Every wait is bounded; before the CTA ends every copy it issued has
// landed and every MMA has completed.
constexpr int HALO_TW = 128;            // output columns per tile (the MMA's M)
constexpr int HALO_W = HALO_TW + 2;     // halo columns
constexpr int HALO_SMEM_MAX = 227 * 1024;

__host__ __device__ constexpr int halo_plane_bytes(int tr) { return ((tr + 2) * HALO_W * 16 + 127) / 128 * 128; }
__host__ __device__ constexpr int halo_stage_bytes(int tr, int n) { return 4 * halo_plane_bytes(tr) + 9 * n * 64; }

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// Where the halo kernel's results go. Forward: y = bf16(relu(acc + bias)).
// Data gradient (yf set): yf = acc, zeroed where mask <= 0 (the ReLU of the
// layer's input; mask optional). Rows of y / yf / mask are ldy elements apart
// (the caller offsets the pointers to an output-channel tile).
struct HaloOut {
  __nv_bfloat16* y;
  float* yf;
  const __nv_bfloat16* mask;
  const float* bias;
  int ldy;
};

constexpr int WS_EPI_WARPS = 8;
constexpr int WS_THREADS = 64 + 32 * WS_EPI_WARPS;

__global__ void __launch_bounds__(WS_THREADS) k_conv3_halo_ws(const __grid_constant__ CUtensorMap xmap, int H,
                                                              int W, int B, const __nv_bfloat16* __restrict__ wimg,
                                                              int N, int nchunks, int TR, int ns, int ncols,
                                                              int stacked, HaloOut out) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int plane = halo_plane_bytes(TR);
  const int stage_a = 4 * plane;
  const int stage_b = 9 * N * 64;
  const int stage_bytes = stage_a + stage_b;
  const uint32_t tx_bytes = (uint32_t)(4 * (TR + 2) * HALO_W * 16 + stage_b);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + 2 * stage_bytes);
  uint64_t* empty = full + 2;
  uint64_t* accf = empty + 2;
  uint64_t* acce = accf + 2;
  uint64_t* done = acce + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_x = (W + HALO_TW - 1) / HALO_TW, tiles_y = (H + TR - 1) / TR;
  const int ntiles = tiles_x * tiles_y * B;
  const int acc_cols = TR * ns;  // one accumulator set

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 32) {
    for (int q = 0; q < 2; q++) {
      mbar_init(smem_u32(&full[q]), 1);
      mbar_init(smem_u32(&empty[q]), 1);
      mbar_init(smem_u32(&accf[q]), 1);
      mbar_init(smem_u32(&acce[q]), WS_EPI_WARPS);
    }
    mbar_init(smem_u32(done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  bool failed = false;
  const long long lim = g_tc_wait_limit;

  if (warp == 0) {
    if (lane == 0) {
      // ---- copies: chunk q (over all of this CTA's tiles) into stage q & 1
      int q = 0;
      for (int t = blockIdx.x; t < ntiles && !failed; t += gridDim.x) {
        const int bx = t % tiles_x, by = (t / tiles_x) % tiles_y, img = t / (tiles_x * tiles_y);
        for (int c = 0; c < nchunks; c++, q++) {
          const int s = q & 1, use = q >> 1;
          if (use > 0 && !mbar_wait(smem_u32(&empty[s]), (uint32_t)((use - 1) & 1), lim)) {
            failed = true;
            break;
          }
          unsigned char* st = smem + s * stage_bytes;
          const uint32_t fb = smem_u32(&full[s]);
          mbar_expect_tx(fb, tx_bytes);
#pragma unroll
          for (int g = 0; g < 4; g++)
            tma_load_4d(smem_u32(st + g * plane), &xmap, c * 32 + 8 * g, bx * HALO_TW - 1, by * TR - 1, img, fb);
          bulk_load(smem_u32(st + stage_a), wimg + (long)c * 9 * 32 * N, (uint32_t)stage_b, fb);
        }
      }
      // nothing issued may still be landing when the CTA ends: the last
      // arming of each stage (chunks q-1 and q-2) has completed
      for (int k = 1; k <= 2 && k <= q; k++) {
        const int qq = q - k;
        if (!mbar_drain(smem_u32(&full[qq & 1]), (uint32_t)((qq >> 1) & 1))) failed = true;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMAs
      const uint32_t idesc = instr_desc(HALO_TW, N);
      const uint32_t lbo_b = (uint32_t)N * 16;
      int q = 0, i = 0;
      for (int t = blockIdx.x; t < ntiles && !failed; t += gridDim.x, i++) {
        const int a = i & 1, ause = i >> 1;
        if (ause > 0 && !mbar_wait(smem_u32(&acce[a]), (uint32_t)((ause - 1) & 1), lim)) {
          failed = true;
          break;
        }
        tc_fence_after();
        const uint32_t dacc = tmem + (uint32_t)(a * acc_cols);
        for (int c = 0; c < nchunks; c++, q++) {
          const int s = q & 1, use = q >> 1;
          if (!mbar_wait(smem_u32(&full[s]), (uint32_t)(use & 1), lim)) {
            failed = true;
            break;
          }
          tc_fence_after();
          const uint32_t a0 = smem_u32(smem + s * stage_bytes), b0 = a0 + (uint32_t)stage_a;
          if (stacked) {
            // B holds, per kx, the three ky taps' weights stacked along N;
            // halo row h (A shifted by kx) times it adds ky's part to output
            // row h - ky, whose slot is N (TR - 1 - r) columns in: the parts
            // of one MMA land in adjacent slots. Rows outside the tile are
            // not computed (lo..hi). The first MMA into each slot (chunk 0,
            // kx 0, the first k-step, ky 0) overwrites; the rest accumulate.
            const uint32_t lbo_s = (uint32_t)(3 * N) * 16;
            for (int h = 0; h < TR + 2; h++) {
              const int lo = h - (TR - 1) > 0 ? h - (TR - 1) : 0;
              const int hi = h < 2 ? h : 2;
              const uint32_t d_lo = dacc + (uint32_t)(N * (TR - 1 - (h - lo)));
              for (int kx = 0; kx < 3; kx++) {
                const uint32_t at = a0 + 16u * (uint32_t)(h * HALO_W + kx);
                const uint32_t bk = b0 + (uint32_t)(kx * 4 * 3 * N * 16);
#pragma unroll
                for (int kk = 0; kk < 2; kk++) {
                  const uint64_t ad = smem_desc(at + (uint32_t)(kk * 2 * plane), (uint32_t)plane, 128);
                  if (c == 0 && kx == 0 && kk == 0 && lo == 0) {
                    mma_bf16(d_lo, ad, smem_desc(bk, lbo_s, 128), instr_desc(HALO_TW, N), 0u);
                    if (hi >= 1)
                      mma_bf16(d_lo + (uint32_t)N, ad, smem_desc(bk + (uint32_t)N * 16, lbo_s, 128),
                               instr_desc(HALO_TW, hi * N), 1u);
                  } else {
                    const uint64_t bd = smem_desc(bk + kk * 2 * lbo_s + (uint32_t)(lo * N * 16), lbo_s, 128);
                    mma_bf16(d_lo, ad, bd, instr_desc(HALO_TW, (hi - lo + 1) * N), 1u);
                  }
                }
              }
            }
            mma_commit(smem_u32(&empty[s]));
            continue;
          }
          // accumulator-major: the tensor core runs consecutive MMAs into
          // one accumulator markedly faster than MMAs alternating between several
          for (int r = 0; r < TR; r++) {
            for (int tp = 0; tp < 9; tp++) {
              const int ky = tp / 3, kx = tp % 3;
              const uint32_t bt = b0 + (uint32_t)(tp * N * 64);
              const uint32_t at = a0 + 16u * (uint32_t)((r + ky) * HALO_W + kx);
#pragma unroll
              for (int kk = 0; kk < 2; kk++) {
                const uint64_t ad = smem_desc(at + (uint32_t)(kk * 2 * plane), (uint32_t)plane, 128);
                const uint64_t bd = smem_desc(bt + kk * 2 * lbo_b, lbo_b, 128);
                mma_bf16(dacc + (uint32_t)(r * ns), ad, bd, idesc, (c > 0 || tp > 0 || kk > 0) ? 1u : 0u);
              }
            }
          }
          mma_commit(smem_u32(&empty[s]));
        }
        if (failed) break;
        mma_commit(smem_u32(&accf[a]));
      }
      // arrives when every MMA issued above has completed
      mma_commit(smem_u32(done));
    }
  } else {
    // ---- epilogue: warps 2..9; TMEM lane quarter warp % 4, rows
    // (warp - 2) / 4, + 2, ...
    const int quarter = warp & 3, row0 = (warp - 2) >> 2;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    int i = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
      const int a = i & 1, ause = i >> 1;
      if (!mbar_wait(smem_u32(&accf[a]), (uint32_t)(ause & 1), lim)) {
        failed = true;
        break;
      }
      tc_fence_after();
      const int bx = t % tiles_x, by = (t / tiles_x) % tiles_y, img = t / (tiles_x * tiles_y);
      const int x = bx * HALO_TW + quarter * 32 + lane;
      for (int r = row0; r < TR; r += 2) {
        const int yy = by * TR + r;
        const bool ok = x < W && yy < H;
        const long pix = ((long)img * H + (ok ? yy : 0)) * W + (ok ? x : 0);
        for (int c0 = 0; c0 < N; c0 += 64) {
          // up to four 16-column loads in flight, one wait
          float v[64];
          const int nc = N - c0 < 64 ? (N - c0) / 16 : 4;
          const int slot = stacked ? N * (TR - 1 - r) : r * ns;
          const uint32_t ta = tmem + lane_base + (uint32_t)(a * acc_cols + slot + c0);
          tmem_ld16_nowait(ta, v);
          if (nc > 1) tmem_ld16_nowait(ta + 16, v + 16);
          if (nc > 2) tmem_ld16_nowait(ta + 32, v + 32);
          if (nc > 3) tmem_ld16_nowait(ta + 48, v + 48);
          tmem_wait_ld();
          if (ok && out.yf == nullptr) {
            __nv_bfloat16* dst = out.y + pix * out.ldy;
#pragma unroll
            for (int q = 0; q < 4; q++) {
              if (q < nc) {
                __align__(16) __nv_bfloat16 o[16];
#pragma unroll
                for (int k = 0; k < 16; k++)
                  o[k] = __float2bfloat16_rn(fmaxf(v[16 * q + k] + out.bias[c0 + 16 * q + k], 0.0f));
                reinterpret_cast<uint4*>(dst + c0 + 16 * q)[0] = reinterpret_cast<const uint4*>(o)[0];
                reinterpret_cast<uint4*>(dst + c0 + 16 * q)[1] = reinterpret_cast<const uint4*>(o)[1];
              }
            }
          } else if (ok) {
            float* dst = out.yf + pix * out.ldy;
            const __nv_bfloat16* m = out.mask != nullptr ? out.mask + pix * out.ldy : nullptr;
#pragma unroll
            for (int q = 0; q < 4; q++) {
              if (q < nc) {
                __align__(16) float o[16];
#pragma unroll
                for (int k = 0; k < 16; k++) {
                  const float g = v[16 * q + k];
                  o[k] = (m != nullptr && !(__bfloat162float(m[c0 + 16 * q + k]) > 0.0f)) ? 0.0f : g;
                }
#pragma unroll
                for (int k = 0; k < 4; k++)
                  reinterpret_cast<float4*>(dst + c0 + 16 * q)[k] = reinterpret_cast<const float4*>(o)[k];
              }
            }
          }
        }
      }
      // this warp's reads of the set are done (tcgen05.wait::ld above)
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&acce[a]));
    }
  }
  __syncwarp();
  if (!mbar_drain(smem_u32(done), 0u)) failed = true;
  failed = __syncthreads_or(failed) != 0;
  if (failed && tid == 0) atomicExch(&g_tc_error, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
  }
}

// Weight image of one layer for the halo form: per 32-channel chunk c, per
// tap t, per 8-channel group g, per output channel n, 8 channels:
// img[(((c * 9 + t) * 4 + g) * N + n) * 8 + j] = w[(n * 9 + t) * Cin + 32c + 8g + j]
// — the shared-memory B tiles of all 9 taps of a chunk, contiguous.
//
// Stacked (3 N <= 256): per chunk c, per kx, per group g, the three ky taps'
// rows stacked along N (row ky N + n), 8 channels:
// img[((((c * 3 + kx) * 4 + g) * 3 + ky) * N + n) * 8 + j] = w[(n * 9 + 3 ky + kx) * Cin + 32c + 8g + j]
__global__ void k_weight_image(const __nv_bfloat16* __restrict__ w, int Cin, int N, int stacked,
                               __nv_bfloat16* __restrict__ img) {
  const long total = 9L * Cin * N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int j = (int)(i & 7);
    long q = i >> 3;
    const int n = (int)(q % N);
    q /= N;
    int t, g, c;
    if (stacked) {
      const int ky = (int)(q % 3);
      q /= 3;
      g = (int)(q & 3);
      q >>= 2;
      const int kx = (int)(q % 3);
      c = (int)(q / 3);
      t = 3 * ky + kx;
    } else {
      g = (int)(q & 3);
      q >>= 2;
      t = (int)(q % 9);
      c = (int)(q / 9);
    }
    img[i] = w[((long)n * 9 + t) * Cin + 32 * c + 8 * g + j];
  }
}

// Layers whose three ky taps fit one MMA's N (<= 256) use the stacked form:
// an M = 128 MMA costs about the same tensor-core time for every N up to 128.
bool halo_stacked(int N) { return 3 * N <= 256; }

// ---------------------------------------------------------- weight gradient
//
// dW[n][tap][ci] = sum over pixels p of g[p][n] * x[p + off(tap)][ci] on the
// tensor cores: D[ci][n] += A[ci][p] B[n][p] with K = pixels. Both tensors
// are NHWC (channels innermost), so both operands are MN-major: a plane of
// 16-byte pixel rows per 8 channels, exactly the halo planes of the forward
// kernel (MN-major no-swizzle descriptors: LBO = 128 bytes between groups of
// 8 pixel rows, SBO = the plane stride between groups of 8 channels). A tile
// is 128 pixels of one image row: its g planes (4 x 8 output channels) and
// the x halo (3 rows x 130 pixels x up to 128 input channels) arrive by TMA;
// tap (ky, kx) reads the halo from row ky, column kx on, so one copy serves
// all 9 taps. A CTA owns 32 output channels x up to 128 input channels (M =
// 128; rows past Cin are computed from unused shared memory and dropped) and
// a range of tiles; its 9 tap accumulators (288 TMEM columns) are added to
// dW with atomics at the end. Warp 0 issues the copies (2-stage ring), warp 1
// the MMAs, warps 2-5 the epilogue; every wait is bounded.
constexpr int WG_TW = 128;                                           // pixels per tile
constexpr int WG_NB = 32;                                            // output channels per CTA (N)
constexpr int WG_CB = 128;                                           // input channels per CTA (M)
constexpr int WG_PL = ((3 * HALO_W * 16 + 127) / 128) * 128;         // x plane: 3 halo rows
constexpr int WG_A = (WG_CB / 8) * WG_PL;
constexpr int WG_GPL = WG_TW * 16;                                   // g plane
constexpr int WG_B = (WG_NB / 8) * WG_GPL;
constexpr int WG_STAGE = WG_A + WG_B;
constexpr int WG_SMEM = 2 * WG_STAGE + 128;
constexpr int WG_THREADS = 192;

__global__ void __launch_bounds__(WG_THREADS) k_conv3_wgrad_tc(const __grid_constant__ CUtensorMap xmap,
                                                               const __grid_constant__ CUtensorMap gmap, int H, int W,
                                                               int B, int Cin, int tiles_per_cta,
                                                               float* __restrict__ dw) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + 2 * WG_STAGE);
  uint64_t* empty = full + 2;
  uint64_t* done = empty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n0 = blockIdx.y * WG_NB, ci0 = blockIdx.z * WG_CB;
  const int cb = Cin - ci0 < WG_CB ? Cin - ci0 : WG_CB;  // input channels of this CTA (multiple of 8)
  const int tiles_x = (W + WG_TW - 1) / WG_TW;
  const long ntiles = (long)tiles_x * H * B;
  const long t0 = (long)blockIdx.x * tiles_per_cta;
  const long t1 = t0 + tiles_per_cta < ntiles ? t0 + tiles_per_cta : ntiles;
  const int mytiles = t1 > t0 ? (int)(t1 - t0) : 0;
  constexpr uint32_t NCOLS = 512;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 32) {
    for (int q = 0; q < 2; q++) {
      mbar_init(smem_u32(&full[q]), 1);
      mbar_init(smem_u32(&empty[q]), 1);
    }
    mbar_init(smem_u32(done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  bool failed = false;
  const long long lim = g_tc_wait_limit;

  if (warp == 0) {
    if (lane == 0) {
      const uint32_t tx = (uint32_t)((cb / 8) * 3 * HALO_W * 16 + (WG_NB / 8) * WG_TW * 16);
      int q = 0;
      for (; q < mytiles; q++) {
        const long t = t0 + q;
        const int bx = (int)(t % tiles_x), y = (int)((t / tiles_x) % H), img = (int)(t / ((long)tiles_x * H));
        const int s = q & 1, use = q >> 1;
        if (use > 0 && !mbar_wait(smem_u32(&empty[s]), (uint32_t)((use - 1) & 1), lim)) {
          failed = true;
          break;
        }
        unsigned char* st = smem + s * WG_STAGE;
        const uint32_t fb = smem_u32(&full[s]);
        mbar_expect_tx(fb, tx);
        for (int g = 0; g < cb / 8; g++)
          tma_load_4d(smem_u32(st + g * WG_PL), &xmap, ci0 + 8 * g, bx * WG_TW - 1, y - 1, img, fb);
        for (int g = 0; g < WG_NB / 8; g++)
          tma_load_4d(smem_u32(st + WG_A + g * WG_GPL), &gmap, n0 + 8 * g, bx * WG_TW, y, img, fb);
      }
      for (int k = 1; k <= 2 && k <= q; k++) {
        const int qq = q - k;
        if (!mbar_drain(smem_u32(&full[qq & 1]), (uint32_t)((qq >> 1) & 1))) failed = true;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // M = 128, N = 32, both operands MN-major (bits 15 and 16)
      const uint32_t idesc = instr_desc(WG_CB, WG_NB) | (1u << 15) | (1u << 16);
      for (int q = 0; q < mytiles; q++) {
        const int s = q & 1, use = q >> 1;
        if (!mbar_wait(smem_u32(&full[s]), (uint32_t)(use & 1), lim)) {
          failed = true;
          break;
        }
        tc_fence_after();
        const uint32_t a0 = smem_u32(smem + s * WG_STAGE), b0 = a0 + (uint32_t)WG_A;
        for (int tp = 0; tp < 9; tp++) {
          const int ky = tp / 3, kx = tp % 3;
          const uint32_t dacc = tmem + (uint32_t)(tp * WG_NB);
#pragma unroll
          for (int k = 0; k < WG_TW / 16; k++) {
            const uint64_t ad = smem_desc(a0 + 16u * (uint32_t)(ky * HALO_W + kx + 16 * k), 128, WG_PL);
            const uint64_t bd = smem_desc(b0 + 16u * (uint32_t)(16 * k), 128, WG_GPL);
            mma_bf16(dacc, ad, bd, idesc, (q > 0 || k > 0) ? 1u : 0u);
          }
        }
        mma_commit(smem_u32(&empty[s]));
      }
      mma_commit(smem_u32(done));
    }
  }
  __syncwarp();
  if (!mbar_drain(smem_u32(done), 0u)) failed = true;
  failed = __syncthreads_or(failed) != 0;
  tc_fence_after();
  if (failed) {
    if (tid == 0) atomicExch(&g_tc_error, 1);
  } else if (warp >= 2 && mytiles > 0) {
    // TMEM lane = input channel ci0 + lane index; column = tap * 32 + output channel
    const int quarter = warp & 3;
    const int ci = ci0 + quarter * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
    for (int tp = 0; tp < 9; tp++) {
      float v[32];
      tmem_ld16_nowait(lane_base + (uint32_t)(tp * WG_NB), v);
      tmem_ld16_nowait(lane_base + (uint32_t)(tp * WG_NB + 16), v + 16);
      tmem_wait_ld();
      if (quarter * 32 + lane < cb) {
#pragma unroll
        for (int j = 0; j < WG_NB; j++) atomicAdd(&dw[((long)(n0 + j) * 9 + tp) * Cin + ci], v[j]);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOLS) : "memory");
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

constexpr int WS_BAR_BYTES = 128;  // 9 barriers and the TMEM slot

// The persistent form's tile height: the tallest tile whose two stages fit
// one CTA per SM and whose two accumulator sets fit TMEM.
bool halo_ws_shape(int N, int* tr, int* ns, int* ncols) {
  int n_s = 32;
  while (n_s < N) n_s <<= 1;
  for (int t = 8; t >= 1; t >>= 1) {
    if (2 * t * n_s > 512) continue;
    if (2 * halo_stage_bytes(t, N) + WS_BAR_BYTES > HALO_SMEM_MAX) continue;
    int cols = 32;
    while (cols < 2 * t * n_s) cols <<= 1;
    *tr = t;
    *ns = n_s;
    *ncols = cols;
    return true;
  }
  return false;
}

bool g_attr_set = false;
bool g_halo_ok = false;

}  // namespace

// Opts the kernel into its dynamic shared memory; called when a network is
// created (outside any stream capture).
void unet_tc_setup() {
  g_attr_set = cudaFuncSetAttribute(k_conv3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) == cudaSuccess;
  g_halo_ok = cudaFuncSetAttribute(k_conv3_halo_ws, cudaFuncAttributeMaxDynamicSharedMemorySize, HALO_SMEM_MAX) ==
                  cudaSuccess &&
              cudaFuncSetAttribute(k_conv3_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, WG_SMEM) ==
                  cudaSuccess;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    g_num_sms = 0;
  g_halo_ok = g_halo_ok && g_num_sms > 0;
  if (!g_encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  g_halo_ok = g_halo_ok && g_encode != nullptr;
  cudaGetLastError();
}

void unet_tc_weight_image(cudaStream_t s, const __nv_bfloat16* w, int Cin, int Cout, __nv_bfloat16* img) {
  const long total = 9L * Cin * Cout;
  k_weight_image<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(w, Cin, Cout, halo_stacked(Cout) ? 1 : 0, img);
}

void unet_tc_enable(bool on) { g_tc_on = on; }
void unet_tc_form(int form) { g_tc_form = form; }
bool unet_tc_enabled() { return g_tc_on; }

namespace {

bool launch_halo(cudaStream_t s, const __nv_bfloat16* x, int B, int H, int W, int Cin, const __nv_bfloat16* wimg,
                 int N, const HaloOut& out) {
  int tr, ns, ncols;
  const int nchunks = Cin / KC;
  if (!halo_ws_shape(N, &tr, &ns, &ncols)) return false;
  // x as a 4-D tensor (channels, columns, rows, images), boxes of 8 channels
  // x 130 columns x (tr + 2) rows; outside the image the box reads zeros
  CUtensorMap map;
  const cuuint64_t dims[4] = {(cuuint64_t)Cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
  const cuuint64_t strides[3] = {(cuuint64_t)Cin * 2, (cuuint64_t)W * Cin * 2, (cuuint64_t)H * W * Cin * 2};
  const cuuint32_t box[4] = {8, (cuuint32_t)HALO_W, (cuuint32_t)(tr + 2), 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  if (g_encode(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(x), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  const int tiles_x = (W + HALO_TW - 1) / HALO_TW, tiles_y = (H + tr - 1) / tr;
  const long ntiles = (long)tiles_x * tiles_y * B;
  if (ntiles >= (1L << 31)) return false;
  const int grid = (int)(ntiles < g_num_sms ? ntiles : g_num_sms);
  const int smem = 2 * halo_stage_bytes(tr, N) + WS_BAR_BYTES;
  if (smem > HALO_SMEM_MAX) return false;
  k_conv3_halo_ws<<<grid, WS_THREADS, smem, s>>>(map, H, W, B, wimg, N, nchunks, tr, ns, ncols,
                                                  halo_stacked(N) ? 1 : 0, out);
  return true;
}

}  // namespace

bool unet_tc_conv_dgrad(cudaStream_t s, const __nv_bfloat16* g, int B, int H, int W, int Cin, const __nv_bfloat16* wimg,
                        int N, float* gx, int ldg, const __nv_bfloat16* mask) {
  if (!g_tc_on || g_tc_form == 0 || !g_halo_ok) return false;
  if (Cin % KC != 0 || N % 16 != 0 || N < 16 || N > 128 || ldg % 4 != 0) return false;
  if ((reinterpret_cast<uintptr_t>(g) | reinterpret_cast<uintptr_t>(wimg)) & 15) return false;
  if (reinterpret_cast<uintptr_t>(gx) & 15) return false;
  const HaloOut out{nullptr, gx, mask, nullptr, ldg};
  return launch_halo(s, g, B, H, W, Cin, wimg, N, out);
}

bool unet_tc_conv_wgrad(cudaStream_t s, const __nv_bfloat16* x, const __nv_bfloat16* g, int B, int H, int W, int Cin,
                        int Cout, float* dw) {
  if (!g_tc_on || g_tc_form == 0 || !g_halo_ok) return false;
  if (Cin % 32 != 0 || Cout % WG_NB != 0) return false;
  if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(g)) & 15) return false;
  CUtensorMap xmap, gmap;
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  {
    const cuuint64_t dims[4] = {(cuuint64_t)Cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)Cin * 2, (cuuint64_t)W * Cin * 2, (cuuint64_t)H * W * Cin * 2};
    const cuuint32_t box[4] = {8, (cuuint32_t)HALO_W, 3, 1};
    if (g_encode(&xmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(x), dims, strides, box, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  {
    const cuuint64_t dims[4] = {(cuuint64_t)Cout, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)Cout * 2, (cuuint64_t)W * Cout * 2, (cuuint64_t)H * W * Cout * 2};
    const cuuint32_t box[4] = {8, (cuuint32_t)WG_TW, 1, 1};
    if (g_encode(&gmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(g), dims, strides, box, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  const int nblk = Cout / WG_NB, cblk = (Cin + WG_CB - 1) / WG_CB;
  const long ntiles = (long)((W + WG_TW - 1) / WG_TW) * H * B;
  long ctas = (g_num_sms + nblk * cblk - 1) / (nblk * cblk);
  if (ctas > ntiles) ctas = ntiles;
  if (ctas < 1) ctas = 1;
  const long per = (ntiles + ctas - 1) / ctas;
  ctas = (ntiles + per - 1) / per;
  if (per >= (1L << 30) || ctas >= 65535) return false;
  dim3 grid((unsigned)ctas, (unsigned)nblk, (unsigned)cblk);
  k_conv3_wgrad_tc<<<grid, WG_THREADS, WG_SMEM, s>>>(xmap, gmap, H, W, B, Cin, (int)per, dw);
  return true;
}

// Polls a progress wait allows before it gives up (<= 0: the default,
// WAIT_LIMIT); on the current device.
int unet_tc_set_wait_limit(long long polls) {
  const long long v = polls > 0 ? polls : WAIT_LIMIT;
  return cudaMemcpyToSymbol(g_tc_wait_limit, &v, sizeof v) == cudaSuccess ? 0 : -1;
}

int unet_tc_take_error() {
  int v = 0, z = 0;
  cudaMemcpyFromSymbol(&v, g_tc_error, sizeof v);
  cudaMemcpyToSymbol(g_tc_error, &z, sizeof z);
  return v;
}

bool unet_tc_conv_fwd(cudaStream_t s, const __nv_bfloat16* x, int B, int H, int W, int Cin, const __nv_bfloat16* w,
                      const __nv_bfloat16* wimg, const float* bias, int Cout, __nv_bfloat16* y) {
  if (!g_tc_on) return false;
  if (Cin % KC != 0 || Cout % 16 != 0 || Cout < 16 || Cout > 128) return false;
  // 16-byte aligned rows of x, w and y
  if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(w) | reinterpret_cast<uintptr_t>(y) |
       reinterpret_cast<uintptr_t>(wimg)) & 15)
    return false;
  if (g_tc_form != 0 && g_halo_ok) {
    const HaloOut out{y, nullptr, nullptr, bias, Cout};
    if (launch_halo(s, x, B, H, W, Cin, wimg, Cout, out)) return true;
  }
  if (!g_attr_set) return false;  // unet_tc_setup not called on this device
  int ncols = 32;
  while (ncols < Cout) ncols <<= 1;
  const long HW = (long)H * W;
  dim3 grid((unsigned)((HW + TM - 1) / TM), (unsigned)B);
  k_conv3_tc<<<grid, 128, SMEM_BYTES, s>>>(x, H, W, Cin, w, bias, Cout, ncols, y);
  return true;
}

}  // namespace fl
