// The pressure warm-start U-Net: forward, backward and Adam on the GPU.
//
// The reference's warm start is the previous step's pressure
// (src/core/pressureSolver.ts:28-30); this network (no reference
// counterpart) maps (b / s_b, fluid mask, p_prev / s_p) to a correction of
// p_prev: p_guess = p_prev + s_p * net(...) on fluid cells, after which the
// multigrid runs to the same tolerance as without it.
//
// Architecture: 4 levels of two 3x3 convolutions + ReLU each (32, 64, 96,
// 128 channels), 2x2 average pooling down, nearest upsampling up with the
// skip concatenated after the upsampled channels, a 1x1 head to one float
// channel. Activations are bfloat16 NHWC, weights bfloat16 copies of float32
// master weights ([cout][ky][kx][cin]), arithmetic and gradients float32.
//
// The 3x3 convolutions are implicit GEMMs: M = pixels, N = output channels,
// K = 9 taps x input channels. Forward and data-gradient convolutions run
// on the tensor cores (tcgen05, fl_unet_tc.cu) when the shapes allow it and
// on the CUDA cores otherwise (this file); both accumulate in float32.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "fl_internal.h"
#include "fl_unet.h"

namespace fl {

// ------------------------------------------------------------- layout

const UnetLayer kUnetLayers[UNET_LAYERS] = {
    {"enc0a", 3, 32, 3},    {"enc0b", 32, 32, 3},   {"enc1a", 32, 64, 3},   {"enc1b", 64, 64, 3},
    {"enc2a", 64, 96, 3},   {"enc2b", 96, 96, 3},   {"mida", 96, 128, 3},   {"midb", 128, 128, 3},
    {"dec2a", 224, 96, 3},  {"dec2b", 96, 96, 3},   {"dec1a", 160, 64, 3},  {"dec1b", 64, 64, 3},
    {"dec0a", 96, 32, 3},   {"dec0b", 32, 32, 3},   {"head", 32, 1, 1},
};

long long unet_num_params() {
  long long n = 0;
  for (const UnetLayer& L : kUnetLayers) n += (long long)L.cout * L.k * L.k * L.cin + L.cout;
  return n;
}

// ------------------------------------------------------------- kernels

namespace {

constexpr int CT = 16;    // pixel tile side of the CUDA-core convolutions
constexpr int CO_T = 32;  // output channels per block
constexpr int CK = 8;     // input channels per shared-memory chunk

__device__ __forceinline__ float ld(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ float ld(const float* p) { return *p; }

// 3x3 "same" convolution, zero padding, on the CUDA cores. EPI_ACT:
// y = bf16(relu(acc + bias)); EPI_GRAD: y = acc * (mask > 0) (float; mask
// optional) — the data gradient through the following ReLU.
enum { EPI_ACT = 0, EPI_GRAD = 1 };

template <typename TI, int EPI>
__global__ void __launch_bounds__(CT* CT) k_conv3(const TI* __restrict__ x, int H, int W, int Cin,
                                                   const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias,
                                                   int Cout, __nv_bfloat16* __restrict__ y_act, float* __restrict__ y_grad,
                                                   const __nv_bfloat16* __restrict__ mask) {
  __shared__ float xs[CK][CT + 2][CT + 3];
  __shared__ __align__(16) float ws[9][CK][CO_T];
  const int tx = threadIdx.x % CT, ty = threadIdx.x / CT;
  const int tiles_x = (W + CT - 1) / CT;
  const int X0 = (blockIdx.x % tiles_x) * CT, Y0 = (blockIdx.x / tiles_x) * CT;
  const int co_tiles = (Cout + CO_T - 1) / CO_T;
  const int b = blockIdx.y / co_tiles, co0 = (blockIdx.y % co_tiles) * CO_T;
  const long img = (long)b * H * W;
  float acc[CO_T];
#pragma unroll
  for (int c = 0; c < CO_T; c++) acc[c] = 0.0f;

  for (int c0 = 0; c0 < Cin; c0 += CK) {
    for (int e = threadIdx.x; e < CK * (CT + 2) * (CT + 2); e += CT * CT) {
      const int ci = e % CK, r = e / CK, lx = r % (CT + 2), ly = r / (CT + 2);
      const int gx = X0 + lx - 1, gy = Y0 + ly - 1;
      float v = 0.0f;
      if (c0 + ci < Cin && gx >= 0 && gy >= 0 && gx < W && gy < H) v = ld(x + (img + (long)gy * W + gx) * Cin + c0 + ci);
      xs[ci][ly][lx] = v;
    }
    for (int e = threadIdx.x; e < 9 * CK * CO_T; e += CT * CT) {
      const int co = e % CO_T, r = e / CO_T, ci = r % CK, tap = r / CK;
      float v = 0.0f;
      if (c0 + ci < Cin && co0 + co < Cout) v = __bfloat162float(w[((long)(co0 + co) * 9 + tap) * Cin + c0 + ci]);
      ws[tap][ci][co] = v;
    }
    __syncthreads();
#pragma unroll 1
    for (int tap = 0; tap < 9; tap++) {
      const int ky = tap / 3, kx = tap % 3;
#pragma unroll
      for (int ci = 0; ci < CK; ci++) {
        const float xv = xs[ci][ty + ky][tx + kx];
        const float4* wv = reinterpret_cast<const float4*>(ws[tap][ci]);
#pragma unroll
        for (int q = 0; q < CO_T / 4; q++) {
          const float4 f = wv[q];
          acc[4 * q + 0] = __fmaf_rn(xv, f.x, acc[4 * q + 0]);
          acc[4 * q + 1] = __fmaf_rn(xv, f.y, acc[4 * q + 1]);
          acc[4 * q + 2] = __fmaf_rn(xv, f.z, acc[4 * q + 2]);
          acc[4 * q + 3] = __fmaf_rn(xv, f.w, acc[4 * q + 3]);
        }
      }
    }
    __syncthreads();
  }
  const int gx = X0 + tx, gy = Y0 + ty;
  if (gx >= W || gy >= H) return;
  const long p = img + (long)gy * W + gx;
#pragma unroll
  for (int c = 0; c < CO_T; c++) {
    const int co = co0 + c;
    if (co >= Cout) break;
    if (EPI == EPI_ACT) {
      y_act[p * Cout + co] = __float2bfloat16_rn(fmaxf(acc[c] + bias[co], 0.0f));
    } else {
      float g = acc[c];
      if (mask != nullptr && !(__bfloat162float(mask[p * Cout + co]) > 0.0f)) g = 0.0f;
      y_grad[p * Cout + co] = g;
    }
  }
}

// The input layer (3 channels in, 32 out): 27 inputs per pixel held in
// registers, the 27 x 32 weights in shared memory read four output channels
// at a time; the generic kernel's 8-channel chunks would be 5/8 empty here.
__global__ void __launch_bounds__(CT* CT) k_conv3_in3(const __nv_bfloat16* __restrict__ x, int H, int W,
                                                       const __nv_bfloat16* __restrict__ w,
                                                       const float* __restrict__ bias, __nv_bfloat16* __restrict__ y) {
  constexpr int CI = 3, CO = 32;
  __shared__ float xs[CI][CT + 2][CT + 3];
  __shared__ __align__(16) float ws[9 * CI][CO];
  const int tx = threadIdx.x % CT, ty = threadIdx.x / CT;
  const int tiles_x = (W + CT - 1) / CT;
  const int X0 = (blockIdx.x % tiles_x) * CT, Y0 = (blockIdx.x / tiles_x) * CT;
  const long img = (long)blockIdx.y * H * W;
  for (int e = threadIdx.x; e < CI * (CT + 2) * (CT + 2); e += CT * CT) {
    const int ci = e % CI, r = e / CI, lx = r % (CT + 2), ly = r / (CT + 2);
    const int gx = X0 + lx - 1, gy = Y0 + ly - 1;
    float v = 0.0f;
    if (gx >= 0 && gy >= 0 && gx < W && gy < H) v = __bfloat162float(x[(img + (long)gy * W + gx) * CI + ci]);
    xs[ci][ly][lx] = v;
  }
  for (int e = threadIdx.x; e < 9 * CI * CO; e += CT * CT) {
    const int co = e % CO, k = e / CO;  // k = tap * CI + ci, the weights' [ky][kx][ci] order
    ws[k][co] = __bfloat162float(w[(long)co * 9 * CI + k]);
  }
  __syncthreads();
  float acc[CO];
#pragma unroll
  for (int c = 0; c < CO; c++) acc[c] = 0.0f;
#pragma unroll
  for (int tap = 0; tap < 9; tap++) {
#pragma unroll
    for (int ci = 0; ci < CI; ci++) {
      const float xv = xs[ci][ty + tap / 3][tx + tap % 3];
      const float4* wv = reinterpret_cast<const float4*>(ws[tap * CI + ci]);
#pragma unroll
      for (int q = 0; q < CO / 4; q++) {
        const float4 f = wv[q];
        acc[4 * q + 0] = __fmaf_rn(xv, f.x, acc[4 * q + 0]);
        acc[4 * q + 1] = __fmaf_rn(xv, f.y, acc[4 * q + 1]);
        acc[4 * q + 2] = __fmaf_rn(xv, f.z, acc[4 * q + 2]);
        acc[4 * q + 3] = __fmaf_rn(xv, f.w, acc[4 * q + 3]);
      }
    }
  }
  const int gx = X0 + tx, gy = Y0 + ty;
  if (gx >= W || gy >= H) return;
  __align__(16) __nv_bfloat16 o[CO];
#pragma unroll
  for (int c = 0; c < CO; c++) o[c] = __float2bfloat16_rn(fmaxf(acc[c] + bias[c], 0.0f));
  uint4* dst = reinterpret_cast<uint4*>(y + (img + (long)gy * W + gx) * CO);
#pragma unroll
  for (int q = 0; q < CO / 8; q++) dst[q] = reinterpret_cast<const uint4*>(o)[q];
}

// W'[ci][2-ky][2-kx][co] = W[co][ky][kx][ci]: the data gradient of a 3x3
// convolution is the convolution of the output gradient with W'.
__global__ void k_flip_weights(const __nv_bfloat16* __restrict__ w, int Cin, int Cout,
                               __nv_bfloat16* __restrict__ wt) {
  const long n = 9L * Cin * Cout;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const int ci = (int)(e % Cin);
    const long r = e / Cin;
    const int tap = (int)(r % 9), co = (int)(r / 9);
    wt[((long)ci * 9 + (8 - tap)) * Cout + co] = w[e];
  }
}

// dW[co][tap][ci] += sum over pixels of g[p][co] * x[p + off(tap)][ci];
// db[co] += sum of g[p][co]. A block covers CT x CT pixels of one image and
// a CO_T x CK slab of (co, ci) for all 9 taps.
__global__ void __launch_bounds__(256) k_conv3_wgrad(const __nv_bfloat16* __restrict__ x, const float* __restrict__ g,
                                                     int H, int W, int Cin, int Cout, float* __restrict__ dw,
                                                     float* __restrict__ db) {
  __shared__ float xs[CK][CT + 2][CT + 2];
  __shared__ float gs[CO_T][CT * CT + 1];
  const int tiles_x = (W + CT - 1) / CT;
  const int X0 = (blockIdx.x % tiles_x) * CT, Y0 = (blockIdx.x / tiles_x) * CT;
  const int co_tiles = (Cout + CO_T - 1) / CO_T, ci_tiles = (Cin + CK - 1) / CK;
  const int b = blockIdx.y / co_tiles, co0 = (blockIdx.y % co_tiles) * CO_T;
  const int c0 = blockIdx.z * CK;
  (void)ci_tiles;
  const long img = (long)b * H * W;
  for (int e = threadIdx.x; e < CK * (CT + 2) * (CT + 2); e += 256) {
    const int ci = e % CK, r = e / CK, lx = r % (CT + 2), ly = r / (CT + 2);
    const int gx = X0 + lx - 1, gy = Y0 + ly - 1;
    float v = 0.0f;
    if (c0 + ci < Cin && gx >= 0 && gy >= 0 && gx < W && gy < H)
      v = __bfloat162float(x[(img + (long)gy * W + gx) * Cin + c0 + ci]);
    xs[ci][ly][lx] = v;
  }
  for (int e = threadIdx.x; e < CO_T * CT * CT; e += 256) {
    const int co = e % CO_T, pix = e / CO_T, lx = pix % CT, ly = pix / CT;
    const int gx = X0 + lx, gy = Y0 + ly;
    float v = 0.0f;
    if (co0 + co < Cout && gx < W && gy < H) v = g[(img + (long)gy * W + gx) * Cout + co0 + co];
    gs[co][pix] = v;
  }
  __syncthreads();
  // 9 taps x CK x CO_T = 2304 sums over 256 pixels; 9 per thread
  for (int e = threadIdx.x; e < 9 * CK * CO_T; e += 256) {
    const int co = e % CO_T, r = e / CO_T, ci = r % CK, tap = r / CK;
    const int ky = tap / 3, kx = tap % 3;
    if (co0 + co >= Cout || c0 + ci >= Cin) continue;
    float s = 0.0f;
    for (int pix = 0; pix < CT * CT; pix++) s = __fmaf_rn(gs[co][pix], xs[ci][pix / CT + ky][pix % CT + kx], s);
    atomicAdd(&dw[((long)(co0 + co) * 9 + tap) * Cin + c0 + ci], s);
  }
  if (blockIdx.z == 0 && threadIdx.x < CO_T && co0 + threadIdx.x < Cout) {
    float s = 0.0f;
    for (int pix = 0; pix < CT * CT; pix++) s += gs[threadIdx.x][pix];
    atomicAdd(&db[co0 + threadIdx.x], s);
  }
}

// db[c] += sum over pixels of g[p][c]: thread t of a block handles channel
// t % C over every (blockDim / C)-th pixel of the block's share (coalesced
// rows); the block's partials meet in shared memory, one atomic per channel.
__global__ void __launch_bounds__(256) k_bias_grad(const float* __restrict__ g, long P, int C, float* __restrict__ db) {
  __shared__ float sdb[256];
  for (int c = threadIdx.x; c < C; c += blockDim.x) sdb[c] = 0.0f;
  __syncthreads();
  const int per = blockDim.x / C;  // pixels in flight per block
  if ((int)threadIdx.x < per * C) {
    const int c = threadIdx.x % C, j = threadIdx.x / C;
    float s = 0.0f;
    for (long p = (long)blockIdx.x * per + j; p < P; p += (long)gridDim.x * per) s += g[p * C + c];
    atomicAdd(&sdb[c], s);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) atomicAdd(&db[c], sdb[c]);
}

// 2x2 average pooling, bf16 -> bf16 (the mean in float32). One thread per
// coarse pixel and group of 8 channels (C is a multiple of 8).
__global__ void k_pool(const __nv_bfloat16* __restrict__ x, int B, int H, int W, int C, __nv_bfloat16* __restrict__ y) {
  const int h = H / 2, w = W / 2, cg = C / 8;
  const int n = B * h * w * cg;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int g = e % cg, q = e / cg;
    const int i = q % w, r = q / w, j = r % h, b = r / h;
    const long base = (((long)b * H + 2 * j) * W + 2 * i) * C + 8 * g;
    const uint4 v00 = *reinterpret_cast<const uint4*>(x + base);
    const uint4 v01 = *reinterpret_cast<const uint4*>(x + base + C);
    const uint4 v10 = *reinterpret_cast<const uint4*>(x + base + (long)W * C);
    const uint4 v11 = *reinterpret_cast<const uint4*>(x + base + (long)W * C + C);
    const __nv_bfloat16* a00 = reinterpret_cast<const __nv_bfloat16*>(&v00);
    const __nv_bfloat16* a01 = reinterpret_cast<const __nv_bfloat16*>(&v01);
    const __nv_bfloat16* a10 = reinterpret_cast<const __nv_bfloat16*>(&v10);
    const __nv_bfloat16* a11 = reinterpret_cast<const __nv_bfloat16*>(&v11);
    __align__(16) __nv_bfloat16 o[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const float s2 = (__bfloat162float(a00[k]) + __bfloat162float(a01[k])) +
                       (__bfloat162float(a10[k]) + __bfloat162float(a11[k]));
      o[k] = __float2bfloat16_rn(s2 * 0.25f);
    }
    *reinterpret_cast<uint4*>(y + (long)q * C + 8 * g) = *reinterpret_cast<const uint4*>(o);
  }
}

// c[p][0:Cu] = u[p/2] (nearest upsampling), c[p][Cu:Cu+Cs] = s[p]; one
// thread per pixel and group of 8 channels (Cu, Cs multiples of 8).
__global__ void k_up_concat(const __nv_bfloat16* __restrict__ u, int Cu, const __nv_bfloat16* __restrict__ s, int Cs,
                            int B, int H, int W, __nv_bfloat16* __restrict__ c) {
  const int C = Cu + Cs, cg = C / 8;
  const int n = B * H * W * cg;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int g = e % cg, p = e / cg;
    uint4 v;
    if (8 * g < Cu) {
      const int i = p % W, r = p / W, j = r % H, b = r / H;
      v = *reinterpret_cast<const uint4*>(u + (((long)b * (H / 2) + j / 2) * (W / 2) + i / 2) * Cu + 8 * g);
    } else {
      v = *reinterpret_cast<const uint4*>(s + (long)p * Cs + 8 * g - Cu);
    }
    *reinterpret_cast<uint4*>(c + (long)p * C + 8 * g) = v;
  }
}

// Backward of up_concat: g_u[q] = (sum of dc over q's 4 children, first Cu
// channels) * (act_u[q] > 0); skip[p] = dc[p][Cu:].
__global__ void k_up_split_bwd(const float* __restrict__ dc, int Cu, int Cs, int B, int H, int W,
                               const __nv_bfloat16* __restrict__ act_u, float* __restrict__ g_u,
                               float* __restrict__ skip) {
  const int C = Cu + Cs;
  const int h = H / 2, w = W / 2;
  const long nu = (long)B * h * w * Cu;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nu; e += (long)gridDim.x * blockDim.x) {
    const int ch = (int)(e % Cu);
    long r = e / Cu;
    const int i = (int)(r % w);
    r /= w;
    const int j = (int)(r % h), b = (int)(r / h);
    const long p = ((long)b * H + 2 * j) * W + 2 * i;
    const float s = (dc[p * C + ch] + dc[(p + 1) * C + ch]) + (dc[(p + W) * C + ch] + dc[(p + W + 1) * C + ch]);
    g_u[e] = __bfloat162float(act_u[e]) > 0.0f ? s : 0.0f;
  }
  const long ns = (long)B * H * W * Cs;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < ns; e += (long)gridDim.x * blockDim.x) {
    const int ch = (int)(e % Cs);
    const long p = e / Cs;
    skip[e] = dc[p * C + Cu + ch];
  }
}

// g_s[p] = (skip[p] + dpool[p/2] / 4) * (act_s[p] > 0): the gradient of a
// skip activation that also fed the pooling.
__global__ void k_pool_bwd_mask(const float* __restrict__ skip, const float* __restrict__ dpool, int B, int H, int W,
                                int C, const __nv_bfloat16* __restrict__ act, float* __restrict__ g) {
  const long n = (long)B * H * W * C;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const int c = (int)(e % C);
    const long p = e / C;
    const int i = (int)(p % W);
    const long r = p / W;
    const int j = (int)(r % H), b = (int)(r / H);
    const float d = skip[e] + 0.25f * dpool[(((long)b * (H / 2) + j / 2) * (W / 2) + i / 2) * C + c];
    g[e] = __bfloat162float(act[e]) > 0.0f ? d : 0.0f;
  }
}

// 1x1 head: out[p] = sum_c d0[p][c] * w[c] + b (C = 32: four 16-byte loads).
__global__ void k_head(const __nv_bfloat16* __restrict__ d0, int C, long P, const __nv_bfloat16* __restrict__ w,
                       const float* __restrict__ b, float* __restrict__ out) {
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
    float s2 = 0.0f;
    for (int c0 = 0; c0 < C; c0 += 8) {
      const uint4 v = *reinterpret_cast<const uint4*>(d0 + p * C + c0);
      const __nv_bfloat16* a = reinterpret_cast<const __nv_bfloat16*>(&v);
#pragma unroll
      for (int k = 0; k < 8; k++) s2 = __fmaf_rn(__bfloat162float(a[k]), __bfloat162float(w[c0 + k]), s2);
    }
    out[p] = s2 + b[0];
  }
}

// Head backward: g_d0[p][c] = dout[p] * w[c] * (d0[p][c] > 0); dw, db.
__global__ void __launch_bounds__(256) k_head_bwd(const __nv_bfloat16* __restrict__ d0, int C, long P,
                                                  const __nv_bfloat16* __restrict__ w, const float* __restrict__ dout,
                                                  float* __restrict__ g_d0, float* __restrict__ dw,
                                                  float* __restrict__ db) {
  // one item = one pixel's group of 8 channels (C a multiple of 8, <= 64):
  // 16-byte loads of d0, 32-byte stores of the gradient; a thread always
  // meets the same group (the grid stride is a multiple of C / 8), so its
  // weight-gradient partials are 8 registers, reduced in shared memory
  __shared__ float sw[64];
  __shared__ float sdb;
  const int G = C / 8;
  for (int c = threadIdx.x; c < C; c += blockDim.x) sw[c] = 0.0f;
  if (threadIdx.x == 0) sdb = 0.0f;
  __syncthreads();
  const long gid = blockIdx.x * (long)blockDim.x + threadIdx.x, stride = (long)gridDim.x * blockDim.x;
  const int q = (int)(gid % G);
  float wq[8], acc[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    wq[k] = __bfloat162float(w[8 * q + k]);
    acc[k] = 0.0f;
  }
  float ldb = 0.0f;
  for (long e = gid; e < P * G; e += stride) {
    const long p = e / G;
    const float d = dout[p];
    if (q == 0) ldb += d;
    const uint4 raw = *reinterpret_cast<const uint4*>(d0 + p * C + 8 * q);
    const __nv_bfloat16* a8 = reinterpret_cast<const __nv_bfloat16*>(&raw);
    __align__(16) float gout[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const float a = __bfloat162float(a8[k]);
      acc[k] = __fmaf_rn(d, a, acc[k]);
      gout[k] = a > 0.0f ? d * wq[k] : 0.0f;
    }
    float4* dst = reinterpret_cast<float4*>(g_d0 + p * C + 8 * q);
    dst[0] = reinterpret_cast<const float4*>(gout)[0];
    dst[1] = reinterpret_cast<const float4*>(gout)[1];
  }
#pragma unroll
  for (int k = 0; k < 8; k++) atomicAdd(&sw[8 * q + k], acc[k]);
  if (q == 0) atomicAdd(&sdb, ldb);
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) atomicAdd(&dw[c], sw[c]);
  if (threadIdx.x == 0) atomicAdd(db, sdb);
}

// Masked mean squared error: dout = 2 (out - t) m / n, loss += (out - t)^2 m.
__global__ void __launch_bounds__(256) k_mse(const float* __restrict__ out, const float* __restrict__ t,
                                             const float* __restrict__ m, long P, float inv_n,
                                             float* __restrict__ dout, double* __restrict__ loss) {
  __shared__ double red[32];
  double s = 0.0;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
    const float d = (out[p] - t[p]) * m[p];
    dout[p] = 2.0f * d * inv_n;
    s += (double)d * (double)d;
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0) atomicAdd(loss, s * (double)inv_n);
}

// Adam (Kingma & Ba 2015) on the float32 master weights, then their bf16
// copies; bias corrections c1 = 1 - b1^t, c2 = 1 - b2^t from the host.
__global__ void k_adam(float* __restrict__ th, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, long n, float lr, float b1, float b2, float c1, float c2, float eps,
                       __nv_bfloat16* __restrict__ th16) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const float gi = g[e];
    const float mi = b1 * m[e] + (1.0f - b1) * gi;
    const float vi = b2 * v[e] + (1.0f - b2) * gi * gi;
    m[e] = mi;
    v[e] = vi;
    const float t = th[e] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    th[e] = t;
    th16[e] = __float2bfloat16_rn(t);
  }
}

__global__ void k_to_bf16(const float* __restrict__ a, long n, __nv_bfloat16* __restrict__ b) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    b[e] = __float2bfloat16_rn(a[e]);
}

unsigned grid_for(long n, int threads = 256) {
  long b = (n + threads - 1) / threads;
  return (unsigned)std::max(1L, std::min(b, 152L * 16));
}

}  // namespace

// ------------------------------------------------------------- the network

int Unet::alloc(long max_pixels, std::string* err) {
  auto A = [&](void** p, size_t bytes, const char* what) {
    if (cudaMalloc(p, bytes) != cudaSuccess) {
      *err = std::string("allocation failed: ") + what;
      return false;
    }
    return true;
  };
  cap = max_pixels;
  nparam = unet_num_params();
  long off = 0;
  for (int l = 0; l < UNET_LAYERS; l++) {
    const UnetLayer& L = kUnetLayers[l];
    woff[l] = off;
    off += (long)L.cout * L.k * L.k * L.cin;
    boff[l] = off;
    off += L.cout;
  }
  bool ok = A((void**)&theta, nparam * 4, "weights") && A((void**)&m, nparam * 4, "adam m") &&
            A((void**)&v, nparam * 4, "adam v") && A((void**)&grad, nparam * 4, "gradient") &&
            A((void**)&theta16, nparam * 2, "bf16 weights") && A((void**)&wimg, nparam * 2, "weight images") &&
            A((void**)&wimg_flip, 9L * 224 * 96 * 2, "flipped weight image") &&
            A((void**)&gbf, max_pixels * 32L * 2, "bf16 gradient") && A((void**)&wflip, 9L * 224 * 96 * 2, "flipped weights") &&
            A((void**)&loss_dev, sizeof(double), "loss");
  if (!ok) return FL_ENOMEM;
  const long P = max_pixels;
  // activations (bf16): per level the largest channel count x pixels at that level
  const long sz[] = {P * 3, P * 32, P * 32, P / 4 * 32, P / 4 * 64, P / 4 * 64, P / 16 * 64, P / 16 * 96, P / 16 * 96,
                     P / 64 * 96, P / 64 * 128, P / 64 * 128, P / 16 * 224, P / 16 * 96, P / 16 * 96, P / 4 * 160,
                     P / 4 * 64, P / 4 * 64, P * 96, P * 32, P * 32};
  static_assert(sizeof(sz) / sizeof(sz[0]) == ACT_COUNT, "activation table");
  for (int k = 0; k < ACT_COUNT; k++) {
    act_size[k] = sz[k];
    if (!A((void**)&act[k], (size_t)sz[k] * 2, "activation")) return FL_ENOMEM;
  }
  // float32 gradient scratch: two buffers of the largest activation + skip grads
  const long gmax = P * 96;
  ok = A((void**)&gbuf[0], gmax * 4, "gradient scratch") && A((void**)&gbuf[1], gmax * 4, "gradient scratch") &&
       A((void**)&gskip[0], P * 32 * 4, "skip gradient") && A((void**)&gskip[1], P / 4 * 64 * 4, "skip gradient") &&
       A((void**)&gskip[2], P / 16 * 96 * 4, "skip gradient") && A((void**)&gpool, P / 4 * 64 * 4, "pool gradient") &&
       A((void**)&out, P * 4, "output") && A((void**)&dout, P * 4, "output gradient") &&
       A((void**)&target, P * 4, "target") && A((void**)&mask, P * 4, "mask") && A((void**)&input, P * 3 * 4, "input") &&
       A((void**)&ws_acc, 2 * sizeof(double), "warm-start sums");
  if (!ok) return FL_ENOMEM;
  cudaMemset(m, 0, nparam * 4);
  cudaMemset(v, 0, nparam * 4);
  return FL_OK;
}

void Unet::release() {
  void* ps[] = {theta, m, v, grad, theta16, wimg, wimg_flip, gbf, wflip, loss_dev, gbuf[0], gbuf[1], gskip[0], gskip[1], gskip[2], gpool,
                out, dout, target, mask, input, ws_acc};
  for (void* p : ps) cudaFree(p);
  for (auto* a : act) cudaFree(a);
}

void Unet::conv_fwd(cudaStream_t s, int l, const __nv_bfloat16* x, int B, int H, int W, __nv_bfloat16* y) {
  const UnetLayer& L = kUnetLayers[l];
  if (unet_tc_conv_fwd(s, x, B, H, W, L.cin, theta16 + woff[l], wimg + woff[l], theta + boff[l], L.cout, y)) return;
  if (L.cin == 3 && L.cout == 32 && L.k == 3) {
    dim3 g((unsigned)(((W + CT - 1) / CT) * ((H + CT - 1) / CT)), (unsigned)B);
    k_conv3_in3<<<g, CT * CT, 0, s>>>(x, H, W, theta16 + woff[l], theta + boff[l], y);
    return;
  }
  dim3 g((unsigned)(((W + CT - 1) / CT) * ((H + CT - 1) / CT)), (unsigned)(B * ((L.cout + CO_T - 1) / CO_T)));
  k_conv3<__nv_bfloat16, EPI_ACT><<<g, CT * CT, 0, s>>>(x, H, W, L.cin, theta16 + woff[l], theta + boff[l], L.cout, y,
                                                        nullptr, nullptr);
}

// Weight gradient of layer l from its input x and pre-activation gradient g,
// then (when gx is set) the data gradient into gx, masked by act_x > 0 when
// act_x is set.
void Unet::conv_bwd(cudaStream_t s, int l, const __nv_bfloat16* x, const float* g, int B, int H, int W, float* gx,
                    const __nv_bfloat16* act_x) {
  const UnetLayer& L = kUnetLayers[l];
  const long P = (long)B * H * W;
  // tensor cores take the output gradient in bf16
  const bool tc = unet_tc_enabled() && L.cout % 32 == 0;
  if (tc) k_to_bf16<<<grid_for(P * L.cout), 256, 0, s>>>(g, P * L.cout, gbf);
  if (tc && L.cin % 32 == 0 && unet_tc_conv_wgrad(s, x, gbf, B, H, W, L.cin, L.cout, grad + woff[l])) {
    k_bias_grad<<<152, 256, 0, s>>>(g, P, L.cout, grad + boff[l]);
  } else {
    dim3 gw((unsigned)(((W + CT - 1) / CT) * ((H + CT - 1) / CT)), (unsigned)(B * ((L.cout + CO_T - 1) / CO_T)),
            (unsigned)((L.cin + CK - 1) / CK));
    k_conv3_wgrad<<<gw, 256, 0, s>>>(x, g, H, W, L.cin, L.cout, grad + woff[l], grad + boff[l]);
  }
  if (gx == nullptr) return;
  k_flip_weights<<<grid_for(9L * L.cin * L.cout), 256, 0, s>>>(theta16 + woff[l], L.cin, L.cout, wflip);
  if (tc) {
    // the data gradient in tiles of at most 128 input channels (each tile's
    // weight image built here)
    const int tiles = (L.cin + 127) / 128, nt = L.cin / tiles;
    bool ok = nt * tiles == L.cin && nt % 16 == 0;
    for (int t = 0; ok && t < tiles; t++) {
      const int n0 = t * nt;
      unet_tc_weight_image(s, wflip + (long)n0 * 9 * L.cout, L.cout, nt, wimg_flip);
      ok = unet_tc_conv_dgrad(s, gbf, B, H, W, L.cout, wimg_flip, nt, gx + n0, L.cin,
                              act_x != nullptr ? act_x + n0 : nullptr);
    }
    if (ok) return;
  }
  dim3 gd((unsigned)(((W + CT - 1) / CT) * ((H + CT - 1) / CT)), (unsigned)(B * ((L.cin + CO_T - 1) / CO_T)));
  k_conv3<float, EPI_GRAD><<<gd, CT * CT, 0, s>>>(g, H, W, L.cout, wflip, nullptr, L.cin, nullptr, gx, act_x);
}

// act[] indices of the forward pass
enum {
  A_X0, A_E0A, A_S0, A_P0, A_E1A, A_S1, A_P1, A_E2A, A_S2, A_P2, A_MA, A_M, A_C2, A_D2A, A_D2, A_C1, A_D1A, A_D1,
  A_C0, A_D0A, A_D0
};

void Unet::forward(cudaStream_t s, int B, int H, int W) {
  const long P = (long)B * H * W;
  const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8;
  k_to_bf16<<<grid_for(P * 3), 256, 0, s>>>(input, P * 3, act[A_X0]);
  conv_fwd(s, 0, act[A_X0], B, H, W, act[A_E0A]);
  conv_fwd(s, 1, act[A_E0A], B, H, W, act[A_S0]);
  k_pool<<<grid_for(P / 4 * 32), 256, 0, s>>>(act[A_S0], B, H, W, 32, act[A_P0]);
  conv_fwd(s, 2, act[A_P0], B, H1, W1, act[A_E1A]);
  conv_fwd(s, 3, act[A_E1A], B, H1, W1, act[A_S1]);
  k_pool<<<grid_for(P / 16 * 64), 256, 0, s>>>(act[A_S1], B, H1, W1, 64, act[A_P1]);
  conv_fwd(s, 4, act[A_P1], B, H2, W2, act[A_E2A]);
  conv_fwd(s, 5, act[A_E2A], B, H2, W2, act[A_S2]);
  k_pool<<<grid_for(P / 64 * 96), 256, 0, s>>>(act[A_S2], B, H2, W2, 96, act[A_P2]);
  conv_fwd(s, 6, act[A_P2], B, H3, W3, act[A_MA]);
  conv_fwd(s, 7, act[A_MA], B, H3, W3, act[A_M]);
  k_up_concat<<<grid_for(P / 16 * 224), 256, 0, s>>>(act[A_M], 128, act[A_S2], 96, B, H2, W2, act[A_C2]);
  conv_fwd(s, 8, act[A_C2], B, H2, W2, act[A_D2A]);
  conv_fwd(s, 9, act[A_D2A], B, H2, W2, act[A_D2]);
  k_up_concat<<<grid_for(P / 4 * 160), 256, 0, s>>>(act[A_D2], 96, act[A_S1], 64, B, H1, W1, act[A_C1]);
  conv_fwd(s, 10, act[A_C1], B, H1, W1, act[A_D1A]);
  conv_fwd(s, 11, act[A_D1A], B, H1, W1, act[A_D1]);
  k_up_concat<<<grid_for(P * 96), 256, 0, s>>>(act[A_D1], 64, act[A_S0], 32, B, H, W, act[A_C0]);
  conv_fwd(s, 12, act[A_C0], B, H, W, act[A_D0A]);
  conv_fwd(s, 13, act[A_D0A], B, H, W, act[A_D0]);
  k_head<<<grid_for(P), 256, 0, s>>>(act[A_D0], 32, P, theta16 + woff[14], theta + boff[14], out);
}

void Unet::backward(cudaStream_t s, int B, int H, int W) {
  const long P = (long)B * H * W;
  const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8;
  float* g0 = gbuf[0];
  float* g1 = gbuf[1];
  cudaMemsetAsync(grad, 0, nparam * 4, s);
  k_head_bwd<<<grid_for(P), 256, 0, s>>>(act[A_D0], 32, P, theta16 + woff[14], dout, g0, grad + woff[14],
                                        grad + boff[14]);
  conv_bwd(s, 13, act[A_D0A], g0, B, H, W, g1, act[A_D0A]);           // dec0b
  conv_bwd(s, 12, act[A_C0], g1, B, H, W, g0, nullptr);               // dec0a -> dc0 (96 ch)
  k_up_split_bwd<<<grid_for(P / 4 * 64), 256, 0, s>>>(g0, 64, 32, B, H, W, act[A_D1], g1, gskip[0]);
  conv_bwd(s, 11, act[A_D1A], g1, B, H1, W1, g0, act[A_D1A]);         // dec1b
  conv_bwd(s, 10, act[A_C1], g0, B, H1, W1, g1, nullptr);             // dec1a -> dc1 (160 ch)
  k_up_split_bwd<<<grid_for(P / 16 * 96), 256, 0, s>>>(g1, 96, 64, B, H1, W1, act[A_D2], g0, gskip[1]);
  conv_bwd(s, 9, act[A_D2A], g0, B, H2, W2, g1, act[A_D2A]);          // dec2b
  conv_bwd(s, 8, act[A_C2], g1, B, H2, W2, g0, nullptr);              // dec2a -> dc2 (224 ch)
  k_up_split_bwd<<<grid_for(P / 64 * 128), 256, 0, s>>>(g0, 128, 96, B, H2, W2, act[A_M], g1, gskip[2]);
  conv_bwd(s, 7, act[A_MA], g1, B, H3, W3, g0, act[A_MA]);            // midb
  conv_bwd(s, 6, act[A_P2], g0, B, H3, W3, gpool, nullptr);           // mida -> dp2 (96 ch, 1/64)
  k_pool_bwd_mask<<<grid_for(P / 16 * 96), 256, 0, s>>>(gskip[2], gpool, B, H2, W2, 96, act[A_S2], g1);
  conv_bwd(s, 5, act[A_E2A], g1, B, H2, W2, g0, act[A_E2A]);          // enc2b
  conv_bwd(s, 4, act[A_P1], g0, B, H2, W2, gpool, nullptr);           // enc2a -> dp1 (64 ch, 1/16)
  k_pool_bwd_mask<<<grid_for(P / 4 * 64), 256, 0, s>>>(gskip[1], gpool, B, H1, W1, 64, act[A_S1], g1);
  conv_bwd(s, 3, act[A_E1A], g1, B, H1, W1, g0, act[A_E1A]);          // enc1b
  conv_bwd(s, 2, act[A_P0], g0, B, H1, W1, gpool, nullptr);           // enc1a -> dp0 (32 ch, 1/4)
  k_pool_bwd_mask<<<grid_for(P * 32), 256, 0, s>>>(gskip[0], gpool, B, H, W, 32, act[A_S0], g1);
  conv_bwd(s, 1, act[A_E0A], g1, B, H, W, g0, act[A_E0A]);            // enc0b
  conv_bwd(s, 0, act[A_X0], g0, B, H, W, nullptr, nullptr);           // enc0a (weights only)
}

void Unet::loss(cudaStream_t s, long P, float inv_n) {
  cudaMemsetAsync(loss_dev, 0, sizeof(double), s);
  k_mse<<<grid_for(P), 256, 0, s>>>(out, target, mask, P, inv_n, dout, loss_dev);
}

void Unet::adam(cudaStream_t s, float lr) {
  step_count++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - std::pow(b1, (float)step_count), c2 = 1.0f - std::pow(b2, (float)step_count);
  k_adam<<<grid_for(nparam), 256, 0, s>>>(theta, m, v, grad, nparam, lr, b1, b2, c1, c2, 1e-8f, theta16);
  refresh_weight_images(s);
}

void Unet::refresh_bf16(cudaStream_t s) {
  k_to_bf16<<<grid_for(nparam), 256, 0, s>>>(theta, nparam, theta16);
  refresh_weight_images(s);
}

// The halo-form tensor-core convolutions read their weights as per-chunk
// images (all 9 taps' B tiles of 32 input channels, contiguous).
void Unet::refresh_weight_images(cudaStream_t s) {
  for (int l = 0; l < UNET_LAYERS; l++) {
    const UnetLayer& L = kUnetLayers[l];
    if (L.k == 3 && L.cin % 32 == 0) unet_tc_weight_image(s, theta16 + woff[l], L.cin, L.cout, wimg + woff[l]);
  }
}

// ------------------------------------------------------------- warm start

namespace {

// p_prev from the float pressure, the float64 one, or the double-float pairs
// stored in the float64 buffers (df)
__device__ __forceinline__ double p_prev_at(const float* p32, const double* p64, int df, long k) {
  if (p64 && df) return df_to_double(reinterpret_cast<const float2*>(p64)[k]);
  return p64 ? p64[k] : (double)p32[k];
}

__global__ void __launch_bounds__(256) k_ws_psq(long n, const uint8_t* __restrict__ label, const float* __restrict__ p32,
                                                const double* __restrict__ p64a, const double* __restrict__ p64b,
                                                const int* __restrict__ par, int df, double* __restrict__ sums) {
  __shared__ double red[32];
  const double* p64 = p64a ? (*par ? p64b : p64a) : nullptr;
  double s = 0.0, c = 0.0;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    if (label[k] != FLUID) continue;
    const double p = p_prev_at(p32, p64, df, k);
    s += p * p;
    c += 1.0;
  }
  s = block_sum(s, red);
  c = block_sum(c, red);
  if (threadIdx.x == 0) {
    atomicAdd(&sums[0], s);
    atomicAdd(&sums[1], c);
  }
}

// scales = {s_b, s_p, 1/s_b, 1/s_p}; s_p falls back to s_b when p_prev
// vanishes; s_b = 0 (nothing to solve) switches the warm start off.
__global__ void k_ws_scales(const StepAccum* __restrict__ acc, const double* __restrict__ sums, float* scales) {
  const double sb = acc->n_fluid ? sqrt(acc->b_sq / (double)acc->n_fluid) : 0.0;
  double sp = sums[1] > 0 ? sqrt(sums[0] / sums[1]) : 0.0;
  if (!(sp > 0)) sp = sb;
  scales[0] = (float)sb;
  scales[1] = (float)sp;
  scales[2] = sb > 0 ? (float)(1.0 / sb) : 0.0f;
  scales[3] = sp > 0 ? (float)(1.0 / sp) : 0.0f;
}

__global__ void k_ws_input(long n, const float* __restrict__ b, const uint8_t* __restrict__ label,
                           const float* __restrict__ p32, const double* __restrict__ p64a,
                           const double* __restrict__ p64b, const int* __restrict__ par, int df,
                           const float* __restrict__ scales, float* __restrict__ x) {
  const double* p64 = p64a ? (*par ? p64b : p64a) : nullptr;
  const float ib = scales[2], ip = scales[3];
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    const bool fl = label[k] == FLUID;
    x[3 * k + 0] = fl ? b[k] * ib : 0.0f;
    x[3 * k + 1] = fl ? 1.0f : 0.0f;
    x[3 * k + 2] = fl ? (float)p_prev_at(p32, p64, df, k) * ip : 0.0f;
  }
}

__global__ void k_ws_apply(long n, const float* __restrict__ out, const uint8_t* __restrict__ label,
                           const float* __restrict__ scales, float* __restrict__ p32, double* __restrict__ p64a,
                           double* __restrict__ p64b, const int* __restrict__ par, int df) {
  if (!(scales[0] > 0.0f)) return;
  double* p64 = p64a ? (*par ? p64b : p64a) : nullptr;
  const float sp = scales[1];
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    if (label[k] != FLUID) continue;
    const float d = sp * out[k];
    if (p64 && df)
      reinterpret_cast<float2*>(p64)[k] = df_add_f(reinterpret_cast<float2*>(p64)[k], d);
    else if (p64)
      p64[k] += (double)d;
    else
      p32[k] += d;
  }
}

}  // namespace

void unet_warm_start(Unet& u, cudaStream_t s, int nx, int ny, const float* b, const uint8_t* label,
                     const StepAccum* acc, float* p32, double* p64a, double* p64b, const int* par,
                     float* scales_dev, bool df) {
  const long n = (long)nx * ny;
  cudaMemsetAsync(u.ws_acc, 0, 2 * sizeof(double), s);
  k_ws_psq<<<grid_for(n), 256, 0, s>>>(n, label, p32, p64a, p64b, par, df, u.ws_acc);
  k_ws_scales<<<1, 1, 0, s>>>(acc, u.ws_acc, scales_dev);
  k_ws_input<<<grid_for(n), 256, 0, s>>>(n, b, label, p32, p64a, p64b, par, df, scales_dev, u.input);
  u.forward(s, 1, ny, nx);
  k_ws_apply<<<grid_for(n), 256, 0, s>>>(n, u.out, label, scales_dev, p32, p64a, p64b, par, df);
}

}  // namespace fl
