// Internal declarations of the pressure warm-start U-Net (fl_unet.cu,
// fl_unet_tc.cu, fl_unet_abi.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>

namespace fl {

constexpr int UNET_LAYERS = 15;
constexpr int ACT_COUNT = 21;

struct UnetLayer {
  const char* name;
  int cin, cout, k;
};
extern const UnetLayer kUnetLayers[UNET_LAYERS];

long long unet_num_params();

struct Unet {
  int device = 0;
  cudaStream_t stream = nullptr;
  long cap = 0;  // max batch * height * width
  long long nparam = 0;
  long woff[UNET_LAYERS] = {}, boff[UNET_LAYERS] = {};
  float* theta = nullptr;  // float32 master weights
  float* m = nullptr;
  float* v = nullptr;
  float* grad = nullptr;
  __nv_bfloat16* theta16 = nullptr;  // bf16 copies used by the kernels
  __nv_bfloat16* wflip = nullptr;    // flipped/transposed weights of one layer
  __nv_bfloat16* wimg = nullptr;     // tensor-core weight images (offsets woff)
  __nv_bfloat16* wimg_flip = nullptr;  // image of one output-channel tile of the flipped weights
  __nv_bfloat16* gbf = nullptr;        // bf16 copy of an output gradient (tensor-core data gradient)
  double* loss_dev = nullptr;
  __nv_bfloat16* act[ACT_COUNT] = {};
  long act_size[ACT_COUNT] = {};
  float* gbuf[2] = {nullptr, nullptr};
  float* gskip[3] = {nullptr, nullptr, nullptr};
  float* gpool = nullptr;
  float* out = nullptr;     // [P] network output
  float* dout = nullptr;    // [P] loss gradient
  float* target = nullptr;  // [P]
  float* mask = nullptr;    // [P]
  float* input = nullptr;   // [P][3] float input (converted to bf16 by forward)
  double* ws_acc = nullptr;  // warm start: sum of p_prev^2 and count over fluid cells
  long step_count = 0;
  std::string err;

  int alloc(long max_pixels, std::string* err);
  void release();
  void forward(cudaStream_t s, int B, int H, int W);
  void backward(cudaStream_t s, int B, int H, int W);
  void loss(cudaStream_t s, long P, float inv_n);
  void adam(cudaStream_t s, float lr);
  void refresh_bf16(cudaStream_t s);
  void refresh_weight_images(cudaStream_t s);
  void conv_fwd(cudaStream_t s, int l, const __nv_bfloat16* x, int B, int H, int W, __nv_bfloat16* y);
  void conv_bwd(cudaStream_t s, int l, const __nv_bfloat16* x, const float* g, int B, int H, int W, float* gx,
                const __nv_bfloat16* act_x);
};

// Tensor-core (tcgen05) forward convolution with bias and ReLU; returns
// false (and launches nothing) when the shape is not covered or the
// tensor-core path is switched off, in which case the caller runs the
// CUDA-core kernel.
// w: [Cout][3][3][Cin]; wimg: the same weights arranged by
// unet_tc_weight_image (read by the halo form).
bool unet_tc_conv_fwd(cudaStream_t s, const __nv_bfloat16* x, int B, int H, int W, int Cin, const __nv_bfloat16* w,
                      const __nv_bfloat16* wimg, const float* bias, int Cout, __nv_bfloat16* y);
void unet_tc_weight_image(cudaStream_t s, const __nv_bfloat16* w, int Cin, int Cout, __nv_bfloat16* img);
// Tensor-core data gradient of a 3x3 convolution over the output-channel
// tile of N channels: gx = conv(g, W') (g bf16 with Cin channels, wimg the
// image of W' rows of the tile), zeroed where mask <= 0 (mask optional);
// gx and mask rows are ldg elements apart. False (nothing launched) when the
// shape is not covered or the tensor cores are off.
// Tensor-core weight gradient of a 3x3 convolution: dw[n][tap][ci] +=
// sum over pixels of g[p][n] x[p + off(tap)][ci] (x and g bf16 NHWC; dw
// float, accumulated with atomics). Cin and Cout multiples of 32. False
// (nothing launched) when not covered or the tensor cores are off.
bool unet_tc_conv_wgrad(cudaStream_t s, const __nv_bfloat16* x, const __nv_bfloat16* g, int B, int H, int W, int Cin,
                        int Cout, float* dw);
bool unet_tc_conv_dgrad(cudaStream_t s, const __nv_bfloat16* g, int B, int H, int W, int Cin, const __nv_bfloat16* wimg,
                        int N, float* gx, int ldg, const __nv_bfloat16* mask);
void unet_tc_setup();
void unet_tc_enable(bool on);
// 1: the halo form (TMA halo tiles) where it applies; 0: always the
// chunked-gather form
void unet_tc_form(int form);
bool unet_tc_enabled();
// Nonzero (and cleared) when a tensor-core launch gave up a bounded wait.
int unet_tc_take_error();
// The tensor-core kernels' progress-wait bound in polls (<= 0: default).
int unet_tc_set_wait_limit(long long polls);

// Warm start inside the engine's step: input from (b, labels, p_prev), the
// forward pass, p = p_prev + s_p * out on fluid cells. p_prev is float
// (p32) or one of two float64 buffers chosen by a device parity word
// (holding double-float pairs when df).
struct StepAccum;
void unet_warm_start(Unet& u, cudaStream_t s, int nx, int ny, const float* b, const uint8_t* label,
                     const StepAccum* acc, float* p32, double* p64a, double* p64b, const int* par,
                     float* scales_dev, bool df);

}  // namespace fl
