// C ABI of the pressure warm-start U-Net (include/flowlab_gb300.h, section
// "Learned warm start"). No reference counterpart: the reference's warm
// start is the previous pressure (src/core/pressureSolver.ts:28-30).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>

#include "fl_internal.h"
#include "fl_unet.h"

using namespace fl;

struct fl_unet {
  Unet u;
  std::atomic<int> busy{0};
};

namespace {

int ufail(fl_unet* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h)
    h->u.err = buf;
  else
    set_global_error("%s", buf);
  return code;
}

int ucuda(fl_unet* h, cudaError_t err, const char* where) {
  if (err == cudaSuccess) return FL_OK;
  return ufail(h, err == cudaErrorMemoryAllocation ? FL_ENOMEM : FL_EDEVICE, "%s: %s", where, cudaGetErrorString(err));
}

int usync(fl_unet* h, const char* where) {
  cudaError_t err = cudaStreamSynchronize(h->u.stream);
  if (err == cudaSuccess) err = cudaGetLastError();
  return ucuda(h, err, where);
}

struct UCall {
  fl_unet* h;
  bool ok;
  explicit UCall(fl_unet* x) : h(x), ok(false) {
    if (!h) return;
    int expected = 0;
    ok = h->busy.compare_exchange_strong(expected, 1);
    if (ok) cudaSetDevice(h->u.device);
  }
  ~UCall() {
    if (ok) h->busy.store(0);
  }
};

#define UENTER(x)                                                      \
  if (!(x)) return ufail(nullptr, FL_EINVAL, "null network");          \
  UCall ucall_(x);                                                     \
  if (!ucall_.ok) return ufail(x, FL_EBUSY, "network call is not re-entrant");

#define UTRY(x)           \
  do {                    \
    int st_ = (x);        \
    if (st_) return st_;  \
  } while (0)

int check_shape(fl_unet* h, int B, int H, int W) {
  if (B < 1 || H < 8 || W < 8 || H % 8 || W % 8)
    return ufail(h, FL_EINVAL, "batch %d of %dx%d: sides must be positive multiples of 8", B, H, W);
  if ((long)B * H * W > h->u.cap)
    return ufail(h, FL_EINVAL, "batch %d of %dx%d exceeds the capacity of %ld pixels", B, H, W, h->u.cap);
  return FL_OK;
}

}  // namespace

extern "C" {

int fl_unet_create(long long max_pixels, int device, fl_unet** out) {
  if (!out) return ufail(nullptr, FL_EINVAL, "null output pointer");
  *out = nullptr;
  if (max_pixels < 64 || max_pixels % 64) return ufail(nullptr, FL_EINVAL, "max_pixels must be a positive multiple of 64");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ufail(nullptr, FL_EDEVICE, "no CUDA device");
  if (device < 0 || device >= ndev) return ufail(nullptr, FL_EINVAL, "device %d of %d", device, ndev);
  cudaSetDevice(device);
  fl_unet* h = new (std::nothrow) fl_unet();
  if (!h) return ufail(nullptr, FL_ENOMEM, "host allocation");
  h->u.device = device;
  std::string err;
  int st = h->u.alloc((long)max_pixels, &err);
  if (st == FL_OK && cudaStreamCreateWithFlags(&h->u.stream, cudaStreamNonBlocking) != cudaSuccess) {
    err = "stream creation failed";
    st = FL_EDEVICE;
  }
  if (st != FL_OK) {
    set_global_error("%s", err.c_str());
    h->u.release();
    delete h;
    return st;
  }
  unet_tc_setup();
  cudaMemset(h->u.theta, 0, h->u.nparam * 4);
  h->u.refresh_bf16(h->u.stream);
  if (cudaStreamSynchronize(h->u.stream) != cudaSuccess) {
    h->u.release();
    delete h;
    return ufail(nullptr, FL_EDEVICE, "initialisation failed");
  }
  *out = h;
  return FL_OK;
}

int fl_unet_destroy(fl_unet* h) {
  if (!h) return FL_OK;
  cudaSetDevice(h->u.device);
  if (h->u.stream) {
    cudaStreamSynchronize(h->u.stream);
    cudaStreamDestroy(h->u.stream);
  }
  h->u.release();
  delete h;
  return FL_OK;
}

const char* fl_unet_last_error(const fl_unet* h) { return h ? h->u.err.c_str() : fl_last_error(nullptr); }

long long fl_unet_num_params(void) { return unet_num_params(); }

int fl_unet_set_params(fl_unet* h, const float* theta) {
  UENTER(h);
  if (!theta) return ufail(h, FL_EINVAL, "null parameters");
  Unet& u = h->u;
  cudaStream_t s = u.stream;
  UTRY(ucuda(h, cudaMemcpyAsync(u.theta, theta, u.nparam * 4, cudaMemcpyHostToDevice, s), "parameters"));
  cudaMemsetAsync(u.m, 0, u.nparam * 4, s);
  cudaMemsetAsync(u.v, 0, u.nparam * 4, s);
  u.step_count = 0;
  u.refresh_bf16(s);
  return usync(h, "set parameters");
}

int fl_unet_get_params(fl_unet* h, float* theta) {
  UENTER(h);
  if (!theta) return ufail(h, FL_EINVAL, "null parameters");
  UTRY(ucuda(h, cudaMemcpyAsync(theta, h->u.theta, h->u.nparam * 4, cudaMemcpyDeviceToHost, h->u.stream),
             "parameters"));
  return usync(h, "get parameters");
}

int fl_unet_forward(fl_unet* h, int B, int H, int W, const float* x, float* out) {
  UENTER(h);
  UTRY(check_shape(h, B, H, W));
  if (!x || !out) return ufail(h, FL_EINVAL, "null pointer");
  Unet& u = h->u;
  const long P = (long)B * H * W;
  UTRY(ucuda(h, cudaMemcpyAsync(u.input, x, P * 3 * 4, cudaMemcpyHostToDevice, u.stream), "input"));
  u.forward(u.stream, B, H, W);
  UTRY(ucuda(h, cudaGetLastError(), "forward"));
  UTRY(ucuda(h, cudaMemcpyAsync(out, u.out, P * 4, cudaMemcpyDeviceToHost, u.stream), "output"));
  UTRY(usync(h, "forward"));
  if (unet_tc_take_error()) return ufail(h, FL_ETIMEOUT, "a tensor-core convolution gave up a bounded wait");
  return FL_OK;
}

int fl_unet_train_step(fl_unet* h, int B, int H, int W, const float* x, const float* target, const float* mask,
                       double lr, int update, double* loss, float* grad) {
  UENTER(h);
  UTRY(check_shape(h, B, H, W));
  if (!x || !target || !mask) return ufail(h, FL_EINVAL, "null pointer");
  Unet& u = h->u;
  cudaStream_t s = u.stream;
  const long P = (long)B * H * W;
  double nmask = 0;
  for (long k = 0; k < P; k++) nmask += mask[k];
  if (!(nmask > 0)) return ufail(h, FL_EINVAL, "empty mask");
  UTRY(ucuda(h, cudaMemcpyAsync(u.input, x, P * 3 * 4, cudaMemcpyHostToDevice, s), "input"));
  UTRY(ucuda(h, cudaMemcpyAsync(u.target, target, P * 4, cudaMemcpyHostToDevice, s), "target"));
  UTRY(ucuda(h, cudaMemcpyAsync(u.mask, mask, P * 4, cudaMemcpyHostToDevice, s), "mask"));
  u.forward(s, B, H, W);
  u.loss(s, P, (float)(1.0 / nmask));
  u.backward(s, B, H, W);
  if (update) u.adam(s, (float)lr);
  UTRY(ucuda(h, cudaGetLastError(), "train step"));
  double l = 0;
  UTRY(ucuda(h, cudaMemcpyAsync(&l, u.loss_dev, sizeof l, cudaMemcpyDeviceToHost, s), "loss"));
  if (grad) UTRY(ucuda(h, cudaMemcpyAsync(grad, u.grad, u.nparam * 4, cudaMemcpyDeviceToHost, s), "gradient"));
  UTRY(usync(h, "train step"));
  if (unet_tc_take_error()) return ufail(h, FL_ETIMEOUT, "a tensor-core convolution gave up a bounded wait");
  if (loss) *loss = l;
  return FL_OK;
}

int fl_unet_set_wait_limit(long long polls) {
  if (unet_tc_set_wait_limit(polls) != 0) return ufail(nullptr, FL_EDEVICE, "setting the wait limit failed");
  return FL_OK;
}

int fl_unet_use_tensor_cores(int mode) {
  if (mode < 0 || mode > 2) return ufail(nullptr, FL_EINVAL, "tensor-core mode %d", mode);
  unet_tc_enable(mode != 0);
  unet_tc_form(mode == 1 ? 1 : 0);
  return FL_OK;
}

}  // extern "C"

// Engine-side hooks live in fl_engine.cu; they reach the network through this.
namespace fl {
Unet* unet_of(fl_unet* h) { return h ? &h->u : nullptr; }
}  // namespace fl
