// Velocity advection on the caller's device buffers, with no device
// allocation by the library.
//
// Who needs this: callers that cannot call cudaMalloc at the point where they
// advect — real-time threads that must not block (cudaMalloc can synchronise
// the device and wait on other work), hosts whose device memory all comes
// from an arena or caching allocator that something else owns, and processes
// that reserve their whole device-memory budget up front and may not grow
// it. They already hold device buffers for the fields they pass in and get
// back; what the MacCormack scheme needs beyond those is a scratch copy of
// the forward-advected faces (advect.ts:161 uHat / vHat) and the step's
// scalars. Here that scratch is one fixed array in the library's own device
// memory, sized for grids up to NOALLOC_MAX_FACES faces.
//
// The array is a file-scope __device__ variable: every GPU that loads the
// library holds it (about 8.8 MB) until the process exits. In host code its
// name is only a host-side stand-in, so its device address is looked up once
// per device with cudaGetSymbolAddress (with that device current) and handed
// to the kernels. That set-up happens on the first call made on each device,
// so the first call on a device should come before any stream capture. Calls
// on one device share the array: two calls whose work overlaps on the GPU
// (for example on two streams) race on it, so order them on one stream.
// Nothing in the scratch has to start at zero: the forward pass writes every
// face of it before the correction reads any, and the scalars are rewritten
// by every call. The looked-up address belongs to the device's current
// context: after cudaDeviceReset the library may be loaded at another
// address, so calls after a reset are not supported.
#include <mutex>

#include "fl_internal.h"

namespace fl {

// u faces + v faces of the largest grid accepted: 1024x1024 has 2,099,200.
constexpr long NOALLOC_MAX_FACES = 2200000;
// Scalars first (256 bytes, keeps the face arrays 256-byte aligned), then the
// forward-pass u and v faces.
constexpr long NOALLOC_SCALAR_FLOATS = 64;

static __device__ __align__(256) float g_noalloc_scratch[NOALLOC_SCALAR_FLOATS + NOALLOC_MAX_FACES];

__global__ void k_noalloc_scalars(StepScalars* sc, float dt) {
  StepScalars s{};
  s.dt = dt;
  s.keep[0] = s.keep[1] = s.keep[2] = 1.0f;
  *sc = s;
}

namespace {

std::mutex g_mu;
constexpr int MAX_DEVICES = 64;
float* g_scratch[MAX_DEVICES] = {};

// Device address of the scratch array on the current device, looked up once
// per device. Also loads the kernels this entry point launches, so later
// calls only launch.
int noalloc_setup(float** out) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) {
    set_global_error("no CUDA device: %s", cudaGetErrorString(err));
    return FL_EDEVICE;
  }
  if (dev < 0 || dev >= MAX_DEVICES) {
    set_global_error("device %d out of range", dev);
    return FL_EINVAL;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess || p == nullptr) {
      set_global_error("cudaGetSymbolAddress of the advection scratch failed: %s", cudaGetErrorString(err));
      return FL_EDEVICE;
    }
    cudaFuncAttributes attr;
    err = cudaFuncGetAttributes(&attr, k_noalloc_scalars);
    if (err == cudaSuccess) err = preload_advect_kernels();
    if (err != cudaSuccess) {
      set_global_error("loading the advection kernels failed: %s", cudaGetErrorString(err));
      return FL_EDEVICE;
    }
    g_scratch[dev] = static_cast<float*>(p);
  }
  *out = g_scratch[dev];
  return FL_OK;
}

}  // namespace
}  // namespace fl

extern "C" int fl_advect_velocity_noalloc(int scheme, int nx, int ny, float h, float dt, const float* u_in,
                                          const float* v_in, float* u_out, float* v_out, const uint8_t* label,
                                          void* stream) {
  using namespace fl;
  if (scheme != FL_SEMI_LAGRANGIAN && scheme != FL_MACCORMACK) {
    set_global_error("scheme %d", scheme);
    return FL_EINVAL;
  }
  if (nx < 2 || ny < 2) {
    set_global_error("grid %dx%d: both sides must be at least 2", nx, ny);
    return FL_EINVAL;
  }
  const long faces = (long)(nx + 1) * ny + (long)nx * (ny + 1);
  if (faces > NOALLOC_MAX_FACES) {
    set_global_error("grid %dx%d has %ld faces; the no-allocation advection scratch holds at most %ld "
                     "(a 1024x1024 grid)", nx, ny, faces, NOALLOC_MAX_FACES);
    return FL_EINVAL;
  }
  if (!u_in || !v_in || !u_out || !v_out || !label || !(h > 0)) {
    set_global_error("null device pointer or non-positive cell size");
    return FL_EINVAL;
  }
  // The advection reads its inputs' neighbours while it writes the outputs:
  // an output that overlaps an input (an in-place call) would read faces
  // already overwritten. Reject it rather than return wrong velocities.
  {
    const uintptr_t nu = (uintptr_t)(nx + 1) * ny * sizeof(float), nv = (uintptr_t)nx * (ny + 1) * sizeof(float);
    const uintptr_t nl = (uintptr_t)nx * ny;
    auto overlap = [](const void* a, uintptr_t na, const void* b, uintptr_t nb) {
      const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
      return x < y + nb && y < x + na;
    };
    if (overlap(u_out, nu, u_in, nu) || overlap(u_out, nu, v_in, nv) || overlap(u_out, nu, label, nl) ||
        overlap(v_out, nv, u_in, nu) || overlap(v_out, nv, v_in, nv) || overlap(v_out, nv, label, nl) ||
        overlap(u_out, nu, v_out, nv)) {
      set_global_error("the output velocity buffers must not overlap each other or the inputs");
      return FL_EINVAL;
    }
  }
  float* scratch = nullptr;
  int st = noalloc_setup(&scratch);
  if (st != FL_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  StepScalars* sc = reinterpret_cast<StepScalars*>(scratch);
  float* u_hat = scratch + NOALLOC_SCALAR_FLOATS;
  float* v_hat = u_hat + (long)(nx + 1) * ny;
  k_noalloc_scalars<<<1, 1, 0, s>>>(sc, dt);
  launch_advect_velocity(s, nx, ny, h, scheme == FL_MACCORMACK, u_in, v_in, u_hat, v_hat, u_out, v_out, label, sc);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) {
    set_global_error("advection launch failed: %s", cudaGetErrorString(err));
    return FL_EDEVICE;
  }
  return FL_OK;
}
