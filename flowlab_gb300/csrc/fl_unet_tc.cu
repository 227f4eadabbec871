// Tensor-core forward convolution of the warm-start U-Net (placeholder
// switch; the tcgen05 kernel is added here).
#include "fl_internal.h"
#include "fl_unet.h"

namespace fl {

namespace {
bool g_tc_on = false;
}

void unet_tc_enable(bool on) { g_tc_on = on; }
bool unet_tc_enabled() { return g_tc_on; }

bool unet_tc_conv_fwd(cudaStream_t, const __nv_bfloat16*, int, int, int, int, const __nv_bfloat16*, const float*, int,
                      __nv_bfloat16*) {
  return false;
}

}  // namespace fl
