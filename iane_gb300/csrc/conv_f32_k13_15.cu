// iane_gb_convolve's FP32 fast path: the instantiations for kernel widths 13 and 15.
#include "conv_f32.cuh"

namespace iane_gb {

IANE_GB_F32_WIDTHS(launch_f32_k13_15, 13, 15)

}  // namespace iane_gb
