// iane_gb_convolve's FP32 fast path: the instantiations for kernel widths 21 and 23.
#include "conv_f32.cuh"

namespace iane_gb {

IANE_GB_F32_WIDTHS(launch_f32_k21_23, 21, 23)

}  // namespace iane_gb
