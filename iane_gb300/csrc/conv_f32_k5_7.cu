// iane_gb_convolve's FP32 fast path: the instantiations for kernel widths 5 and 7.
#include "conv_f32.cuh"

namespace iane_gb {

IANE_GB_F32_WIDTHS(launch_f32_k5_7, 5, 7)

}  // namespace iane_gb
