// iane_gb_convolve's FP32 fast path: the instantiations for kernel widths 1 and 3.
#include "conv_f32.cuh"

namespace iane_gb {

IANE_GB_F32_WIDTHS(launch_f32_k1_3, 1, 3)

}  // namespace iane_gb
