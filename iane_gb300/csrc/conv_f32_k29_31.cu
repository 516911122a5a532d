// iane_gb_convolve's FP32 fast path: the instantiations for kernel widths 29 and 31.
#include "conv_f32.cuh"

namespace iane_gb {

IANE_GB_F32_WIDTHS(launch_f32_k29_31, 29, 31)

}  // namespace iane_gb
