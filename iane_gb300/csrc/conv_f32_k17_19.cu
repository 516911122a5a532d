// iane_gb_convolve's FP32 fast path: the instantiations for kernel widths 17 and 19.
#include "conv_f32.cuh"

namespace iane_gb {

IANE_GB_F32_WIDTHS(launch_f32_k17_19, 17, 19)

}  // namespace iane_gb
