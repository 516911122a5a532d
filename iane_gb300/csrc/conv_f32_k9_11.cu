// iane_gb_convolve's FP32 fast path: the instantiations for kernel widths 9 and 11.
#include "conv_f32.cuh"

namespace iane_gb {

IANE_GB_F32_WIDTHS(launch_f32_k9_11, 9, 11)

}  // namespace iane_gb
