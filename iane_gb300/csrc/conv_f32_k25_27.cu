// iane_gb_convolve's FP32 fast path: the instantiations for kernel widths 25 and 27.
#include "conv_f32.cuh"

namespace iane_gb {

IANE_GB_F32_WIDTHS(launch_f32_k25_27, 25, 27)

}  // namespace iane_gb
