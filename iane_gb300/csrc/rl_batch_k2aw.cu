// Batch-pass kernel: 64x64 tiles, pass A, wide PSFs.
#include "rl_batch_kernel.cuh"

namespace iane_gb {

IANE_GB_BATCH_LAUNCHER(2, false, true)

}  // namespace iane_gb
