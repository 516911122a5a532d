// Batch-pass kernel: 32x32 tiles, pass A, wide PSFs.
#include "rl_batch_kernel.cuh"

namespace iane_gb {

IANE_GB_BATCH_LAUNCHER(1, false, true)

}  // namespace iane_gb
