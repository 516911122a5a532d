// Batch-pass kernel: 64x64 tiles, pass A, narrow PSFs.
#include "rl_batch_kernel.cuh"

namespace iane_gb {

IANE_GB_BATCH_LAUNCHER(2, false, false)

}  // namespace iane_gb
