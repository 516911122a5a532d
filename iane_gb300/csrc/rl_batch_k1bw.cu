// Batch-pass kernel: 32x32 tiles, pass B, wide PSFs.
#include "rl_batch_kernel.cuh"

namespace iane_gb {

IANE_GB_BATCH_LAUNCHER(1, true, true)

template<>
const void* batch_kernel_handle_impl<1, true>()
{
	return reinterpret_cast<const void*>(batch_pass_kernel<1, true, true>);
}

}  // namespace iane_gb
