// Batch-pass kernel: 64x64 tiles, pass B, wide PSFs.
#include "rl_batch_kernel.cuh"

namespace iane_gb {

IANE_GB_BATCH_LAUNCHER(2, true, true)

template<>
const void* batch_kernel_handle_impl<2, true>()
{
	return reinterpret_cast<const void*>(batch_pass_kernel<2, true, true>);
}

}  // namespace iane_gb
