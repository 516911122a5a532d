// Batch-pass kernel: 32x32 tiles, pass B, narrow PSFs.
#include "rl_batch_kernel.cuh"

namespace iane_gb {

IANE_GB_BATCH_LAUNCHER(1, true, false)

template<>
const void* batch_kernel_handle_impl<1, false>()
{
	return reinterpret_cast<const void*>(batch_pass_kernel<1, true, false>);
}

}  // namespace iane_gb
