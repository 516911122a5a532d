// Batch-pass kernel: 64x64 tiles, pass B.
#include "rl_batch_kernel.cuh"

namespace iane_gb {

template<>
int launch_batch_kernel<2, true>(const BatchImage* images, const BatchItem* items, int count,
	unsigned int* counter, int last, int grid, size_t total, cudaStream_t stream)
{
	auto kernel = batch_pass_kernel<2, true>;
	IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(total)),
		"batch pass: set shared memory size");
	kernel<<<grid, 128, total, stream>>>(images, items, count, counter, last, static_cast<unsigned int>(total));
	IANE_GB_CUDA(cudaGetLastError(), "batch pass: launch");
	return IANE_GB_OK;
}

template<>
const void* batch_kernel_handle_impl<2>()
{
	return reinterpret_cast<const void*>(batch_pass_kernel<2, true>);
}

}  // namespace iane_gb
