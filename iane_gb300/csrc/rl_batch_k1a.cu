// Batch-pass kernel: 32x32 tiles, pass A.
#include "rl_batch_kernel.cuh"

namespace iane_gb {

template<>
int launch_batch_kernel<1, false>(const BatchImage* images, const BatchItem* items, int count,
	unsigned int* counter, int last, int grid, size_t total, cudaStream_t stream)
{
	auto kernel = batch_pass_kernel<1, false>;
	IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(total)),
		"batch pass: set shared memory size");
	kernel<<<grid, 32, total, stream>>>(images, items, count, counter, last, static_cast<unsigned int>(total));
	IANE_GB_CUDA(cudaGetLastError(), "batch pass: launch");
	return IANE_GB_OK;
}

}  // namespace iane_gb
