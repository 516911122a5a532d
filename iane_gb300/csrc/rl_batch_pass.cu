// Persistent work-queue kernels of the batched Richardson-Lucy passes: launch dispatch. The
// four kernel variants (tile shape x pass) are instantiated in rl_batch_k*.cu.
#include "rl_batch_kernel.cuh"

namespace iane_gb {
size_t batch_tile_smem(int wx, int kx, int ky)
{
	const int H = 32 * wx + 2 * (ky / 2);
	const size_t plane = (static_cast<size_t>(tile_pitch(kx, wx)) * H * 4 + 127) & ~size_t(127);
	const size_t taps = (static_cast<size_t>(ky) * ((kx + 3) & ~3) * 4 + 127) & ~size_t(127);
	return plane + taps + 16; // 2-D images: one tile buffer and one tap buffer
}

const void* batch_kernel_handle(int wx)
{
	return wx == 1 ? batch_kernel_handle_impl<1>() : batch_kernel_handle_impl<2>();
}

int launch_batch_pass(int wx, bool pass_b, const BatchImage* images, const BatchItem* items, int count,
	unsigned int* counter, int last, int grid, size_t smem, cudaStream_t stream)
{
	if (count <= 0) {
		return IANE_GB_OK;
	}
	const size_t total = smem + kBatchTail;
	if (wx == 1) {
		return pass_b ? launch_batch_kernel<1, true>(images, items, count, counter, last, grid, total, stream)
			: launch_batch_kernel<1, false>(images, items, count, counter, last, grid, total, stream);
	}
	return pass_b ? launch_batch_kernel<2, true>(images, items, count, counter, last, grid, total, stream)
		: launch_batch_kernel<2, false>(images, items, count, counter, last, grid, total, stream);
}

}  // namespace iane_gb
