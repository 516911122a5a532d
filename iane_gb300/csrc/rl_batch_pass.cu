// Persistent work-queue kernels of the batched Richardson-Lucy passes: launch dispatch. The
// eight kernel variants (tile shape x pass x PSF width class) are instantiated in
// rl_batch_k*.cu.
#include "rl_batch_kernel.cuh"

namespace iane_gb {
size_t batch_tile_smem(int wx, int kx, int ky)
{
	const int H = 32 * wx + 2 * (ky / 2);
	const size_t plane = (static_cast<size_t>(tile_pitch(kx, wx)) * H * 4 + 127) & ~size_t(127);
	const size_t taps = (static_cast<size_t>(ky) * ((kx + 3) & ~3) * 4 + 127) & ~size_t(127);
	return plane + taps + 16; // 2-D images: one tile buffer and one tap buffer
}

const void* batch_kernel_handle(int wx, bool wide)
{
	if (wx == 1) return wide ? batch_kernel_handle_impl<1, true>() : batch_kernel_handle_impl<1, false>();
	return wide ? batch_kernel_handle_impl<2, true>() : batch_kernel_handle_impl<2, false>();
}

int launch_batch_pass(int wx, bool wide, bool pass_b, const BatchImage* images, const BatchItem* items, int count,
	unsigned int* counter, int last, int grid, size_t smem, cudaStream_t stream)
{
	if (count <= 0) {
		return IANE_GB_OK;
	}
	const size_t total = smem + kBatchTail;
#define IANE_GB_BATCH_DISPATCH(WXV)                                                                                   \
	if (wide) {                                                                                                      \
		return pass_b ? launch_batch_kernel<WXV, true, true>(images, items, count, counter, last, grid, total, stream)  \
			: launch_batch_kernel<WXV, false, true>(images, items, count, counter, last, grid, total, stream);         \
	}                                                                                                                \
	return pass_b ? launch_batch_kernel<WXV, true, false>(images, items, count, counter, last, grid, total, stream)     \
		: launch_batch_kernel<WXV, false, false>(images, items, count, counter, last, grid, total, stream);
	if (wx == 1) {
		IANE_GB_BATCH_DISPATCH(1)
	}
	IANE_GB_BATCH_DISPATCH(2)
#undef IANE_GB_BATCH_DISPATCH
}

}  // namespace iane_gb
