// The persistent batch-pass kernel template (instantiated once per tile shape and pass in
// rl_batch_k*.cu so that the variants compile in parallel).
#pragma once

#include "rl_batch.cuh"

namespace iane_gb {

// Bytes after the largest tiles/taps of a launch: the two tile mbarriers and the work item.
constexpr size_t kBatchTail = 32;

template<int WX, bool PASS_B, bool WIDE, class Epi>
__device__ __forceinline__ void batch_run_item(const BatchImage& im, Epi& epi, int x0, int y0, uint32_t& phases,
	uint64_t* bars)
{
	const CUtensorMap* map = PASS_B ? &im.map_ratio : &im.map_est;
	const TileArgs& a = PASS_B ? im.pass_b : im.pass_a;
#define IANE_GB_BATCH_KX(K) \
	case K: conv_tile_body<K, WX, WX, kTileTma, Epi, true>(map, a, epi, x0, y0, 0, phases, bars); break;
	if constexpr (WIDE) {
		switch (im.kx) {
		IANE_GB_BATCH_KX(17) IANE_GB_BATCH_KX(19) IANE_GB_BATCH_KX(21) IANE_GB_BATCH_KX(23)
		IANE_GB_BATCH_KX(25) IANE_GB_BATCH_KX(27) IANE_GB_BATCH_KX(29) IANE_GB_BATCH_KX(31)
		default: break;
		}
	} else {
		switch (im.kx) {
		IANE_GB_BATCH_KX(1) IANE_GB_BATCH_KX(3) IANE_GB_BATCH_KX(5) IANE_GB_BATCH_KX(7)
		IANE_GB_BATCH_KX(9) IANE_GB_BATCH_KX(11) IANE_GB_BATCH_KX(13) IANE_GB_BATCH_KX(15)
		default: break;
		}
	}
#undef IANE_GB_BATCH_KX
}

// total = dynamic shared memory of the launch: the largest tiles/taps + kBatchTail.
template<int WX, bool PASS_B, bool WIDE>
__global__ void __launch_bounds__(32 * WX * WX) batch_pass_kernel(const BatchImage* __restrict__ images,
	const BatchItem* __restrict__ items, int count, unsigned int* counter, int last, unsigned int total)
{
	extern __shared__ __align__(128) unsigned char smem_raw[];
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + total - kBatchTail);
	int* item_s = reinterpret_cast<int*>(smem_raw + total - kBatchTail + 16);
	if (threadIdx.x == 0) {
		mbar_init(&bars[0], 1);
		mbar_init(&bars[1], 1);
		fence_barrier_init();
	}
	uint32_t phases = 0;
	for (;;) {
		__syncthreads(); // the previous item is finished everywhere; barriers initialised
		if (threadIdx.x == 0) {
			*item_s = static_cast<int>(atomicAdd(counter, 1u));
		}
		__syncthreads();
		const int it = *item_s;
		if (it >= count) {
			break;
		}
		const BatchItem w = items[it];
		const BatchImage& im = images[w.image];
		const int x0 = (w.tile % im.tiles_x) * 32 * WX;
		const int y0 = (w.tile / im.tiles_x) * 32 * WX;
		if constexpr (PASS_B) {
			EpiUpdate epi = im.epi_b;
			epi.write_out = last && im.write_out_final;
			batch_run_item<WX, true, WIDE>(im, epi, x0, y0, phases, bars);
		} else {
			EpiRatio epi = im.epi_a;
			batch_run_item<WX, false, WIDE>(im, epi, x0, y0, phases, bars);
		}
	}
}

template<int WX, bool PASS_B, bool WIDE>
int launch_batch_kernel(const BatchImage* images, const BatchItem* items, int count, unsigned int* counter, int last,
	int grid, size_t total, cudaStream_t stream);

template<int WX, bool WIDE>
const void* batch_kernel_handle_impl();

// One kernel variant per translation unit (rl_batch_k*.cu), so that they compile in parallel;
// the pass-B variant also answers occupancy queries for its shape and class.
#define IANE_GB_BATCH_LAUNCHER(WXV, PB, WD)                                                                  \
	template<>                                                                                              \
	int launch_batch_kernel<WXV, PB, WD>(const BatchImage* images, const BatchItem* items, int count,       \
		unsigned int* counter, int last, int grid, size_t total, cudaStream_t stream)                       \
	{                                                                                                       \
		auto kernel = batch_pass_kernel<WXV, PB, WD>;                                                       \
		IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,              \
			static_cast<int>(total)), "batch pass: set shared memory size");                                \
		kernel<<<grid, 32 * WXV * WXV, total, stream>>>(images, items, count, counter, last,               \
			static_cast<unsigned int>(total));                                                              \
		IANE_GB_CUDA(cudaGetLastError(), "batch pass: launch");                                             \
		return IANE_GB_OK;                                                                                  \
	}

}  // namespace iane_gb
