// The persistent kernel of the batched Richardson-Lucy run (rl_batch.cuh): one launch takes
// every (phase, image, tile) item of the run from a device queue, waits for the item's image
// to finish its previous phase, runs the fused tiled convolution body of the item's pass and
// PSF width, and counts the tile as done for its image.
#include "rl_batch.cuh"

namespace iane_gb {
namespace {

// Bytes after the tiles and taps: the two tile mbarriers and the item index.
constexpr size_t kBatchTail = 32;

// The sums of one item's tile for its PSF width (the epilogue is applied by the caller).
__device__ __forceinline__ void item_sums(const BatchImage& im, bool pass_b, int x0, int y0, uint32_t& phases,
	uint64_t* bars, float (&acc)[kRY][kRX], bool taps_resident)
{
	const CUtensorMap* map = pass_b ? &im.map_ratio : &im.map_est;
	const TileArgs& a = pass_b ? im.pass_b : im.pass_a;
#define IANE_GB_BATCH_KX(K) \
	case K: conv_tile_sums<K, 2, 2, kTileTma, true>(map, a, x0, y0, 0, phases, bars, acc, taps_resident); break;
	switch (im.kx) {
	IANE_GB_BATCH_KX(1) IANE_GB_BATCH_KX(3) IANE_GB_BATCH_KX(5) IANE_GB_BATCH_KX(7)
	IANE_GB_BATCH_KX(9) IANE_GB_BATCH_KX(11) IANE_GB_BATCH_KX(13) IANE_GB_BATCH_KX(15)
	IANE_GB_BATCH_KX(17) IANE_GB_BATCH_KX(19) IANE_GB_BATCH_KX(21) IANE_GB_BATCH_KX(23)
	IANE_GB_BATCH_KX(25) IANE_GB_BATCH_KX(27) IANE_GB_BATCH_KX(29) IANE_GB_BATCH_KX(31)
	default: break;
	}
#undef IANE_GB_BATCH_KX
}

// total = dynamic shared memory of the launch: the largest tile and taps + kBatchTail.
__global__ void __launch_bounds__(128) batch_persistent_kernel(const BatchImage* __restrict__ images,
	const BatchItem* __restrict__ items, int items_per_phase, int phases, BatchSync sync, int* status,
	unsigned int total)
{
	extern __shared__ __align__(128) unsigned char smem_raw[];
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + total - kBatchTail);
	int* shared_item = reinterpret_cast<int*>(smem_raw + total - kBatchTail + 16);
	if (threadIdx.x == 0) {
		mbar_init(&bars[0], 1);
		mbar_init(&bars[1], 1);
		fence_barrier_init();
	}
	const unsigned int count = static_cast<unsigned int>(items_per_phase) * static_cast<unsigned int>(phases);
	uint32_t tile_phases = 0;
	for (;;) {
		__syncthreads(); // the previous item is finished everywhere; barriers initialised
		if (threadIdx.x == 0) {
			const unsigned int k = load_volatile(sync.abort) ? count : atomicAdd(sync.queue, 1u);
			int go = k < count;
			if (go) {
				const int phase = static_cast<int>(k / static_cast<unsigned int>(items_per_phase));
				const BatchItem w = items[k - static_cast<unsigned int>(phase) * items_per_phase];
				// the item's tensor map into the descriptor cache while the wait and the taps proceed
				const CUtensorMap* map = (phase & 1) ? &images[w.image].map_ratio : &images[w.image].map_est;
				asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
				if (phase > 0) {
					// the image's previous phase complete (bounded: a wait that gives up aborts the run)
					go = wait_counter(&sync.done[w.image], static_cast<unsigned int>(phase) * w.image_tiles, sync.abort,
						status);
					fence_proxy_async_global(); // the image's previous phase, written by generic stores, before TMA
				}
			}
			*shared_item = go ? static_cast<int>(k) : -1;
		}
		__syncthreads();
		const int k = *shared_item;
		if (k < 0) {
			break;
		}
		const int phase = k / items_per_phase;
		const BatchItem w = items[k - phase * items_per_phase];
		const BatchImage& im = images[w.image];
		const int y0 = (w.tile / im.tiles_x) * kBatchTile;
		// the item's tiles, left to right along one tile row; the PSF taps stay in shared memory
		// from the first tile to the last
		for (int c = 0; c < w.count; ++c) {
			const int x0 = (w.tile % im.tiles_x + c) * kBatchTile;
			float acc[kRY][kRX];
			int xo = 0, yo = 0;
			tile_origin<2>(x0, y0, xo, yo);
			item_sums(im, phase & 1, x0, y0, tile_phases, bars, acc, c > 0);
			if (phase & 1) {
				EpiUpdate epi = im.epi_b; // read only after the sums: not live during them
				epi.want_stats = 0;
				epi.write_out = phase == phases - 1 && im.write_out_final;
#pragma unroll
				for (int j = 0; j < kRY; ++j) epi.row(xo, yo + j, 0, acc[j]);
			} else {
				const EpiRatio epi = im.epi_a;
#pragma unroll
				for (int j = 0; j < kRY; ++j) epi.row(xo, yo + j, 0, acc[j]);
			}
		}
		fence_proxy_async_global(); // this thread's epilogue stores, before other tiles' TMA reads
		__syncthreads();
		if (threadIdx.x == 0) {
			__threadfence();
			atomicAdd(&sync.done[w.image], static_cast<unsigned int>(w.count));
		}
	}
}

}  // namespace

size_t batch_tile_smem(int kx, int ky)
{
	const int H = kBatchTile + 2 * (ky / 2);
	const size_t plane = (static_cast<size_t>(tile_pitch(kx, 2)) * H * 4 + 127) & ~size_t(127);
	const size_t taps = (static_cast<size_t>(ky) * ((kx + 3) & ~3) * 4 + 127) & ~size_t(127);
	return plane + taps + 16; // 2-D images: one tile buffer and one tap buffer
}

int batch_blocks_per_sm(size_t smem)
{
	const size_t total = smem + kBatchTail;
	int per_sm = 0;
	if (cudaFuncSetAttribute(batch_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
	        static_cast<int>(total)) != cudaSuccess ||
	    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_persistent_kernel, 128, total) != cudaSuccess) {
		cudaGetLastError();
		return 1;
	}
	return per_sm > 0 ? per_sm : 1;
}

int launch_batch_persistent(const BatchImage* images, const BatchItem* items, int items_per_phase, int phases,
	BatchSync sync, int* status, int grid, size_t smem, cudaStream_t stream)
{
	if (items_per_phase <= 0 || phases <= 0) {
		return IANE_GB_OK;
	}
	const size_t total = smem + kBatchTail;
	IANE_GB_CUDA(cudaFuncSetAttribute(batch_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
		static_cast<int>(total)), "batch: set shared memory size");
	batch_persistent_kernel<<<grid, 128, total, stream>>>(images, items, items_per_phase, phases, sync, status,
		static_cast<unsigned int>(total));
	IANE_GB_CUDA(cudaGetLastError(), "batch: launch");
	return IANE_GB_OK;
}

}  // namespace iane_gb
