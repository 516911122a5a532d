// Richardson-Lucy on one image as ONE persistent launch for the whole run.
//
// With one launch per pass, each pass ends in a grid-wide drain: a 256x256x64 volume is 1024
// tiles of 64x64 outputs on 608 resident slots (152 SMs x 4), so the second wave of every pass
// runs on about two thirds of the slots. Here the passes of all iterations form one device
// work queue -- phase 2t = pass A of iteration t, 2t + 1 = pass B, and within a phase the
// (tile, z plane) items in raster order, z slowest -- that a grid of resident CTAs takes from an
// atomic counter. A pass reads, with a halo of rz = kz / 2 planes, what the previous pass wrote
// and overwrites what the previous pass read, so an item of phase p at plane z waits until
// planes z - rz .. z + rz have completed phase p - 1 (a per-plane completion counter that
// reaches p x tiles-per-plane) instead of waiting for the whole volume. Items are taken in
// queue order and an item waits only for earlier items, which CTAs that are running hold, so the
// earliest unfinished item can always proceed; every wait is bounded (two seconds of global
// time), and a wait that gives up records IANE_GB_DEVICE_TIMEOUT and raises an abort flag that
// every other wait and the queue check.
//
// Each item runs the same tile body and epilogue as the per-pass launches (conv_tile_sums,
// EpiRatio / EpiUpdate), so the results are the same bits.
#pragma once

#include "rl.cuh"

namespace iane_gb {

// Everything one persistent run reads (a __grid_constant__ kernel parameter).
struct RlPersistArgs {
	CUtensorMap map_est;   // pass A source: the work estimate
	CUtensorMap map_ratio; // pass B source: the ratio image
	TileArgs pass_a;       // kernel = PSF
	TileArgs pass_b;       // kernel = adjoint
	EpiRatio epi_a;
	EpiUpdate epi_b;       // want_stats is ignored; write_out applies to the last phase only
	int tiles_x, tiles_y, nz;
	int phases;            // 2 x iterations
	unsigned int* queue;   // item counter, cleared before the launch
	int* abort;            // cleared before the launch
	unsigned int* done;    // nz per-plane completion counters, cleared before the launch
};

// Device words of a persistent run: the queue counter, the abort flag, then one counter per plane.
inline size_t rl_persist_sync_bytes(int nz) { return static_cast<size_t>(nz + 2) * sizeof(unsigned int); }

// Launch the persistent run for PSF width kx (rl_persist_lo.cu: kx <= 15, rl_persist_hi.cu: 17..31).
int launch_rl_persist(int kx, const RlPersistArgs& p, cudaStream_t stream);
int launch_rl_persist_lo(int kx, const RlPersistArgs& p, cudaStream_t stream);
int launch_rl_persist_hi(int kx, const RlPersistArgs& p, cudaStream_t stream);

// Lane geometry of the persistent kernel's tile body: 16 x by 2 y outputs per lane (conv_tile.cuh).
constexpr int kPersistRX = 16;
constexpr int kPersistRY = 2;

// Shared memory of the persistent kernel: the tiled body's tiles, taps and barriers, then the
// item index.
template<int KX>
inline size_t rl_persist_smem(int ky, int kz)
{
	return tile_smem_bytes<KX, 2, 2>(ky, kz, kTileTma) + 16;
}

template<int KX>
__global__ void __launch_bounds__(128, 4) rl_persist_kernel(const __grid_constant__ RlPersistArgs p)
{
	const int ky = p.pass_a.ky, kz = p.pass_a.kz;
	uint64_t* bars = tile_barriers<KX, 2, 2>(ky, kz);
	int* shared_item = reinterpret_cast<int*>(bars + 2);
	if (threadIdx.x == 0) {
		mbar_init(&bars[0], 1);
		mbar_init(&bars[1], 1);
		fence_barrier_init();
	}
	const unsigned int per_plane = static_cast<unsigned int>(p.tiles_x) * static_cast<unsigned int>(p.tiles_y);
	const unsigned int per_phase = per_plane * static_cast<unsigned int>(p.nz);
	const unsigned int count = per_phase * static_cast<unsigned int>(p.phases);
	const int rz = kz / 2;
	int* status = p.pass_a.status;
	uint32_t tile_phases = 0;
	for (;;) {
		__syncthreads(); // the previous item is finished everywhere; barriers initialised
		if (threadIdx.x == 0) {
			const unsigned int k = load_volatile(p.abort) ? count : atomicAdd(p.queue, 1u);
			*shared_item = k < count ? static_cast<int>(k) : -1;
		}
		__syncthreads();
		const int k = *shared_item;
		if (k < 0) {
			break;
		}
		const int phase = static_cast<int>(static_cast<unsigned int>(k) / per_phase);
		const unsigned int rem = static_cast<unsigned int>(k) - static_cast<unsigned int>(phase) * per_phase;
		const int z = static_cast<int>(rem / per_plane);
		const int tile = static_cast<int>(rem - static_cast<unsigned int>(z) * per_plane);
		if (phase > 0) {
			// thread t waits for planes z - rz + t, z - rz + t + 128, ... to finish the previous phase
			bool failed = false;
			for (int t = static_cast<int>(threadIdx.x); t <= 2 * rz && !failed; t += blockDim.x) {
				const int zz = z - rz + t;
				if (zz >= 0 && zz < p.nz) {
					failed = !wait_counter(&p.done[zz], static_cast<unsigned int>(phase) * per_plane, p.abort, status);
				}
			}
			if (__syncthreads_or(failed)) {
				break;
			}
			if (threadIdx.x == 0) {
				fence_proxy_async_global(); // the previous phase's generic stores, before this item's TMA
			}
		}
		const int x0 = (tile % p.tiles_x) * 64;
		const int y0 = (tile / p.tiles_x) * 64;
		const bool pass_b = phase & 1;
		float acc[kPersistRY][kPersistRX];
		conv_tile_sums<KX, 2, 2, kTileTma, false, kPersistRX, kPersistRY>(pass_b ? &p.map_ratio : &p.map_est,
			pass_b ? p.pass_b : p.pass_a, x0, y0, z, tile_phases, bars, acc);
		int xo = 0, yo = 0;
		tile_origin<2, kPersistRX, kPersistRY>(x0, y0, xo, yo);
		if (pass_b) {
			EpiUpdate epi = p.epi_b; // read only after the sums: not live during them
			epi.want_stats = 0;
			epi.write_out = phase == p.phases - 1 ? p.epi_b.write_out : 0;
#pragma unroll
			for (int j = 0; j < kPersistRY; ++j) epi.row(xo, yo + j, z, acc[j]);
		} else {
			const EpiRatio epi = p.epi_a;
#pragma unroll
			for (int j = 0; j < kPersistRY; ++j) epi.row(xo, yo + j, z, acc[j]);
		}
		fence_proxy_async_global(); // this thread's epilogue stores, before other items' TMA reads
		__syncthreads();
		if (threadIdx.x == 0) {
			__threadfence();
			atomicAdd(&p.done[z], 1u);
		}
	}
}

template<int KX>
int launch_rl_persist_kx(const RlPersistArgs& p, cudaStream_t stream)
{
	auto kernel = rl_persist_kernel<KX>;
	const size_t smem = rl_persist_smem<KX>(p.pass_a.ky, p.pass_a.kz);
	IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
		"persistent RL: set shared memory size");
	int per_sm = 0;
	IANE_GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, smem),
		"persistent RL: occupancy");
	const long long items = static_cast<long long>(p.tiles_x) * p.tiles_y * p.nz * p.phases;
	long long grid = static_cast<long long>(per_sm > 0 ? per_sm : 1) * device_sm_count();
	if (grid > items) grid = items;
	if (grid < 1) return IANE_GB_OK;
	kernel<<<static_cast<unsigned int>(grid), 128, smem, stream>>>(p);
	IANE_GB_CUDA(cudaGetLastError(), "persistent RL: launch");
	return IANE_GB_OK;
}

}  // namespace iane_gb
