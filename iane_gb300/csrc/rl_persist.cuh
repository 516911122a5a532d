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
//
// Per-iteration statistics (flux, relative change): each pass B item reduces its threads' FP32
// Kahan partials to three doubles and stores them at its index within the pass, in one of two
// buffers by iteration parity; the item that completes an iteration's pass B last combines that
// buffer in index order (deterministic) and publishes the iteration as combined. A pass B item
// of iteration t >= 2 first waits until iteration t - 2 is combined, as it reuses that buffer.
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
	EpiUpdate epi_b;       // write_out applies to the last phase only
	int tiles_x, tiles_y, nz;
	int phases;            // 2 x iterations
	unsigned int* queue;   // item counter, cleared before the launch
	int* abort;            // cleared before the launch
	unsigned int* done;    // nz per-plane completion counters, cleared before the launch
	// statistics (stats != null): 2 x items-per-pass x 3 doubles of partials, 2 doubles per
	// iteration of results, per-parity pass B completion counts and the count of combined
	// iterations (cleared before the launch)
	double* parts;
	double* stats;
	unsigned int* stat_count;
	unsigned int* stat_done;
};

// Device words of a persistent run: the queue counter, the abort flag, one counter per plane,
// then the two statistics counts and the count of combined iterations.
inline size_t rl_persist_sync_bytes(int nz) { return static_cast<size_t>(nz + 5) * sizeof(unsigned int); }

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

// The statistics of one pass B item (see above). Uses the start of shared memory, which no thread
// reads once the item's sums are done and into which no copy is in flight.
__device__ __forceinline__ void persist_stats(const RlPersistArgs& p, const EpiUpdate& epi, int it, int item,
	unsigned int per_phase)
{
	extern __shared__ __align__(128) unsigned char smem_raw[];
	double* red = reinterpret_cast<double*>(smem_raw);
	int& last = *reinterpret_cast<int*>(red + 3 * 32);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
	double v[3] = {static_cast<double>(epi.f_s) - static_cast<double>(epi.f_c),
		static_cast<double>(epi.c_s) - static_cast<double>(epi.c_c), static_cast<double>(epi.n_s) - static_cast<double>(epi.n_c)};
#pragma unroll
	for (int k = 0; k < 3; ++k) {
#pragma unroll
		for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
	}
	__syncthreads();
	if (lane == 0) {
		for (int k = 0; k < 3; ++k) red[warp * 3 + k] = v[k];
	}
	__syncthreads();
	double* slot = p.parts + static_cast<size_t>(it & 1) * per_phase * 3;
	if (threadIdx.x == 0) {
		double t[3] = {0.0, 0.0, 0.0};
		for (int w = 0; w < warps; ++w)
			for (int k = 0; k < 3; ++k) t[k] += red[w * 3 + k];
		for (int k = 0; k < 3; ++k) slot[static_cast<size_t>(item) * 3 + k] = t[k];
		__threadfence();
		last = atomicAdd(&p.stat_count[it & 1], 1u) == per_phase - 1;
	}
	__syncthreads();
	if (!last) {
		return;
	}
	// the iteration's last pass B item: combine the partials in item order
	__threadfence();
	double t[3] = {0.0, 0.0, 0.0};
	for (unsigned int b = threadIdx.x; b < per_phase; b += blockDim.x) {
		for (int k = 0; k < 3; ++k) t[k] += __ldcg(&slot[static_cast<size_t>(b) * 3 + k]);
	}
#pragma unroll
	for (int k = 0; k < 3; ++k) {
#pragma unroll
		for (int off = 16; off > 0; off >>= 1) t[k] += __shfl_down_sync(0xffffffffu, t[k], off);
	}
	__syncthreads();
	if (lane == 0) {
		for (int k = 0; k < 3; ++k) red[warp * 3 + k] = t[k];
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		double s[3] = {0.0, 0.0, 0.0};
		for (int w = 0; w < warps; ++w)
			for (int k = 0; k < 3; ++k) s[k] += red[w * 3 + k];
		p.stats[2 * it] = s[0];
		p.stats[2 * it + 1] = s[2] > 0.0 ? sqrt(s[1] / s[2]) : 0.0;
		p.stat_count[it & 1] = 0u;
		__threadfence();
		atomicAdd(p.stat_done, 1u); // iterations are combined in order: this makes it it + 1
	}
}

// STATS: per-iteration statistics are gathered (a separate instantiation, so that runs without
// them keep the leaner kernel)
template<int KX, bool STATS>
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
			// statistics of iteration t >= 2 reuse the buffer of iteration t - 2: wait until it is combined
			const int it = phase >> 1;
			if (STATS && (phase & 1) && it >= 2 && threadIdx.x == 0 && !failed) {
				failed = !wait_counter(p.stat_done, static_cast<unsigned int>(it - 1), p.abort, status);
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
			epi.want_stats = STATS ? 1 : 0;
			epi.write_out = phase == p.phases - 1 ? p.epi_b.write_out : 0;
#pragma unroll
			for (int j = 0; j < kPersistRY; ++j) epi.row(xo, yo + j, z, acc[j]);
			if constexpr (STATS) {
				persist_stats(p, epi, phase >> 1, static_cast<int>(rem), per_phase);
			}
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
	auto kernel = p.stats ? rl_persist_kernel<KX, true> : rl_persist_kernel<KX, false>;
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
