// BF16 tensor-core convolution for the Richardson-Lucy precision path with output z planes
// along the MMA's N dimension (tcgen05, FP32 accumulation in TMEM).
//
// A CTA computes a 128 (y) x 16 (x) x ZC (z) block of outputs. For input plane z_in, kernel
// row b and the 16-column output block, the contribution to all ZC output planes at once is
//
//     D[m, (i, n)] += sum_k A_{z_in, b}[m, k] * T_{b, qz = i + Z + rz - z_in}[k, n]
//
// with m = output row y0 + m, k = 32 input columns x0 - 8 + k (the A operand: the input
// plane's halo tile shifted by 2 ry - b rows, as in rl_tc.cuh), n = output column x0 + n,
// i = output plane Z + i, and T the banded x-Toeplitz matrices of rl_tc.cuh. The T matrices
// of all kernel planes qz are stored N-contiguous per (b, 8-column K chunk) -- [b][chunk][qz]
// [16 n][8 k] -- so the planes an input plane reaches, i in [max(0, -s), min(ZC, kz - s))
// with s = Z + rz - z_in, are one contiguous B operand (a descriptor offset) and the MMA's
// D operand starts at TMEM column 16 * i_first: one M128 x N(16..128) x K16 MMA serves up to
// ZC output planes, where the per-plane kernel needs one N16 MMA per plane. Every A tile is
// thus read once per ZC outputs instead of once per output plane.
//
// TMEM holds ZC x 16 FP32 columns, zeroed with tcgen05.st first so that every MMA
// accumulates. All T matrices (ky x 4 x kz KB) are loaded once per CTA by bulk copies; input
// planes stream through three TMA stages. Warp specialised: one thread of warp 4 issues the
// loads and MMAs and, once the last input plane reaching output plane i has been issued,
// commits plane i to its own mbarrier; eight epilogue warps (one TMEM lane = one output row,
// two warps per lane quarter, each taking 8 of the plane's 16 columns) finish plane i meanwhile
// -- read its columns and hand each thread's 8 voxels to the pass epilogue (EpiRatioTc /
// EpiUpdateTc row_pre<8>: vector loads issued a plane ahead, vector stores) -- so the epilogue of the early planes
// overlaps the MMAs of the later ones.
#pragma once

#include "rl_tc.cuh"

namespace iane_gb {

constexpr int kTczZ = 8;         // output planes per CTA
constexpr int kTczStages = 3;
constexpr int kTczChunks = 4;    // 8-column chunks of the A tile (32 input columns)

inline __host__ __device__ size_t tcz_tmat_bytes(int ky, int kz) { return static_cast<size_t>(ky) * kTczChunks * kz * 256; }
inline __host__ __device__ size_t tcz_tile_bytes(int ky) { return static_cast<size_t>(kTczChunks) * tc_rows(ky) * 16; }
inline size_t tcz_smem_bytes(int ky, int kz)
{
	return tcz_tmat_bytes(ky, kz) + kTczStages * tcz_tile_bytes(ky) + (2 * kTczStages + 1 + kTczZ + 1) * 8 + 16;
}
// warps 0-3 and 5-8: epilogue, warp w reading TMEM lanes 32 (w % 4) .. + 31 (a warp may only
// read its own lane quarter) and columns 8 (w > 4) .. + 7 of each plane; warp 4: loads and MMAs
constexpr int kTczThreads = 288;

__device__ __forceinline__ void tmem_st_zero16(uint32_t taddr)
{
	asm volatile(
		"tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1};"
		::"r"(taddr), "r"(0u)
		: "memory");
}

template<class Epi>
__global__ void __launch_bounds__(kTczThreads) tcz_conv_kernel(const __grid_constant__ CUtensorMap map, const TcArgs a,
	const Epi epi_in)
{
	extern __shared__ __align__(128) unsigned char smem_raw[];
	const int tid = threadIdx.x;
	const int warp = tid >> 5, lane = tid & 31;
	const int ky = a.ky, kz = a.kz;
	const int ry = ky / 2, rz = kz / 2;
	const int H = tc_rows(ky);
	const uint32_t chunk_bytes = static_cast<uint32_t>(H) * 16;
	const uint32_t tile_bytes = chunk_bytes * kTczChunks;
	const uint32_t tmat_bytes = static_cast<uint32_t>(tcz_tmat_bytes(ky, kz));
	const int x0 = blockIdx.x * 16, y0 = blockIdx.y * kTcM, Z = blockIdx.z * kTczZ;
	const int nout = min(kTczZ, a.nz - Z); // output planes of this block
	// input planes that reach them and lie in the volume (zero border: the others add nothing)
	const int zin_lo = max(0, Z - rz);
	const int zin_hi = min(a.nz - 1, Z + nout - 1 + rz);
	const int np = zin_hi - zin_lo + 1;

	unsigned char* tmat_s = smem_raw;
	unsigned char* stages = smem_raw + tmat_bytes;
	uint64_t* bars = reinterpret_cast<uint64_t*>(stages + kTczStages * tile_bytes);
	uint64_t* full = bars;
	uint64_t* empty = bars + kTczStages;
	uint64_t* tmat_bar = bars + 2 * kTczStages;
	uint64_t* plane_bar = tmat_bar + 1;   // [kTczZ]: output plane i's accumulators are final
	uint32_t& tmem_base_s = *reinterpret_cast<uint32_t*>(plane_bar + kTczZ);
	constexpr uint32_t kCols = kTczZ * 16;

	if (warp == 0) {
		tc::tmem_alloc(&tmem_base_s, kCols);
	}
	if (tid == 0) {
		for (int s = 0; s < 2 * kTczStages + 1 + kTczZ; ++s) mbar_init(&bars[s], 1);
		fence_barrier_init();
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tmem = tmem_base_s;
	// zero the accumulators (warps 0-3, one TMEM lane quarter each): every MMA accumulates
	const uint32_t lane_base = static_cast<uint32_t>(32 * (warp & 3)) << 16;
	if (warp < 4) {
#pragma unroll
		for (int c = 0; c < static_cast<int>(kCols); c += 16) tmem_st_zero16(tmem + lane_base + c);
		asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();

	if (tid == 128) {
		bool ok = true;
		// all T matrices, one bulk copy per kernel row
		mbar_arrive_expect_tx(tmat_bar, tmat_bytes);
		const uint32_t row_bytes = tmat_bytes / ky;
		for (int b = 0; b < ky; ++b) {
			tc::bulk_load(tmat_s + b * row_bytes, reinterpret_cast<const unsigned char*>(a.tmat) + b * row_bytes, row_bytes,
				tmat_bar);
		}
		auto load = [&](int p) {
			const int s = p % kTczStages;
			unsigned char* st = stages + s * tile_bytes;
			mbar_arrive_expect_tx(&full[s], tile_bytes);
			for (int c = 0; c < kTczChunks; ++c) {
				tma_load_3d(st + c * chunk_bytes, &map, x0 - kTcXA + 8 * c, y0 - ry, zin_lo + p, &full[s]);
			}
		};
		for (int p = 0; p < kTczStages && p < np; ++p) load(p);
		if (!mbar_wait_bounded(tmat_bar, 0)) {
			ok = false;
			report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
		}
		const uint32_t tm = smem_addr(tmat_s);
		const uint32_t lbo_b = static_cast<uint32_t>(kz) * 256;   // next 8-column K chunk
		for (int p = 0; p < np; ++p) {
			const int s = p % kTczStages;
			if (ok && !mbar_wait_bounded(&full[s], (p / kTczStages) & 1)) {
				ok = false;
				report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
			}
			tc::fence_after_sync();
			const int z_in = zin_lo + p;
			const int sh = Z + rz - z_in;                          // qz = i + sh
			const int i0 = max(0, -sh), i1 = min(nout, kz - sh);  // output planes reached
			if (i1 > i0) {
				const uint32_t idesc = tc::idesc_bf16_f32(kTcM, 16 * (i1 - i0));
				const uint32_t tile = smem_addr(stages + s * tile_bytes);
				for (int b = 0; b < ky; ++b) {
					const uint32_t a_row = tile + static_cast<uint32_t>(2 * ry - b) * 16;
					const uint32_t b_row = tm + static_cast<uint32_t>(b) * kTczChunks * lbo_b +
						static_cast<uint32_t>(i0 + sh) * 256;
#pragma unroll
					for (int ks = 0; ks < 2; ++ks) {
						const uint64_t ad = tc::smem_desc(a_row + 2 * ks * chunk_bytes, chunk_bytes, 128);
						const uint64_t bd = tc::smem_desc(b_row + 2 * ks * lbo_b, lbo_b, 128);
						tc::mma_bf16(tmem + 16 * i0, ad, bd, idesc, true);
					}
				}
			}
			tc::commit(&empty[s]);
			// output planes whose last input plane this was are final once these MMAs finish
			for (int i = 0; i < nout; ++i) {
				if (min(zin_hi, Z + i + rz) - zin_lo == p) tc::commit(&plane_bar[i]);
			}
			// the previous plane's stage is free once its MMAs finish: refill it
			if (p >= 1 && p - 1 + kTczStages < np) {
				const int sp = (p - 1) % kTczStages;
				if (ok && !mbar_wait_bounded(&empty[sp], ((p - 1) / kTczStages) & 1)) {
					ok = false;
					report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
				}
				load(p - 1 + kTczStages);
			}
		}
	}
	// Epilogue (warps 0-3 and 5-8), one output plane at a time as its accumulators become
	// final: the thread holds row y0 + 32 (warp % 4) + lane and 8 consecutive columns of it
	// and finishes them with 16-byte loads and stores. The memory operand of plane i + 1 (the
	// observed row, or the old estimate) is loaded before the wait for plane i, so its latency
	// overlaps the MMAs instead of following them.
	Epi epi = epi_in;
	if (warp != 4) {
		const int quarter = warp & 3, half = warp > 4 ? 1 : 0;
		const uint32_t lanes = static_cast<uint32_t>(32 * quarter) << 16;
		const int ex = x0 + 8 * half, ey = y0 + 32 * quarter + lane;
		float next[8] = {};
		if (nout > 0) epi.template preload<8>(ex, ey, Z, next);
		for (int i = 0; i < nout; ++i) {
			float cur[8];
#pragma unroll
			for (int c = 0; c < 8; ++c) cur[c] = next[c];
			if (i + 1 < nout) epi.template preload<8>(ex, ey, Z + i + 1, next);
			if (!mbar_wait_bounded(&plane_bar[i], 0)) {
				report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
			}
			__syncwarp(); // tcgen05.ld is warp-collective
			tc::fence_after_sync();
			float v[8];
			tc::ld_32x32b_x8(tmem + lanes + 16 * i + 8 * half, v);
			epi.template row_pre<8>(ex, ey, Z + i, v, cur);
		}
	}
	tc::fence_before_sync();
	__syncthreads();
	if (warp == 0) {
		tc::tmem_dealloc(tmem, kCols);
	}
	epi.finish();
}

}  // namespace iane_gb
