// BF16 tensor-core convolution for the Richardson-Lucy precision path (tcgen05 implicit GEMM
// with FP32 accumulation in TMEM).
//
// Banded-Toeplitz formulation. For one kernel row (b, qz) the contribution to a block of
// output rows is a GEMM:
//     D[m, n] += sum_k A[m, k] * T_{b,qz}[k, n]
// with m = 128 consecutive output rows y at one z, n = 16 consecutive output columns x,
// k = 32 input columns x_in = x0 + 16 j - 8 + k, A = the input plane's halo tile and
// T_{b,qz}[k, n] = psf[qz][b][n + rx + 8 - k] (zero outside the kernel): the PSF row
// written as a band. One CTA covers 128 (y) x 64 (x) outputs of one z plane with four such
// 16-column accumulators (64 TMEM columns) and sums all kernel rows into them.
//
// Shared-memory layout of a halo tile ("chunk-major"): for each 8-element x chunk c, all
// rows are stored at 16-byte stride, chunk after chunk. Every 8 consecutive rows of a chunk
// then form a 128-byte core matrix, so the A operand of kernel row b -- the same tile
// shifted down by 2 ry - b rows -- is the same descriptor with its start moved by
// (2 ry - b) * 16 bytes; no data is rearranged. Each chunk column is one TMA box {8, H}.
// The T matrices of a kernel plane (ky x 1 KB, precomputed at prepare) arrive by one 1-D
// bulk copy beside the tile. Three stages double-buffer TMA/bulk loads against the MMAs of
// the previous plane; one elected thread issues both, the four warps run the epilogue.
#pragma once

#include "rl.cuh"
#include "tc.cuh"

namespace iane_gb {

constexpr int kTcM = 128;     // output rows (y) per CTA
constexpr int kTcN = 64;      // output columns (x) per CTA
constexpr int kTcJ = 4;       // 16-column accumulators
constexpr int kTcXA = 8;      // x halo rounded to 8 elements (16 bytes)
constexpr int kTcChunks = (kTcN + 2 * kTcXA) / 8;  // 10
constexpr int kTcStages = 3;
constexpr int kTcTmatBytes = 32 * 16 * 2;          // one T matrix (K 32 x N 16 bf16)
constexpr int kTcTmemCols = 64;

inline __host__ __device__ int tc_rows(int ky) { return (kTcM + 2 * (ky / 2) + 7) & ~7; }

inline __host__ __device__ size_t tc_stage_bytes(int ky)
{
	const size_t tile = static_cast<size_t>(kTcChunks) * tc_rows(ky) * 16;
	return (tile + static_cast<size_t>(ky) * kTcTmatBytes + 127) & ~size_t(127);
}

// Shared memory the stages and barriers need.
inline size_t tc_smem_bytes(int ky) { return kTcStages * tc_stage_bytes(ky) + (2 * kTcStages + 2) * 8; }

struct TcArgs {
	int nx, ny, nz;
	int ky, kz;
	const __nv_bfloat16* tmat; // [kz][ky][4 chunks][16 n][8 k] bf16
	int* status;
	int smem_bytes;            // dynamic shared memory of the launch (>= the stages)
	int tmem_cols;             // TMEM columns to allocate (>= kTcTmemCols)
};

template<class Epi>
__global__ void __launch_bounds__(128, 2) tc_conv_kernel(const __grid_constant__ CUtensorMap map, const TcArgs a,
	const Epi epi_in)
{
	extern __shared__ __align__(128) unsigned char smem_raw[];

	const int tid = threadIdx.x;
	const int warp = tid >> 5, lane = tid & 31;
	const int ky = a.ky, kz = a.kz;
	const int ry = ky / 2, rz = kz / 2;
	const int H = tc_rows(ky);
	const uint32_t chunk_bytes = static_cast<uint32_t>(H) * 16;
	const uint32_t tile_bytes = chunk_bytes * kTcChunks;
	const uint32_t tmat_bytes = static_cast<uint32_t>(ky) * kTcTmatBytes;
	const size_t stage_bytes = tc_stage_bytes(ky);
	const int x0 = blockIdx.x * kTcN, y0 = blockIdx.y * kTcM, z = blockIdx.z;
	const int qz_lo = max(0, z + rz - (a.nz - 1));
	const int qz_hi = min(kz - 1, z + rz);
	const int np = qz_hi - qz_lo + 1;
	// after the stages: full[s], empty[s], done, then the TMEM base address
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + kTcStages * stage_bytes);
	uint32_t& tmem_base_s = *reinterpret_cast<uint32_t*>(bars + 2 * kTcStages + 1);
	uint64_t* full = bars;
	uint64_t* empty = bars + kTcStages;
	uint64_t* done = bars + 2 * kTcStages;

	if (warp == 0) {
		tc::tmem_alloc(&tmem_base_s, static_cast<uint32_t>(a.tmem_cols));
	}
	if (tid == 0) {
		for (int s = 0; s < 2 * kTcStages + 1; ++s) mbar_init(&bars[s], 1);
		fence_barrier_init();
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tmem = tmem_base_s;

	if (tid == 0) {
		const uint32_t idesc = tc::idesc_bf16_f32(kTcM, 16);
		auto stage_ptr = [&](int s) { return smem_raw + s * stage_bytes; };
		auto load = [&](int p) {
			const int s = p % kTcStages;
			const int qz = qz_lo + p;
			unsigned char* st = stage_ptr(s);
			mbar_arrive_expect_tx(&full[s], tile_bytes + tmat_bytes);
			for (int c = 0; c < kTcChunks; ++c) {
				tma_load_3d(st + c * chunk_bytes, &map, x0 - kTcXA + 8 * c, y0 - ry, z + rz - qz, &full[s]);
			}
			tc::bulk_load(st + tile_bytes, a.tmat + static_cast<size_t>(qz) * ky * (kTcTmatBytes / 2), tmat_bytes, &full[s]);
		};
		bool ok = true;
		for (int p = 0; p < kTcStages && p < np; ++p) load(p);
		for (int p = 0; p < np; ++p) {
			const int s = p % kTcStages;
			if (ok && !mbar_wait_bounded(&full[s], (p / kTcStages) & 1)) {
				ok = false;
				report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
			}
			tc::fence_after_sync();
			const uint32_t tile = smem_addr(stage_ptr(s));
			const uint32_t tm = tile + tile_bytes;
			for (int b = 0; b < ky; ++b) {
				const uint32_t a_row = tile + static_cast<uint32_t>(2 * ry - b) * 16;
				const uint32_t b_mat = tm + static_cast<uint32_t>(b) * kTcTmatBytes;
#pragma unroll
				for (int j = 0; j < kTcJ; ++j) {
#pragma unroll
					for (int ks = 0; ks < 2; ++ks) {
						const uint64_t ad = tc::smem_desc(a_row + (2 * j + 2 * ks) * chunk_bytes, chunk_bytes, 128);
						const uint64_t bd = tc::smem_desc(b_mat + ks * 512, 256, 128);
						tc::mma_bf16(tmem + 16 * j, ad, bd, idesc, p > 0 || b > 0 || ks > 0);
					}
				}
			}
			tc::commit(&empty[s]);
			// the previous plane's stage is free once its MMAs finish: refill it
			if (p >= 1 && p - 1 + kTcStages < np) {
				const int sp = (p - 1) % kTcStages;
				if (ok && !mbar_wait_bounded(&empty[sp], ((p - 1) / kTcStages) & 1)) {
					ok = false;
					report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
				}
				load(p - 1 + kTcStages);
			}
		}
		tc::commit(done);
	}
	__syncwarp();
	// epilogue: lane l of warp w owns output row y0 + 32 w + l, columns x0 .. x0 + 63
	if (!mbar_wait_bounded(done, 0)) {
		report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
	}
	__syncwarp(); // tcgen05.ld is warp-collective
	tc::fence_after_sync();
	float v[kTcN];
#pragma unroll
	for (int j = 0; j < kTcJ; ++j) {
		float part[16];
		tc::ld_32x32b_x16(tmem + (static_cast<uint32_t>(32 * warp) << 16) + 16 * j, part);
#pragma unroll
		for (int i = 0; i < 16; ++i) v[16 * j + i] = part[i];
	}
	tc::fence_before_sync();
	__syncthreads();
	if (warp == 0) {
		tc::tmem_dealloc(tmem, static_cast<uint32_t>(a.tmem_cols));
	}
	Epi epi = epi_in;
	epi.row(x0, y0 + 32 * warp + lane, z, v);
	epi.finish();
}

// ---------------------------------------------------------------------------------------
// epilogues

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi)
{
	const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
	return *reinterpret_cast<const uint32_t*>(&p);
}

// pass A: ratio = observed / max(pred, eps), stored as bf16 (the next convolution's input)
struct EpiRatioTc {
	__nv_bfloat16* ratio;
	long long pitch, plane; // elements
	const char* obs;
	long long os[3];
	int obs_u8;
	float eps;
	int nx, ny;

	__device__ __forceinline__ void row(int x0, int y, int z, const float (&v)[kTcN]) const
	{
		if (y >= ny) return;
		__nv_bfloat16* out = ratio + z * plane + y * pitch + x0;
		const char* orow = obs + y * os[1] + z * os[2];
#pragma unroll
		for (int g = 0; g < kTcN / 8; ++g) {
			float r[8];
#pragma unroll
			for (int i = 0; i < 8; ++i) {
				const int x = x0 + 8 * g + i;
				float o = 0.0f;
				if (x < nx) {
					const char* p = orow + x * os[0];
					o = obs_u8 ? static_cast<float>(*reinterpret_cast<const uint8_t*>(p)) : *reinterpret_cast<const float*>(p);
				}
				const float pr = v[8 * g + i];
				r[i] = o / (pr > eps ? pr : eps);
			}
			if (x0 + 8 * g + 8 <= nx) {
				uint4 pk = make_uint4(pack_bf16x2(r[0], r[1]), pack_bf16x2(r[2], r[3]), pack_bf16x2(r[4], r[5]),
					pack_bf16x2(r[6], r[7]));
				*reinterpret_cast<uint4*>(out + 8 * g) = pk;
			} else {
#pragma unroll
				for (int i = 0; i < 8; ++i) {
					if (x0 + 8 * g + i < nx) out[8 * g + i] = __float2bfloat16_rn(r[i]);
				}
			}
		}
	}
	__device__ __forceinline__ void finish() const {}
};

// pass B: estimate *= edge(conv(ratio, adjoint), sensitivity); the FP32 estimate is the
// master copy, its bf16 shadow feeds the next pass A.
struct EpiUpdateTc {
	float* est;
	long long pitch, plane;
	__nv_bfloat16* est16;
	long long pitch16, plane16;
	float eps;
	int nx, ny, nz;
	const int* cls;
	const float* sens;
	int cx_count, cy_count;
	int ilo[3], ihi[3];
	float s_interior;
	int want_stats;
	double* partials;
	unsigned int* counter;
	double* stats;
	int write_out;
	char* out;
	long long outs[3];
	int out_u8;
	float f_s, f_c, c_s, c_c, n_s, n_c;

	__device__ __forceinline__ void row(int x0, int y, int z, const float (&v)[kTcN])
	{
		if (y >= ny) return;
		const bool rows_in = y >= ilo[1] && y <= ihi[1] && z >= ilo[2] && z <= ihi[2];
		const int cyz = cx_count * (cls[nx + y] + cy_count * cls[nx + ny + z]);
		float* e = est + z * plane + y * pitch + x0;
		__nv_bfloat16* e16 = est16 + z * plane16 + y * pitch16 + x0;
#pragma unroll
		for (int g = 0; g < kTcN / 8; ++g) {
			const bool full = x0 + 8 * g + 8 <= nx;
			float old[8], upd[8];
			if (full) {
				const float4 p0 = reinterpret_cast<const float4*>(e + 8 * g)[0];
				const float4 p1 = reinterpret_cast<const float4*>(e + 8 * g)[1];
				old[0] = p0.x; old[1] = p0.y; old[2] = p0.z; old[3] = p0.w;
				old[4] = p1.x; old[5] = p1.y; old[6] = p1.z; old[7] = p1.w;
			} else {
#pragma unroll
				for (int i = 0; i < 8; ++i) old[i] = x0 + 8 * g + i < nx ? e[8 * g + i] : 0.0f;
			}
#pragma unroll
			for (int i = 0; i < 8; ++i) {
				const int x = x0 + 8 * g + i;
				float s = s_interior;
				if (!(rows_in && x >= ilo[0] && x <= ihi[0]) && x < nx) s = sens[cls[x] + cyz];
				const float factor = s > 0.0f ? v[8 * g + i] / (s > eps ? s : eps) : 0.0f;
				upd[i] = old[i] * factor;
			}
			if (full) {
				reinterpret_cast<float4*>(e + 8 * g)[0] = make_float4(upd[0], upd[1], upd[2], upd[3]);
				reinterpret_cast<float4*>(e + 8 * g)[1] = make_float4(upd[4], upd[5], upd[6], upd[7]);
				*reinterpret_cast<uint4*>(e16 + 8 * g) = make_uint4(pack_bf16x2(upd[0], upd[1]),
					pack_bf16x2(upd[2], upd[3]), pack_bf16x2(upd[4], upd[5]), pack_bf16x2(upd[6], upd[7]));
			}
#pragma unroll
			for (int i = 0; i < 8; ++i) {
				const int x = x0 + 8 * g + i;
				if (x >= nx) continue;
				if (!full) {
					e[8 * g + i] = upd[i];
					e16[8 * g + i] = __float2bfloat16_rn(upd[i]);
				}
				if (want_stats) {
					kahan_add(f_s, f_c, upd[i]);
					const float d = upd[i] - old[i];
					kahan_add(c_s, c_c, d * d);
					kahan_add(n_s, n_c, old[i] * old[i]);
				}
				if (write_out) {
					char* p = out + x * outs[0] + y * outs[1] + z * outs[2];
					if (out_u8) {
						*reinterpret_cast<uint8_t*>(p) = to_gray8(upd[i]);
					} else {
						*reinterpret_cast<float*>(p) = upd[i];
					}
				}
			}
		}
	}

	__device__ void finish()
	{
		// same reduction as the FP32 path's EpiUpdate
		EpiUpdate r{};
		r.want_stats = want_stats;
		r.partials = partials;
		r.counter = counter;
		r.stats = stats;
		r.f_s = f_s; r.f_c = f_c; r.c_s = c_s; r.c_c = c_c; r.n_s = n_s; r.n_c = n_c;
		r.finish();
	}
};

int launch_tc_pass_a(const CUtensorMap& map, const TcArgs& a, const EpiRatioTc& e, cudaStream_t stream);
int launch_tc_pass_b(const CUtensorMap& map, const TcArgs& a, const EpiUpdateTc& e, cudaStream_t stream);

}  // namespace iane_gb
