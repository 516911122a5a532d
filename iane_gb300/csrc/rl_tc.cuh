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
	// Transpose through shared memory (the stages are idle now): thread = row above, warp =
	// row below, so that every global access of the epilogue is a coalesced row segment.
	float* E = reinterpret_cast<float*>(smem_raw);
	constexpr int EP = kTcN + 1; // pitch: thread t writes row t without bank conflicts
#pragma unroll
	for (int i = 0; i < kTcN; ++i) E[tid * EP + i] = v[i];
	__syncthreads();
	if (warp == 0) {
		tc::tmem_dealloc(tmem, static_cast<uint32_t>(a.tmem_cols));
	}
	Epi epi = epi_in;
	for (int r = warp; r < kTcM; r += 4) {
		epi.row_pair(x0 + lane, y0 + r, z, E[r * EP + lane], E[r * EP + lane + 32]);
	}
	epi.finish();
}

// ---------------------------------------------------------------------------------------
// epilogues

// pass A: ratio = observed / max(pred, eps), stored as bf16 (the next convolution's input)
struct EpiRatioTc {
	__nv_bfloat16* ratio;
	long long pitch, plane; // elements
	const char* obs;
	long long os[3];
	int obs_u8;
	float eps;
	int nx, ny;

	// one output voxel (x, y, z) with prediction pr
	__device__ __forceinline__ void one(int xx, int y, int z, float pr) const
	{
		if (y >= ny || xx >= nx) return;
		const char* q = obs + xx * os[0] + y * os[1] + z * os[2];
		const float o = obs_u8 ? static_cast<float>(*reinterpret_cast<const uint8_t*>(q)) : *reinterpret_cast<const float*>(q);
		ratio[z * plane + y * pitch + xx] = __float2bfloat16_rn(o / (pr > eps ? pr : eps));
	}

	// one warp, one row: this lane's columns x and x + 32
	__device__ __forceinline__ void row_pair(int x, int y, int z, float p0, float p1) const
	{
		one(x, y, z, p0);
		one(x + 32, y, z, p1);
	}

	// whether N consecutive outputs from x0 (a multiple of N) of row y take the vector path: the
	// run lies inside the image and the observed row is f32 and 16-byte aligned
	template<int N>
	__device__ __forceinline__ bool vector_run(int x0, int y, int z) const
	{
		const char* orow = obs + y * os[1] + z * os[2] + x0 * os[0];
		return y < ny && x0 + N <= nx && !obs_u8 && os[0] == 4 && (reinterpret_cast<uintptr_t>(orow) & 15) == 0;
	}

	// The observed values the vector path of row_pre<N> needs, loaded ahead of time (callers
	// issue them before they wait for the accumulators); nothing is read off the vector path.
	template<int N>
	__device__ __forceinline__ void preload(int x0, int y, int z, float (&o)[N]) const
	{
		if (!vector_run<N>(x0, y, z)) return;
		const char* orow = obs + y * os[1] + z * os[2] + x0 * os[0];
#pragma unroll
		for (int q = 0; q < N / 4; ++q) {
			const float4 v = *reinterpret_cast<const float4*>(orow + 16 * q);
			o[4 * q] = v.x;
			o[4 * q + 1] = v.y;
			o[4 * q + 2] = v.z;
			o[4 * q + 3] = v.w;
		}
	}

	// N (8 or 16) consecutive outputs x0 .. x0 + N - 1 of row y with their observed values o
	// from preload<N>: vector loads and stores on the vector path, one voxel at a time otherwise
	template<int N>
	__device__ __forceinline__ void row_pre(int x0, int y, int z, const float (&pr)[N], const float (&o)[N]) const
	{
		if (y >= ny) return;
		if (vector_run<N>(x0, y, z)) {
			uint32_t w[N / 2];
#pragma unroll
			for (int c = 0; c < N / 2; ++c) {
				const float r0 = o[2 * c] / (pr[2 * c] > eps ? pr[2 * c] : eps);
				const float r1 = o[2 * c + 1] / (pr[2 * c + 1] > eps ? pr[2 * c + 1] : eps);
				const __nv_bfloat162 h = __floats2bfloat162_rn(r0, r1);
				w[c] = *reinterpret_cast<const uint32_t*>(&h);
			}
			uint4* dst = reinterpret_cast<uint4*>(ratio + z * plane + y * pitch + x0);
#pragma unroll
			for (int q = 0; q < N / 8; ++q) dst[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
			return;
		}
#pragma unroll
		for (int c = 0; c < N; ++c) one(x0 + c, y, z, pr[c]);
	}

	template<int N>
	__device__ __forceinline__ void row_n(int x0, int y, int z, const float (&pr)[N]) const
	{
		float o[N] = {};
		preload<N>(x0, y, z, o);
		row_pre<N>(x0, y, z, pr, o);
	}
	__device__ __forceinline__ void row16(int x0, int y, int z, const float (&pr)[16]) const { row_n<16>(x0, y, z, pr); }
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

	// one output voxel (x, y, z) with correction cv
	__device__ __forceinline__ void one(int xx, int y, int z, float cv)
	{
		if (y >= ny || xx >= nx) return;
		const bool in = xx >= ilo[0] && xx <= ihi[0] && y >= ilo[1] && y <= ihi[1] && z >= ilo[2] && z <= ihi[2];
		const float s = in ? s_interior : sens[cls[xx] + cx_count * (cls[nx + y] + cy_count * cls[nx + ny + z])];
		const float factor = s > 0.0f ? cv / (s > eps ? s : eps) : 0.0f;
		float* e = est + z * plane + y * pitch + xx;
		const float old = *e;
		const float upd = old * factor;
		*e = upd;
		est16[z * plane16 + y * pitch16 + xx] = __float2bfloat16_rn(upd);
		if (want_stats) {
			kahan_add(f_s, f_c, upd);
			const float d = upd - old;
			kahan_add(c_s, c_c, d * d);
			kahan_add(n_s, n_c, old * old);
		}
		if (write_out) {
			char* q = out + xx * outs[0] + y * outs[1] + z * outs[2];
			if (out_u8) {
				*reinterpret_cast<uint8_t*>(q) = to_gray8(upd);
			} else {
				*reinterpret_cast<float*>(q) = upd;
			}
		}
	}

	// one warp, one row: this lane's columns x and x + 32
	__device__ __forceinline__ void row_pair(int x, int y, int z, float c0, float c1)
	{
		one(x, y, z, c0);
		one(x + 32, y, z, c1);
	}

	// whether N consecutive outputs from x0 (a multiple of N) of row y take the vector path: the
	// run lies inside the image and no final copy to the caller's view is due
	template<int N>
	__device__ __forceinline__ bool vector_run(int x0, int y) const
	{
		return y < ny && x0 + N <= nx && !write_out;
	}

	// The old estimate values the vector path of row_pre<N> needs, loaded ahead of time
	// (callers issue them before they wait for the accumulators; the thread alone owns these
	// voxels); nothing is read off the vector path.
	template<int N>
	__device__ __forceinline__ void preload(int x0, int y, int z, float (&old)[N]) const
	{
		if (!vector_run<N>(x0, y)) return;
		const float* e = est + z * plane + y * pitch + x0;  // rows are 16-byte aligned, x0 % 8 == 0
#pragma unroll
		for (int q = 0; q < N / 4; ++q) {
			const float4 v = reinterpret_cast<const float4*>(e)[q];
			old[4 * q] = v.x;
			old[4 * q + 1] = v.y;
			old[4 * q + 2] = v.z;
			old[4 * q + 3] = v.w;
		}
	}

	// N (8 or 16) consecutive outputs x0 .. x0 + N - 1 of row y with their old estimate values
	// from preload<N>: vector stores of the estimate and its BF16 shadow on the vector path, one
	// voxel at a time otherwise
	template<int N>
	__device__ __forceinline__ void row_pre(int x0, int y, int z, const float (&cv)[N], const float (&old)[N])
	{
		if (y >= ny) return;
		if (!vector_run<N>(x0, y)) {
#pragma unroll
			for (int c = 0; c < N; ++c) one(x0 + c, y, z, cv[c]);
			return;
		}
		const bool rows_in = y >= ilo[1] && y <= ihi[1] && z >= ilo[2] && z <= ihi[2];
		const bool all_in = rows_in && x0 >= ilo[0] && x0 + N - 1 <= ihi[0];
		const int cyz = cx_count * (cls[nx + y] + cy_count * cls[nx + ny + z]);
		float* e = est + z * plane + y * pitch + x0;
		float upd[N];
#pragma unroll
		for (int c = 0; c < N; ++c) {
			float sv = s_interior;
			if (!all_in && !(rows_in && x0 + c >= ilo[0] && x0 + c <= ihi[0])) sv = sens[cls[x0 + c] + cyz];
			const float factor = sv > 0.0f ? cv[c] / (sv > eps ? sv : eps) : 0.0f;
			upd[c] = old[c] * factor;
			if (want_stats) {
				kahan_add(f_s, f_c, upd[c]);
				const float d = upd[c] - old[c];
				kahan_add(c_s, c_c, d * d);
				kahan_add(n_s, n_c, old[c] * old[c]);
			}
		}
#pragma unroll
		for (int q = 0; q < N / 4; ++q) {
			reinterpret_cast<float4*>(e)[q] = make_float4(upd[4 * q], upd[4 * q + 1], upd[4 * q + 2], upd[4 * q + 3]);
		}
		uint32_t w[N / 2];
#pragma unroll
		for (int c = 0; c < N / 2; ++c) {
			const __nv_bfloat162 h = __floats2bfloat162_rn(upd[2 * c], upd[2 * c + 1]);
			w[c] = *reinterpret_cast<const uint32_t*>(&h);
		}
		uint4* d16 = reinterpret_cast<uint4*>(est16 + z * plane16 + y * pitch16 + x0);
#pragma unroll
		for (int q = 0; q < N / 8; ++q) d16[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
	}

	template<int N>
	__device__ __forceinline__ void row_n(int x0, int y, int z, const float (&cv)[N])
	{
		float old[N] = {};
		preload<N>(x0, y, z, old);
		row_pre<N>(x0, y, z, cv, old);
	}
	__device__ __forceinline__ void row16(int x0, int y, int z, const float (&cv)[16]) { row_n<16>(x0, y, z, cv); }

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
// The z-planes-along-N variant (rl_tcz.cuh): PSFs whose T matrices fit in shared memory.
bool tcz_supported(int kx, int ky, int kz);
int launch_tcz_pass_a(const CUtensorMap& map, const TcArgs& a, const EpiRatioTc& e, cudaStream_t stream);
int launch_tcz_pass_b(const CUtensorMap& map, const TcArgs& a, const EpiUpdateTc& e, cudaStream_t stream);

}  // namespace iane_gb
