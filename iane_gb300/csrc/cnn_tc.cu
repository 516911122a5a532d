// Tensor-core forward 3x3x3 convolution of the warm-start CNN (tcgen05 implicit GEMM, BF16
// operands, FP32 accumulation in TMEM).
//
// Per CTA: a block of 16 (x) x 8 (y) voxels on BZ consecutive z planes. For each plane the
// 128 voxels are the M rows of a GEMM with N = output channels (16, 32 or 64; padded) and
// K = input channels x taps, 16 channels per MMA:
//
//     D_tx[zb][r, n] += sum_{ty, tz, ci} A_{ty,tz}[r, ci] * W[tx, ty, tz][ci, n]
//
// where row r is the voxel (x0 - 1 + r % 16, y0 + r / 16) and A_{ty,tz} the input at that
// voxel moved by (0, ty - 1, zb + tz - 1). The x tap is NOT applied to the operand: each tx
// has its own accumulator and the epilogue forms out[r] = D_0[r - 1] + D_1[r] + D_2[r + 1]
// by lane shuffles, so rows r % 16 in 1..14 are outputs (14 columns per block) and the A
// operand of every tap is the same shared-memory tile at a row offset -- a descriptor start
// address, no data movement. Because the three tx accumulators share that A operand, the
// weights of the three x taps are stacked along N: one MMA of N = 3 x (16, 32 or 64) per
// (ty, tz) fills D_0 | D_1 | D_2 side by side in TMEM. (Three separate N-wide MMAs would read
// the 4 KB A tile from shared memory three times; at N = 16 those operand reads, not the
// math, bound the kernel.)
//
// Input tile: one 5-D TMA box of the C8 activation tensor, dims (8 channels, x, y, z,
// octet), box (8, 16, 10, BZ + 2, 2) -> shared memory [octet][z][y][x][8 channels]: every 8
// consecutive voxels of an octet are one 128-byte K-major core matrix (LBO = the octet
// stride, SBO = 128 bytes). Out-of-range voxels and octets arrive as zeros (the padding).
// BZ = 2 planes per block; TMEM holds 3 x BZ x N columns (128, 256 or 512 for N = 16, 32,
// 64), which also sets how many CTAs share an SM (4, 2, 1).
// Weights: packed per 16-channel step as [ty, tz][8-channel half][tx][n][8] (a K-major
// 3N x 16 operand per (ty, tz)), one 1-D bulk copy per step. Two stages; one thread issues TMA and MMAs,
// four warps run the epilogue (bias, ReLU, BF16 C8 store or FP32 planar store + residual).
#include "common.cuh"
#include "tc.cuh"

#include <cstdint>

namespace iane_gb {
namespace {

constexpr int TX = 16, TY = 8;           // voxels per M tile (x, y)
constexpr int OUT_X = 14;                // output columns per block
constexpr int HY = TY + 2;               // halo rows
constexpr int MAX_STAGES = 2;

__device__ __forceinline__ uint16_t to_bf16(float f)
{
	const __nv_bfloat16 b = __float2bfloat16_rn(f);
	return *reinterpret_cast<const uint16_t*>(&b);
}

__host__ __device__ constexpr int a_bytes(int bz) { return 2 * (bz + 2) * HY * TX * 16; }
__host__ __device__ constexpr int b_bytes(int n) { return 27 * 2 * n * 16; }
__host__ __device__ constexpr int stage_bytes(int n, int bz) { return a_bytes(bz) + b_bytes(n); }
__host__ __device__ constexpr int tmem_cols(int n, int bz)
{
	return 3 * bz * n <= 32 ? 32 : (3 * bz * n <= 64 ? 64 : (3 * bz * n <= 128 ? 128 : (3 * bz * n <= 256 ? 256 : 512)));
}
__host__ __device__ constexpr size_t smem_total(int n, int bz, int stages) { return stages * stage_bytes(n, bz) + 8 * 8; }

struct TcConvArgs {
	int d, h, w;
	int steps0, steps;        // 16-channel K steps from x0, and in all
	const uint16_t* packed;   // [steps][9 (ty, tz)][2][3 tx][N][8]
	const float* bias;        // [co] or null
	int co;
	uint16_t* y16;            // C8 output or null
	float* y32;               // planar FP32 output or null
	const float* residual;    // planar FP32, added before the activation, or null
	int act;
	int tiles_x, tiles_y;
	int stages;               // 1 (single K step) or 2
	int* status;
};

template<int N, int BZ>
__global__ void __launch_bounds__(128) cnn_tc_conv_kernel(const __grid_constant__ CUtensorMap map0,
	const __grid_constant__ CUtensorMap map1, const TcConvArgs a)
{
	extern __shared__ __align__(128) unsigned char smem[];
	constexpr int SB = stage_bytes(N, BZ);
	constexpr int AB = a_bytes(BZ);
	constexpr uint32_t OCTET = (BZ + 2) * HY * TX * 16;  // LBO of the A operand
	constexpr int COLS = tmem_cols(N, BZ);
	const int S = a.stages;
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S * SB);
	uint64_t* full = bars;
	uint64_t* empty = bars + S;
	uint64_t* done = bars + 2 * S;
	uint32_t& tmem_base_s = *reinterpret_cast<uint32_t*>(bars + 2 * S + 1);

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int tx_i = blockIdx.x % a.tiles_x, ty_i = blockIdx.x / a.tiles_x;
	const int x0 = tx_i * OUT_X, y0 = ty_i * TY, z0 = blockIdx.y * BZ;

	if (warp == 0) tc::tmem_alloc(&tmem_base_s, COLS);
	if (tid == 0) {
		for (int s = 0; s < 2 * S + 1; ++s) mbar_init(&bars[s], 1);
		fence_barrier_init();
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tmem = tmem_base_s;

	if (tid == 0) {
		const uint32_t idesc = tc::idesc_bf16_f32(128, 3 * N);
		auto load = [&](int p) {
			unsigned char* st = smem + (p % S) * SB;
			mbar_arrive_expect_tx(&full[p % S], static_cast<uint32_t>(SB));
			if (p < a.steps0) {
				tma_load_5d(st, &map0, 0, x0 - 1, y0 - 1, z0 - 1, 2 * p, &full[p % S]);
			} else {
				tma_load_5d(st, &map1, 0, x0 - 1, y0 - 1, z0 - 1, 2 * (p - a.steps0), &full[p % S]);
			}
			tc::bulk_load(st + AB, a.packed + static_cast<size_t>(p) * (b_bytes(N) / 2), b_bytes(N), &full[p % S]);
		};
		bool ok = true;
		for (int p = 0; p < S && p < a.steps; ++p) load(p);
		for (int p = 0; p < a.steps; ++p) {
			const int s = p % S;
			if (ok && !mbar_wait_bounded(&full[s], (p / S) & 1)) {
				ok = false;
				report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
			}
			tc::fence_after_sync();
			const uint32_t a_base = smem_addr(smem + s * SB);
			const uint32_t b_base = a_base + AB;
#pragma unroll 1
			for (int zb = 0; zb < BZ; ++zb) {
#pragma unroll 1
				for (int tz = 0; tz < 3; ++tz) {
#pragma unroll
					for (int ty = 0; ty < 3; ++ty) {
						const uint32_t a_start = a_base + static_cast<uint32_t>(((zb + tz) * HY + ty) * TX * 16);
						const uint64_t ad = tc::smem_desc(a_start, OCTET, 128);
						const bool acc = p > 0 || tz > 0 || ty > 0;
						const int tyz = ty + 3 * tz;
						const uint64_t bd = tc::smem_desc(b_base + static_cast<uint32_t>(tyz * 2 * 3 * N * 16), 3 * N * 16, 128);
						tc::mma_bf16(tmem + static_cast<uint32_t>(zb * 3 * N), ad, bd, idesc, acc);
					}
				}
			}
			tc::commit(&empty[s]);
			// A stage is free once the MMAs reading it finish. Two stages: refill the previous
			// step's stage while this step's MMAs run. One stage: wait for this step's MMAs.
			const int q = S == 1 ? p : p - 1;
			if (q >= 0 && q + S < a.steps) {
				const int sq = q % S;
				if (ok && !mbar_wait_bounded(&empty[sq], (q / S) & 1)) {
					ok = false;
					report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
				}
				load(q + S);
			}
		}
		tc::commit(done);
	}
	__syncwarp();
	if (!mbar_wait_bounded(done, 0)) report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
	__syncwarp();
	tc::fence_after_sync();

	// epilogue: lane l of warp w holds row r = 32 w + l
	const int r = 32 * warp + lane;
	const int x = x0 - 1 + (r & 15), y = y0 + (r >> 4);
	const bool valid = (r & 15) >= 1 && (r & 15) <= OUT_X && x < a.w && y < a.h;
	const long long plane = static_cast<long long>(a.h) * a.w, vol = plane * a.d;
	const uint32_t lane_base = static_cast<uint32_t>(32 * warp) << 16;
#pragma unroll 1
	for (int zb = 0; zb < BZ; ++zb) {
		const int z = z0 + zb;
		const long long v = z * plane + static_cast<long long>(y) * a.w + x;
#pragma unroll 1
		for (int j = 0; j < N / 16; ++j) {
			__syncwarp(); // tcgen05.ld is warp-collective
			float d0[16], d1[16], d2[16];
			tc::ld_32x32b_x16(tmem + lane_base + static_cast<uint32_t>((zb * 3 + 0) * N + 16 * j), d0);
			tc::ld_32x32b_x16(tmem + lane_base + static_cast<uint32_t>((zb * 3 + 1) * N + 16 * j), d1);
			tc::ld_32x32b_x16(tmem + lane_base + static_cast<uint32_t>((zb * 3 + 2) * N + 16 * j), d2);
			float o[16];
#pragma unroll
			for (int i = 0; i < 16; ++i) {
				o[i] = __shfl_up_sync(0xffffffffu, d0[i], 1) + d1[i] + __shfl_down_sync(0xffffffffu, d2[i], 1);
			}
			if (valid && z < a.d) {
#pragma unroll
			for (int i = 0; i < 16; ++i) {
				const int c = 16 * j + i;
				float val = o[i] + ((a.bias && c < a.co) ? a.bias[c] : 0.0f);
				if (a.residual && c < a.co) val += a.residual[c * vol + v];
				if (a.act == 1) val = val > 0.0f ? val : 0.0f;
				o[i] = val;
				if (a.y32 && c < a.co) a.y32[c * vol + v] = val;
			}
			if (a.y16) {
#pragma unroll
				for (int h = 0; h < 2; ++h) {
					const int oct = 2 * j + h;
					if (8 * oct >= a.co) break;
					uint4 q;
					q.x = static_cast<uint32_t>(to_bf16(o[8 * h + 0])) | (static_cast<uint32_t>(to_bf16(o[8 * h + 1])) << 16);
					q.y = static_cast<uint32_t>(to_bf16(o[8 * h + 2])) | (static_cast<uint32_t>(to_bf16(o[8 * h + 3])) << 16);
					q.z = static_cast<uint32_t>(to_bf16(o[8 * h + 4])) | (static_cast<uint32_t>(to_bf16(o[8 * h + 5])) << 16);
					q.w = static_cast<uint32_t>(to_bf16(o[8 * h + 6])) | (static_cast<uint32_t>(to_bf16(o[8 * h + 7])) << 16);
					*reinterpret_cast<uint4*>(a.y16 + ((static_cast<long long>(oct) * vol + v) << 3)) = q;
				}
			}
			}
		}
	}
	tc::fence_before_sync();
	__syncthreads();
	if (warp == 0) tc::tmem_dealloc(tmem, COLS);
}

// packed[s][tyz][h][tx][n][k] = w[n][ci][tx + 3 tyz] with ci the (8 h + k)-th channel of
// step s: steps 0 .. steps0 - 1 cover x0's channels 16 s .., the rest x1's (index c0 + ...).
__global__ void pack_kernel(const uint16_t* w, int co, int c0, int c1, int n_pad, int steps0, int steps, uint16_t* packed)
{
	const long long n = static_cast<long long>(steps) * 27 * 2 * n_pad * 8;
	const int ci_total = c0 + c1;
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int k = static_cast<int>(i % 8);
		const int nn = static_cast<int>((i / 8) % n_pad);
		const int tx = static_cast<int>((i / (8LL * n_pad)) % 3);
		const int h = static_cast<int>((i / (24LL * n_pad)) % 2);
		const int tyz = static_cast<int>((i / (48LL * n_pad)) % 9);
		const int t = tx + 3 * tyz;
		const int s = static_cast<int>(i / (16LL * n_pad * 27));
		const int local = 16 * (s < steps0 ? s : s - steps0) + 8 * h + k;
		const int ci = s < steps0 ? (local < c0 ? local : -1) : (local < c1 ? c0 + local : -1);
		packed[i] = (nn < co && ci >= 0) ? w[(static_cast<long long>(nn) * ci_total + ci) * 27 + t] : 0;
	}
}

int n_pad_of(int co) { return co <= 16 ? 16 : (co <= 32 ? 32 : 64); }
int steps_of(int c) { return (c + 15) / 16; }

template<int N, int BZ>
int launch(const CUtensorMap& m0, const CUtensorMap& m1, const TcConvArgs& a, cudaStream_t st)
{
	const auto kernel = cnn_tc_conv_kernel<N, BZ>;
	static bool configured = false;
	if (!configured) {
		IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
			static_cast<int>(smem_total(N, BZ, MAX_STAGES))), "cnn_conv3_tc: shared memory attribute");
		configured = true;
	}
	// Co-resident CTAs per SM are bounded by TMEM (512 columns per SM): ask for enough shared
	// memory that no more CTAs than that land on an SM (228 KB per SM, 1 KB reserved per CTA).
	const int per_sm = 512 / tmem_cols(N, BZ);
	const size_t floor_bytes = 228 * 1024 / (per_sm + 1) - 1024 + 16;
	size_t smem = smem_total(N, BZ, a.stages);
	if (smem < floor_bytes) smem = floor_bytes;
	const dim3 grid(static_cast<unsigned>(a.tiles_x * a.tiles_y), static_cast<unsigned>((a.d + BZ - 1) / BZ));
	kernel<<<grid, 128, smem, st>>>(m0, m1, a);
	IANE_GB_CUDA(cudaGetLastError(), "cnn_conv3_tc: launch");
	return IANE_GB_OK;
}

int encode_c8_map(CUtensorMap* map, const uint16_t* base, int c, int d, int h, int w, int bz)
{
	const long long dims[5] = {8, w, h, d, (c + 7) / 8};
	const long long strides[4] = {16, 16LL * w, 16LL * w * h, 16LL * w * h * d};
	const int box[5] = {8, TX, HY, bz + 2, 2};
	return encode_tensor_map_nd(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, base, dims, strides, box);
}

}  // namespace
}  // namespace iane_gb

using namespace iane_gb;

extern "C" {

size_t iane_gb_cnn_tc_packed_bytes(int co, int c0, int c1)
{
	if (co < 1 || co > 64 || c0 < 1 || c1 < 0) return 0;
	return static_cast<size_t>(steps_of(c0) + steps_of(c1)) * b_bytes(n_pad_of(co));
}

int iane_gb_cnn_tc_pack(const uint16_t* weights, int co, int c0, int c1, uint16_t* packed, void* stream)
{
	if (!weights || !packed || co < 1 || co > 64 || c0 < 1 || c1 < 0) {
		return fail(IANE_GB_INVALID_ARGUMENT, "cnn_tc_pack: bad arguments");
	}
	const int steps0 = steps_of(c0), steps = steps0 + steps_of(c1);
	const int n_pad = n_pad_of(co);
	const long long n = static_cast<long long>(steps) * 27 * 2 * n_pad * 8;
	const int grid = static_cast<int>((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
	pack_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(weights, co, c0, c1, n_pad, steps0, steps, packed);
	IANE_GB_CUDA(cudaGetLastError(), "cnn_tc_pack: launch");
	return IANE_GB_OK;
}

int iane_gb_cnn_conv3_tc(const uint16_t* x0, int c0, const uint16_t* x1, int c1, int d, int h, int w,
	const uint16_t* packed, const float* bias, int co, uint16_t* y16, float* y32, const float* residual, int act,
	void* stream)
{
	if (!x0 || c0 < 1 || c1 < 0 || (c1 > 0 && (!x1 || c0 % 16 != 0)) || d < 1 || h < 1 || w < 1 || !packed || co < 1 ||
	    co > 64 || (!y16 && !y32) || (residual && co != 1) || (y16 && co % 8 != 0)) {
		return fail(IANE_GB_INVALID_ARGUMENT, "cnn_conv3_tc: bad arguments");
	}
	if (reinterpret_cast<uintptr_t>(x0) % 16 || reinterpret_cast<uintptr_t>(x1) % 16 ||
	    reinterpret_cast<uintptr_t>(packed) % 16 || reinterpret_cast<uintptr_t>(y16) % 16) {
		return fail(IANE_GB_INVALID_ARGUMENT, "cnn_conv3_tc: buffers must be 16-byte aligned");
	}
	const int n_pad = n_pad_of(co);
	const int bz = 2;
	int* status = device_status_ptr();
	if (!status) return IANE_GB_CUDA_ERROR;
	CUtensorMap m0{}, m1{};
	int rc = encode_c8_map(&m0, x0, c0, d, h, w, bz);
	if (rc) return rc;
	rc = encode_c8_map(&m1, c1 > 0 ? x1 : x0, c1 > 0 ? c1 : c0, d, h, w, bz);
	if (rc) return rc;
	TcConvArgs a{};
	a.d = d;
	a.h = h;
	a.w = w;
	a.steps0 = steps_of(c0);
	a.steps = a.steps0 + steps_of(c1);
	a.packed = packed;
	a.bias = bias;
	a.co = co;
	a.y16 = y16;
	a.y32 = y32;
	a.residual = residual;
	a.act = act;
	a.tiles_x = (w + OUT_X - 1) / OUT_X;
	a.tiles_y = (h + TY - 1) / TY;
	a.stages = a.steps > 1 ? 2 : 1;
	a.status = status;
	if ((d + bz - 1) / bz > 65535) return fail(IANE_GB_UNSUPPORTED, "cnn_conv3_tc: volume too deep");
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	switch (n_pad) {
	case 16: return launch<16, 2>(m0, m1, a, st);
	case 32: return launch<32, 2>(m0, m1, a, st);
	default: return launch<64, 2>(m0, m1, a, st);
	}
}

}  // extern "C"
