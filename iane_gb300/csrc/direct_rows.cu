// Bandwidth-oriented direct FP32 convolution of large 2-D f32 images, or stacks of 2-D planes
// each filtered on its own (a 3-D view with a kernel one plane deep), with small kernels
// (KX x KY, each odd and at most 7, line filters included): at 2 KX KY flop per 8 bytes of
// traffic these reach from HBM-bound to the FP32 pipe / HBM ridge (7 x 7), so both the
// instruction stream and the memory stream must keep going. RX = KX / 2, RY = KY / 2.
//
// A block owns a strip of kDrSW = 128 output columns and a chunk of rows of one plane, and
// marches down the chunk in steps of kDrStep = 32 output rows:
//   * input rows arrive by TMA in boxes of 32 rows x (128 + 2 RA) columns (RA = RX rounded up to
//     4: the box's x start is 16-byte aligned; zero fill outside the image) into a ring of
//     kDrSlots = 3 boxes -- 96 rows, row pitch AW floats. Step s reads boxes s and s + 1 (its 32
//     output rows need 32 + 2 RY input rows), box s + 2 is in flight, and box s + 3 is issued
//     into box s's slot once every thread is past step s (one block barrier per step). Each
//     input row is loaded once per chunk; a 64x64-tile kernel loads 2 RY halo rows per 64 again;
//   * clamp and mirror borders are applied once per box in shared memory, at the end of the step
//     before the box is first read (under that step's barrier): in the first and last strip the
//     RX columns beside the image are rewritten from the columns the rule maps them to, and rows
//     outside the image (top box of the first chunk, bottom boxes of the last) are replaced by
//     the rows they map to, which lie in the same box or the one before it (resident). The zero
//     border keeps the TMA's zeros. The sums then run without a check. (A fix-up with its own
//     barrier and the general border rule per cell made the edge strips' blocks, which end the
//     last wave, 13% slower under mirror: 8192^2 7x7 0.157 ms against 0.139 with zeros);
//   * a warp covers 32 columns x 32 rows, a lane 4 consecutive columns x 8 consecutive rows:
//     its 8 + 2 RY window rows each give one segment of at most 12 floats by 128-bit shared
//     loads, and the eight lanes of a quarter-warp read 128 contiguous bytes (no bank conflict).
//     The kernel's KX KY taps stay in registers for the whole launch, so the loop body is FMAs and
//     segment loads. Lanes of 4 x 4 outputs in 16-row steps spent twice the share of their
//     issue slots on row addressing, loads, stores and barriers (5 blocks per SM at 96
//     registers): 8192^2 3x3 / 5x5 mirror 0.101 / 0.096 ms against 0.087 / 0.088 ms now; 7x7,
//     bound by the FMA pipe's issue share either way, 0.138 ms with zeros in both. Visiting the
//     FMAs output row innermost instead (each segment value reused across the lane's rows)
//     measured the same; three blocks per SM with 158 registers for 7x7 instead of four with
//     127, 0.145 ms.
// Each output adds its taps in the order of the tiled kernel's single-plane path (input rows
// ascending, taps ascending within a row, starting from +0), so the results are the same bits.
//
// Coordinates follow the reference's convolution_filter (include/iane/algorithms/
// convolution.hpp:37-45): out[p] = sum_q K[q] * in[p + size/2 - q].
#include "common.cuh"
#include "kernels.h"

#include <algorithm>

namespace iane_gb {
namespace {

constexpr int kDrSW = 128;       // output columns per strip
constexpr int kDrStep = 32;      // output rows per step = input rows per box
constexpr int kDrSlots = 3;      // ring slots (boxes)
constexpr int kDrRing = kDrSlots * kDrStep;
constexpr int kDrThreads = 128;  // four warps side by side along x
constexpr int kDrLaneRows = 8;   // output rows of a lane (4 lanes along y per warp)

// Box width (floats) of a kernel kx wide: the strip and its x halo rounded up to 16 bytes.
inline int dr_box_width(int kx) { return kDrSW + 2 * (((kx / 2) + 3) & ~3); }

template<int KX, int KY>
struct DrGeom {
	static constexpr int RX = KX / 2, RY = KY / 2;
	static constexpr int RA = (RX + 3) & ~3;              // x halo rounded up to 16 bytes
	static constexpr int D = RA - RX;                     // segment lead-in
	static constexpr int AW = kDrSW + 2 * RA;             // box width = ring row pitch (floats)
	static constexpr int SEG = (D + 4 + 2 * RX + 3) & ~3; // segment floats per window row
	static constexpr int ROWS = kDrLaneRows + 2 * RY;     // window rows of a lane per step
	static constexpr int BOX = AW * kDrStep;              // floats per box
	static constexpr size_t BYTES = static_cast<size_t>(kDrSlots) * BOX * 4 + kDrSlots * 8;
	static_assert(2 * RY <= kDrStep, "a step's window spans two boxes");
	static_assert(4 * kDrLaneRows == kDrStep, "four lanes along y cover a step");
	static_assert(4 * (kDrSW / 4 - 1) + SEG <= AW, "segments stay inside the box row");
};

struct DirectRowsArgs {
	char* dst;
	long long d_stride[3];
	int vec4;          // destination rows 16-byte aligned with packed x: float4 stores
	int nx, ny;
	int border;
	int chunk;         // output rows per block
	int* status;
	const char* kernel;
	long long k_stride[2];
};

// STACK: blockIdx.z selects a plane of a stack (a separate instantiation, so that the one-plane
// kernel carries no plane offset: 0.139 against 0.142 ms at 8192^2 7x7 mirror).
template<int KX, int KY, bool STACK>
__global__ void __launch_bounds__(kDrThreads, 4) direct_rows_kernel(const __grid_constant__ CUtensorMap map,
	const DirectRowsArgs a)
{
	using G = DrGeom<KX, KY>;
	constexpr int RX = G::RX, RY = G::RY;
	extern __shared__ __align__(128) unsigned char smem_raw[];
	float* ring = reinterpret_cast<float*>(smem_raw);                       // [kDrRing][AW]
	uint64_t* bars = reinterpret_cast<uint64_t*>(ring + kDrSlots * G::BOX);

	const int tid = threadIdx.x;
	const int lane = tid & 31, warp = tid >> 5;
	const int cx = 8 * warp + (lane & 7);  // column group: outputs x0 + 4 cx .. + 3
	const int cy = lane >> 3;              // row group: output rows 8 cy .. + 7 of a step
	const int x0 = blockIdx.x * kDrSW;
	const int c0 = blockIdx.y * a.chunk;
	const int plane = STACK ? static_cast<int>(blockIdx.z) : 0;
	const int c1 = min(c0 + a.chunk, a.ny);
	const int g0 = c0 - RY;                 // input row of box 0, row 0
	const int nsteps = (c1 - c0 + kDrStep - 1) / kDrStep;
	const int nboxes = nsteps + 1;
	const bool mapped = a.border != IANE_GB_BORDER_ZERO;
	const bool edge_x = mapped && (x0 - RX < 0 || x0 + kDrSW + RX > a.nx);

	float tap[KY][KX]; // [kernel row][kernel column]
#pragma unroll
	for (int b = 0; b < KY; ++b)
#pragma unroll
		for (int q = 0; q < KX; ++q)
			tap[b][q] = *reinterpret_cast<const float*>(a.kernel + q * a.k_stride[0] + b * a.k_stride[1]);

	if (tid == 0) {
		for (int b = 0; b < kDrSlots; ++b) mbar_init(&bars[b], 1);
		fence_barrier_init();
	}
	__syncthreads();

	auto issue = [&](int k) {
		const int b = k % kDrSlots;
		// order this slot's earlier generic-proxy accesses (fix-ups, reads) before the TMA write
		asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
		mbar_arrive_expect_tx(&bars[b], static_cast<uint32_t>(G::BOX * 4));
		tma_load_3d(ring + b * G::BOX, &map, x0 - G::RA, g0 + kDrStep * k, plane, &bars[b]);
	};
	if (tid == 0) {
		for (int k = 0; k < kDrSlots && k < nboxes; ++k) issue(k);
	}

	bool ok = true;
	auto wait_box = [&](int k) {
		if (ok && !mbar_wait_bounded(&bars[k % kDrSlots], (k / kDrSlots) & 1)) {
			ok = false;
			report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
		}
	};
	// clamp / mirror, box k: the RX columns beside the image (first and last strip), then the rows
	// outside the image from the rows the rule maps them to. The caller's next block barrier
	// publishes the fixed cells; the row copy, which reads fixed columns, has its own barrier.
	const bool clamp = a.border == IANE_GB_BORDER_CLAMP;
	auto fix_box = [&](int k) {
		float* box = ring + (k % kDrSlots) * G::BOX;
		if (edge_x && tid < 2 * kDrStep) {
			// a thread per row and side; one reflection suffices (RX < nx)
			float* row = box + (tid % kDrStep) * G::AW;
			const bool right = tid >= kDrStep;
#pragma unroll
			for (int j = 0; j < RX; ++j) {
				const int gx = right ? a.nx + j : -RX + j;
				const int gm = right ? (clamp ? a.nx - 1 : 2 * a.nx - 1 - gx) : (clamp ? 0 : -gx - 1);
				const int c = gx - (x0 - G::RA), cs = gm - (x0 - G::RA);
				if (c >= 0 && c < G::AW && cs >= 0 && cs < G::AW) row[c] = row[cs];
			}
		}
		const int top = g0 + kDrStep * k;
		if (mapped && (top < 0 || top + kDrStep > a.ny)) {
			__syncthreads(); // columns fixed before rows are copied
			// whole rows from the rows the rule maps them to: inside the image, in this box or
			// the one before
			constexpr int V = G::AW / 4;
			for (int i = tid; i < kDrStep * V; i += kDrThreads) {
				const int r = i / V, v = i % V;
				const int g = top + r;
				if ((g >= 0 && g < a.ny) || g < -RY || g >= a.ny + RY) continue; // rows no stored output reads stay
				int gm = 0;
				map_coord(g, a.ny, a.border, gm);
				const int src_row = (gm - g0) % kDrRing;
				const int dst_row = (kDrStep * k + r) % kDrRing;
				reinterpret_cast<float4*>(ring + dst_row * G::AW)[v] = reinterpret_cast<const float4*>(ring + src_row * G::AW)[v];
			}
		}
	};

	// boxes 0 and 1 ready before step 0; box s + 2 is waited for and fixed at the end of step s,
	// before the step's barrier, so the edge strips need no barrier of their own
	wait_box(0);
	fix_box(0);
	wait_box(1);
	fix_box(1);
	__syncthreads();
	const bool x_in = x0 + 4 * cx < a.nx;
	for (int s = 0; s < nsteps; ++s) {
		// the lane's window: ring rows base .. base + ROWS - 1 (mod kDrRing)
		const int base = kDrStep * (s % kDrSlots) + kDrLaneRows * cy;
		const int room = kDrRing - base; // rows before the ring wraps
		const float* lo = ring + base * G::AW + 4 * cx;
		const float* hi = lo - kDrRing * G::AW;
		float acc[kDrLaneRows][4];
#pragma unroll
		for (int j = 0; j < kDrLaneRows; ++j)
#pragma unroll
			for (int i = 0; i < 4; ++i) acc[j][i] = 0.0f;
#pragma unroll
		for (int m = 0; m < G::ROWS; ++m) {
			const float4* row = reinterpret_cast<const float4*>((m < room ? lo : hi) + m * G::AW);
			float seg[G::SEG];
#pragma unroll
			for (int v = 0; v < G::SEG / 4; ++v) {
				const float4 t = row[v];
				seg[4 * v + 0] = t.x;
				seg[4 * v + 1] = t.y;
				seg[4 * v + 2] = t.z;
				seg[4 * v + 3] = t.w;
			}
#pragma unroll
			for (int j = 0; j < kDrLaneRows; ++j) {
				const int b = j + 2 * RY - m; // kernel row pairing window row m with output row j
				if (b >= 0 && b < KY) {
#pragma unroll
					for (int q = 0; q < KX; ++q)
#pragma unroll
						for (int i = 0; i < 4; ++i) acc[j][i] = fmaf(tap[b][q], seg[G::D + i + 2 * RX - q], acc[j][i]);
				}
			}
		}
		if (x_in) {
			const int x = x0 + 4 * cx;
#pragma unroll
			for (int j = 0; j < kDrLaneRows; ++j) {
				const int y = c0 + kDrStep * s + kDrLaneRows * cy + j;
				if (y >= c1) break;
				char* p = a.dst + y * a.d_stride[1];
				if constexpr (STACK) p += plane * a.d_stride[2];
				if (a.vec4 && x + 4 <= a.nx) {
					*reinterpret_cast<float4*>(p + x * 4LL) = make_float4(acc[j][0], acc[j][1], acc[j][2], acc[j][3]);
				} else {
#pragma unroll
					for (int i = 0; i < 4; ++i) {
						if (x + i < a.nx) *reinterpret_cast<float*>(p + (x + i) * a.d_stride[0]) = acc[j][i];
					}
				}
			}
		}
		if (s + 2 < nboxes) {
			wait_box(s + 2);
			fix_box(s + 2);
		}
		__syncthreads(); // every lane is done with box s; box s + 2 is fixed
		if (tid == 0 && s + kDrSlots < nboxes) issue(s + kDrSlots);
	}
}

template<int KX, int KY, bool STACK>
int launch_rows_k(const CUtensorMap& map, const DirectRowsArgs& args, int nz, cudaStream_t stream)
{
	using G = DrGeom<KX, KY>;
	const size_t smem = G::BYTES;
	auto kernel = direct_rows_kernel<KX, KY, STACK>;
	IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
		"direct rows: set shared memory size");
	int per_sm = 1;
	IANE_GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kDrThreads, smem),
		"direct rows: occupancy");
	const int strips = (args.nx + kDrSW - 1) / kDrSW;
	// chunks of at least four steps that fill whole waves of resident blocks
	const long long slots = static_cast<long long>(std::max(per_sm, 1)) * device_sm_count();
	const int chunks = strip_chunks(static_cast<long long>(strips) * nz, args.ny, slots, kDrStep);
	DirectRowsArgs a = args;
	a.chunk = (args.ny + chunks - 1) / chunks;
	const dim3 grid(strips, static_cast<unsigned int>((args.ny + a.chunk - 1) / a.chunk), static_cast<unsigned int>(nz));
	kernel<<<grid, kDrThreads, smem, stream>>>(map, a);
	IANE_GB_CUDA(cudaGetLastError(), "direct rows: launch");
	return IANE_GB_OK;
}

// The instantiations for kernel heights 1..7 at width KX, one-plane and stack.
template<int KX>
int launch_rows_kx(int ky, bool stack, const CUtensorMap& map, const DirectRowsArgs& a, int nz, cudaStream_t stream)
{
	switch (ky) {
	case 1:
		if constexpr (KX > 1) { // 1 x 1 is not taken
			return stack ? launch_rows_k<KX, 1, true>(map, a, nz, stream) : launch_rows_k<KX, 1, false>(map, a, 1, stream);
		}
		return IANE_GB_UNSUPPORTED;
	case 3: return stack ? launch_rows_k<KX, 3, true>(map, a, nz, stream) : launch_rows_k<KX, 3, false>(map, a, 1, stream);
	case 5: return stack ? launch_rows_k<KX, 5, true>(map, a, nz, stream) : launch_rows_k<KX, 5, false>(map, a, 1, stream);
	case 7: return stack ? launch_rows_k<KX, 7, true>(map, a, nz, stream) : launch_rows_k<KX, 7, false>(map, a, 1, stream);
	default: return IANE_GB_UNSUPPORTED;
	}
}

}  // namespace

int launch_direct_rows(const DevView& src, const DevView& kernel, const DevView& dst, int border, cudaStream_t stream)
{
	const int kx = kernel.ext[0], ky = kernel.ext[1];
	// f32 source, taps and destination; 2-D planes (one or a stack) and a kernel one plane deep;
	// odd kernel extents up to 7 (1 x 1 excepted); at least 4 M pixels in all (the tiled kernel
	// fills the GPU better below), planes a strip wide and four steps tall; rows and planes TMA
	// can address
	const int nz = src.ext[2];
	if (src.dtype != IANE_GB_F32 || kernel.dtype != IANE_GB_F32 || dst.dtype != IANE_GB_F32) return IANE_GB_UNSUPPORTED;
	if (kernel.ext[2] != 1 || kx % 2 == 0 || ky % 2 == 0 || kx < 1 || ky < 1 || kx > 7 || ky > 7 ||
	    (kx == 1 && ky == 1) || nz < 1 || nz > 65535) {
		return IANE_GB_UNSUPPORTED;
	}
	if (src.ext[0] < kDrSW || src.ext[1] < 4 * kDrStep ||
	    static_cast<long long>(src.ext[0]) * src.ext[1] * nz < (1LL << 22) || src.ext[1] > (1 << 30) ||
	    !rows_aligned16(src) || src.stride[1] < 4LL * src.ext[0] ||
	    (nz > 1 && src.stride[2] < src.stride[1] * src.ext[1]) || !kernel.ptr) {
		return IANE_GB_UNSUPPORTED;
	}
	DirectRowsArgs a{};
	a.dst = dst.ptr;
	a.d_stride[0] = dst.stride[0];
	a.d_stride[1] = dst.stride[1];
	a.d_stride[2] = dst.stride[2];
	a.vec4 = rows_aligned16(dst) ? 1 : 0;
	a.nx = src.ext[0];
	a.ny = src.ext[1];
	a.border = border;
	a.kernel = kernel.ptr;
	a.k_stride[0] = kernel.stride[0];
	a.k_stride[1] = kernel.stride[1];
	a.status = device_status_ptr();
	if (!a.status) return IANE_GB_CUDA_ERROR;
	CUtensorMap map{};
	const int status = encode_tensor_map_f32(&map, src.ptr, src.ext[0], src.ext[1], nz, src.stride[1],
		nz > 1 ? src.stride[2] : src.stride[1] * src.ext[1], dr_box_width(kx), kDrStep);
	if (status) return status;
	const bool stack = nz > 1;
	switch (kx) {
	case 1: return launch_rows_kx<1>(ky, stack, map, a, nz, stream);
	case 3: return launch_rows_kx<3>(ky, stack, map, a, nz, stream);
	case 5: return launch_rows_kx<5>(ky, stack, map, a, nz, stream);
	case 7: return launch_rows_kx<7>(ky, stack, map, a, nz, stream);
	default: return IANE_GB_UNSUPPORTED;
	}
}

}  // namespace iane_gb
