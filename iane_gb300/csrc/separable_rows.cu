// Bandwidth-oriented separable FP32 convolution of large 2-D images (radius R <= 7 on both axes).
//
// A block owns a strip of kRowsSW = 128 output columns and a chunk of rows, and marches down the
// chunk in steps of kRowsStep = 16 input rows:
//   1. each step's (128 + 2 RA) x 16 input tile lands in shared memory by one TMA, three steps
//      ahead (three stage buffers; zero fill outside the image). RA = R rounded up to 4, so the
//      TMA's x start is 16-byte aligned. In the first and last strip, clamp and mirror borders
//      rewrite the R out-of-image columns next to the image from the columns they map to;
//   2. axis 0: a warp filters one tile row -- each lane four consecutive outputs from a register
//      window read with 128-bit shared loads -- into a ring of 48 x-filtered rows (three steps);
//   3. axis 1: each thread takes one column and eight consecutive output rows and filters them
//      from the 8 + 2R ring rows they need. Output rows trail the input rows by 2R, so the rows
//      a step needs were filtered in this step or the one before; the clamp and mirror borders
//      along y read the ring row the border rule maps the row to (they copy whole rows, so they
//      commute with the x filter), the zero border reads zero.
// The 2R halo rows of each step come from the ring instead of being filtered again, each input
// row is loaded once per chunk, and a step needs one block barrier: a ring row is overwritten
// three steps after it was written, when every thread has passed the barrier of the step after
// its last reader. Taps are zero-padded to 2R + 1 and applied in the order of the other
// separable kernels, so the result is the same bits (successive 1-D convolutions with an f32
// intermediate).
#include "common.cuh"
#include "kernels.h"

#include <algorithm>

namespace iane_gb {
namespace {

constexpr int kRowsSW = 128;     // output columns per strip
constexpr int kRowsStep = 16;    // input rows per step
constexpr int kRowsRing = 48;    // x-filtered rows kept (three steps)
constexpr int kRowsStages = 3;   // TMA stage buffers
constexpr int kRowsThreads = 256;

template<int R>
struct RowsGeom {
	static constexpr int K = 2 * R + 1;
	static constexpr int RA = (R + 3) & ~3;
	static constexpr int D = RA - R;
	static constexpr int AW = kRowsSW + 2 * RA;              // tile width = TMA box width
	static constexpr int SEG = (D + 4 + 2 * R + 3) & ~3;     // axis-0 window per lane
	static constexpr int STAGE_FLOATS = AW * kRowsStep;
	static constexpr size_t BYTES = static_cast<size_t>(kRowsStages * STAGE_FLOATS + kRowsRing * kRowsSW) * 4 +
		kRowsStages * 8;
};

struct RowsArgs {
	char* dst;
	long long d_stride[2];
	int nx, ny;
	int border;
	int chunk;        // output rows per block
	int* status;
	const char* tap_ptr[2];
	long long tap_stride[2];
	int k[2];
};

template<int R>
__global__ void __launch_bounds__(kRowsThreads) separable_rows_kernel(const __grid_constant__ CUtensorMap map,
	const RowsArgs a)
{
	using G = RowsGeom<R>;
	constexpr int K = G::K;
	extern __shared__ __align__(128) unsigned char smem_raw[];
	float* stages = reinterpret_cast<float*>(smem_raw);
	float* ring = stages + kRowsStages * G::STAGE_FLOATS;        // [kRowsRing][kRowsSW]
	uint64_t* bars = reinterpret_cast<uint64_t*>(ring + kRowsRing * kRowsSW);

	const int tid = threadIdx.x;
	const int x0 = blockIdx.x * kRowsSW;
	const int c0 = blockIdx.y * a.chunk;
	const int c1 = min(c0 + a.chunk, a.ny);
	const int g0 = c0 - R;                                       // input row of step 0, tile row 0
	const int nsteps = (c1 - c0 + 2 * R + kRowsStep - 1) / kRowsStep;
	const bool edge_x = a.border != IANE_GB_BORDER_ZERO && (x0 - R < 0 || x0 + kRowsSW + R > a.nx);

	auto tap = [&](int axis, int i) -> float {
		const int q = i - (R - a.k[axis] / 2);
		return q >= 0 && q < a.k[axis] ? *reinterpret_cast<const float*>(a.tap_ptr[axis] + q * a.tap_stride[axis]) : 0.0f;
	};
	float tx[K], ty[K];
#pragma unroll
	for (int i = 0; i < K; ++i) {
		tx[i] = tap(0, i);
		ty[i] = tap(1, i);
	}
	if (tid == 0) {
		for (int b = 0; b < kRowsStages; ++b) mbar_init(&bars[b], 1);
		fence_barrier_init();
	}
	__syncthreads();

	auto issue = [&](int s) {
		const int b = s % kRowsStages;
		// order this buffer's earlier generic-proxy writes (the x fix-up) before the TMA
		asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
		mbar_arrive_expect_tx(&bars[b], static_cast<uint32_t>(G::STAGE_FLOATS * 4));
		tma_load_3d(stages + b * G::STAGE_FLOATS, &map, x0 - G::RA, g0 + kRowsStep * s, 0, &bars[b]);
	};
	if (tid == 0) {
		for (int s = 0; s < kRowsStages && s < nsteps; ++s) issue(s);
	}

	// axis 1 roles: column xc, output rows 8 h .. 8 h + 7 of the step's 16
	const int xc = tid & (kRowsSW - 1), h = tid >> 7;
	const bool x_in = x0 + xc < a.nx;
	char* dcol = a.dst + static_cast<long long>(x0 + xc) * 4;
	bool ok = true;
	for (int s = 0; s < nsteps; ++s) {
		const int b = s % kRowsStages;
		if (ok && !mbar_wait_bounded(&bars[b], (s / kRowsStages) & 1)) {
			ok = false;
			report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
		}
		float* tile = stages + b * G::STAGE_FLOATS;
		if (edge_x) {
			// the R columns next to each side of the image, from the columns the rule maps them to
			for (int i = tid; i < 2 * R * kRowsStep; i += kRowsThreads) {
				const int r = i / (2 * R), j = i % (2 * R);
				const int gx = j < R ? -R + j : a.nx + (j - R);
				const int c = gx - (x0 - G::RA);
				if (c < 0 || c >= G::AW) continue;
				int mx = 0;
				map_coord(gx, a.nx, a.border, mx);
				const int cs = mx - (x0 - G::RA); // inside the tile for images at least a strip wide
				if (cs >= 0 && cs < G::AW) tile[r * G::AW + c] = tile[r * G::AW + cs];
			}
			__syncthreads(); // fixed columns visible
		}
		// axis 0: row r = warp (+ 8), four outputs per lane into ring row (16 s + r) mod 48
#pragma unroll
		for (int t = 0; t < 2; ++t) {
			const int task = tid + kRowsThreads * t;
			const int r = task >> 5, q = task & 31;
			float seg[G::SEG];
			const float4* srow = reinterpret_cast<const float4*>(tile + r * G::AW + 4 * q);
#pragma unroll
			for (int m = 0; m < G::SEG / 4; ++m) {
				const float4 v = srow[m];
				seg[4 * m] = v.x;
				seg[4 * m + 1] = v.y;
				seg[4 * m + 2] = v.z;
				seg[4 * m + 3] = v.w;
			}
			float o[4];
#pragma unroll
			for (int i = 0; i < 4; ++i) {
				float acc = 0.0f;
#pragma unroll
				for (int qq = 0; qq < K; ++qq) acc = fmaf(tx[qq], seg[G::D + i + 2 * R - qq], acc);
				o[i] = acc;
			}
			const int slot = (kRowsStep * s + r) % kRowsRing;
			*reinterpret_cast<float4*>(ring + slot * kRowsSW + 4 * q) = make_float4(o[0], o[1], o[2], o[3]);
		}
		__syncthreads(); // the step's ring rows complete; its tile is free
		if (tid == 0 && s + kRowsStages < nsteps) issue(s + kRowsStages);
		// axis 1: output rows y = c0 - 2R + 16 s + 8 h + j (those in [c0, c1)); their input rows
		// y - R .. y + R are filtered and still in the ring
		const int ybase = c0 - 2 * R + kRowsStep * s + 8 * h;
		if (ybase + 8 > c0 && ybase < c1) {
			float w[8 + 2 * R];
			const int rel0 = ybase - R - g0; // ring position of the window's first row
			if (rel0 >= 0 && ybase - R >= 0 && ybase + 7 + R < a.ny) {
				// the whole window lies in the image and in the ring: consecutive slots, one wrap
				const float* base = ring + (rel0 % kRowsRing) * kRowsSW + xc;
				const int room = kRowsRing - rel0 % kRowsRing; // slots before the wrap
#pragma unroll
				for (int m = 0; m < 8 + 2 * R; ++m) {
					w[m] = base[(m < room ? m : m - kRowsRing) * kRowsSW];
				}
			} else {
#pragma unroll
				for (int m = 0; m < 8 + 2 * R; ++m) {
					int g = ybase - R + m;
					bool present = true;
					if (g < 0 || g >= a.ny) present = map_coord(g, a.ny, a.border, g);
					// rows before the chunk's first input row feed only outputs above the chunk
					// (not stored); every other row read lies in the last 48 filtered rows
					const int rel = g - g0;
					w[m] = present && rel >= 0 ? ring[(rel % kRowsRing) * kRowsSW + xc] : 0.0f;
				}
			}
#pragma unroll
			for (int j = 0; j < 8; ++j) {
				const int y = ybase + j;
				float acc = 0.0f;
#pragma unroll
				for (int qq = 0; qq < K; ++qq) acc = fmaf(ty[qq], w[j + 2 * R - qq], acc);
				if (x_in && y >= c0 && y < c1) {
					*reinterpret_cast<float*>(dcol + y * a.d_stride[1]) = acc;
				}
			}
		}
	}
}

template<int R>
int launch_rows(const CUtensorMap& map, const RowsArgs& args, cudaStream_t stream)
{
	using G = RowsGeom<R>;
	const size_t smem = G::BYTES;
	auto kernel = separable_rows_kernel<R>;
	IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
		"separable rows: set shared memory size");
	int per_sm = 1;
	IANE_GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kRowsThreads, smem),
		"separable rows: occupancy");
	const int strips = (args.nx + kRowsSW - 1) / kRowsSW;
	// chunks of at least four steps that fill whole waves of resident blocks
	const long long slots = static_cast<long long>(std::max(per_sm, 1)) * device_sm_count();
	const int chunks = strip_chunks(strips, args.ny, slots, kRowsStep);
	RowsArgs a = args;
	a.chunk = (args.ny + chunks - 1) / chunks;
	const dim3 grid(strips, static_cast<unsigned int>((args.ny + a.chunk - 1) / a.chunk));
	kernel<<<grid, kRowsThreads, smem, stream>>>(map, a);
	IANE_GB_CUDA(cudaGetLastError(), "separable rows: launch");
	return IANE_GB_OK;
}

}  // namespace

int launch_separable_rows(const DevView& src, const DevView* taps, const DevView& dst, int border, cudaStream_t stream)
{
	int r = 0;
	for (int i = 0; i < 2; ++i) r = max(r, taps[i].ext[0] / 2);
	const bool two_d = src.rank <= 2 || (src.ext[2] == 1 && taps[2].ext[0] == 1);
	// large images only (from 4 M pixels: smaller ones are launch-bound and take the tiled
	// kernel; the border rules also assume a strip's width and four steps of rows), f32 rows TMA
	// can address, radius <= 7 on both axes
	if (!two_d || r > 7 || src.ext[0] < kRowsSW || src.ext[1] < 4 * kRowsStep ||
	    static_cast<long long>(src.ext[0]) * src.ext[1] < (1LL << 22) || src.stride[0] != 4 ||
	    !rows_aligned16(src) || (src.ext[1] > 1 && src.stride[1] < 4LL * src.ext[0]) || dst.stride[0] != 4 ||
	    dst.stride[1] % 4 != 0 || dst.stride[1] < 4LL * dst.ext[0]) {
		return IANE_GB_UNSUPPORTED;
	}
	RowsArgs a{};
	a.dst = dst.ptr;
	a.d_stride[0] = dst.stride[0];
	a.d_stride[1] = dst.stride[1];
	a.nx = src.ext[0];
	a.ny = src.ext[1];
	a.border = border;
	a.status = device_status_ptr();
	if (!a.status) return IANE_GB_CUDA_ERROR;
	for (int axis = 0; axis < 2; ++axis) {
		a.tap_ptr[axis] = taps[axis].ptr;
		a.tap_stride[axis] = taps[axis].stride[0];
		a.k[axis] = taps[axis].ext[0];
		if (!a.tap_ptr[axis]) { // an axis beyond the rank: the single tap 1 is not expected here
			return IANE_GB_UNSUPPORTED;
		}
	}
	const int rr = r < 1 ? 1 : r;
	const int rxa = (rr + 3) & ~3;
	CUtensorMap map{};
	const int status = encode_tensor_map_f32(&map, src.ptr, src.ext[0], src.ext[1], 1, src.stride[1],
		src.stride[1] * src.ext[1], kRowsSW + 2 * rxa, kRowsStep);
	if (status) return status;
	switch (rr) {
	case 1: return launch_rows<1>(map, a, stream);
	case 2: return launch_rows<2>(map, a, stream);
	case 3: return launch_rows<3>(map, a, stream);
	case 4: return launch_rows<4>(map, a, stream);
	case 5: return launch_rows<5>(map, a, stream);
	case 6: return launch_rows<6>(map, a, stream);
	case 7: return launch_rows<7>(map, a, stream);
	default: return IANE_GB_UNSUPPORTED;
	}
}

}  // namespace iane_gb
