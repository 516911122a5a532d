// Bandwidth-oriented fused separable FP32 convolution (radius R <= 7 on every used axis).
//
// A block owns a 64 (x) x 16 (y) column of the volume and marches along z through a chunk
// of planes. Per input plane:
//   1. the (64 + 2 RA) x (16 + 2 R) halo tile lands in shared memory, three planes ahead of
//      the one being filtered (four buffers), by one TMA (zero fill outside the image = the
//      zero border; planes outside the volume load as zeros). For clamp and mirror borders
//      the block then rewrites only its out-of-image halo cells from their mapped in-image
//      cells. Views TMA cannot address use 4-byte cp.async with the border rule applied per
//      element. RA = R rounded up to 4 so that the TMA's x start is 16-byte aligned;
//   2. axis 0: each thread filters 4 consecutive x of one or two tile rows from a register
//      window read with 128-bit shared loads, into a 64 x (16 + 2R) buffer;
//   3. axis 1: each thread filters a 2 (x) x 2 (y) patch, the x pair as one float2 so that
//      the multiply-adds are packed f32x2 FMAs (same tap, neighbouring columns);
//   4. axis 2: the filtered patch enters a register window of 2R + 1 planes (shifted by one
//      slot per plane) and, once full, produces the output plane R behind, written as float2
//      pairs.
// Taps of every axis are zero-padded to 2R + 1, centred, so one radius serves all axes.
// Rounding points are those of successive 1-D convolutions with an f32 intermediate.
#include "common.cuh"
#include "kernels.h"

#include <algorithm>
#include <cmath>

namespace iane_gb {
namespace {

constexpr int kFX = 64;
constexpr int kFY = 16;
constexpr int kFThreads = 256;
constexpr int kNBuf = 4; // tile buffers: three planes load while one is filtered

template<int R>
struct SepGeom {
	static constexpr int K = 2 * R + 1;
	static constexpr int RA = (R + 3) & ~3;
	static constexpr int D = RA - R;
	static constexpr int AW = kFX + 2 * RA;            // tile width = TMA box width (floats)
	static constexpr int AH = kFY + 2 * R;             // tile height
	static constexpr int SEG = (D + 4 + 2 * R + 3) & ~3; // axis-0 window per thread
	static constexpr int A_FLOATS = (AW * AH + 31) & ~31;
	static constexpr int B_FLOATS = kFX * AH;
};

struct SepFastArgs {
	const char* src;
	long long s_stride[3];
	char* dst;
	long long d_stride[3];
	int nx, ny, nz;
	int border;
	int zchunk;
	int use_tma;      // source is TMA-addressable
	int dst_pairs;    // destination rows take aligned float2 stores
	int* status;
	const char* tap_ptr[3];  // 1-D f32 device views of the taps (null: axis beyond the rank)
	long long tap_stride[3];
	int k[3];
};

template<int R, bool Z>
__global__ void __launch_bounds__(kFThreads) separable_fast_kernel(const __grid_constant__ CUtensorMap map,
	const SepFastArgs a)
{
	using G = SepGeom<R>;
	constexpr int K = G::K;
	extern __shared__ __align__(128) unsigned char smem_raw[];
	float* A = reinterpret_cast<float*>(smem_raw);           // kNBuf tile buffers
	float* B = A + kNBuf * G::A_FLOATS;                       // axis-0 result
	float2* tpair = reinterpret_cast<float2*>(B + G::B_FLOATS); // (t, t) pairs of axes 1 and 2
	uint64_t* bars = reinterpret_cast<uint64_t*>(tpair + 2 * 16);

	const int tid = threadIdx.x;
	const int x0 = blockIdx.x * kFX;
	const int zs = Z ? blockIdx.z * a.zchunk : 0;
	const int ze = Z ? min(zs + a.zchunk, a.nz) : 1;
	// 3-D: the block's planes stream through the buffers. 2-D: its tiles do -- tile p is tile
	// row blockIdx.y + p * gridDim.y, so consecutive tiles' loads overlap their filtering.
	const int ytiles = (a.ny + kFY - 1) / kFY;
	const int nplanes = Z ? (ze - zs) + 2 * R
		: (ytiles - static_cast<int>(blockIdx.y) + static_cast<int>(gridDim.y) - 1) / static_cast<int>(gridDim.y);
	auto y0_of = [&](int p) -> int {
		return Z ? static_cast<int>(blockIdx.y) * kFY : (static_cast<int>(blockIdx.y) + p * static_cast<int>(gridDim.y)) * kFY;
	};
	const bool tma = a.use_tma;
	auto fixup_of = [&](int p) -> bool {
		const int y0 = y0_of(p);
		const bool interior = x0 - G::RA >= 0 && x0 + kFX + G::RA <= a.nx && y0 - R >= 0 && y0 + kFY + R <= a.ny;
		return tma && !interior && a.border != IANE_GB_BORDER_ZERO;
	};

	// Taps centred and zero-padded to 2R + 1; an axis beyond the rank is the single tap 1.
	auto tap = [&](int axis, int i) -> float {
		if (!a.tap_ptr[axis]) {
			return i == R ? 1.0f : 0.0f;
		}
		const int q = i - (R - a.k[axis] / 2);
		return q >= 0 && q < a.k[axis] ? *reinterpret_cast<const float*>(a.tap_ptr[axis] + q * a.tap_stride[axis])
			: 0.0f;
	};
	float tx[K];
#pragma unroll
	for (int i = 0; i < K; ++i) tx[i] = tap(0, i);
	if (tid < 2 * K) {
		const float t = tap(1 + tid / K, tid % K);
		tpair[(tid / K) * 16 + tid % K] = make_float2(t, t);
	}
	if (tid == 0) {
		for (int b = 0; b < kNBuf; ++b) mbar_init(&bars[b], 1);
		fence_barrier_init();
	}
	__syncthreads();

	// plane p of this block's sequence is input plane zs - R + p (Z) or 0
	auto plane_of = [&](int p, int& zi) -> bool {
		const int z = Z ? zs - R + p : 0;
		return map_coord(z, a.nz, a.border, zi);
	};
	auto issue = [&](int p) {
		float* dst = A + (p % kNBuf) * G::A_FLOATS;
		const int y0 = y0_of(p);
		int zi = 0;
		const bool present = plane_of(p, zi);
		if (tma) {
			// every plane gets one TMA (an out-of-volume plane reads as zeros), so the k-th
			// completion of buffer b belongs to plane b + k * kNBuf
			if (tid == 0) {
				// order this buffer's earlier generic-proxy use (a previous tile's fix-up) before
				// the TMA's async-proxy write
				asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
				mbar_arrive_expect_tx(&bars[p % kNBuf], static_cast<uint32_t>(G::AW * G::AH * 4));
				tma_load_3d(dst, &map, x0 - G::RA, y0 - R, present ? zi : (Z ? zs - R + p : 0), &bars[p % kNBuf]);
			}
			return;
		}
		if (present) {
			const char* plane = a.src + zi * a.s_stride[2];
			for (int i = tid; i < G::AW * G::AH; i += kFThreads) {
				const int r = i / G::AW, c = i - r * G::AW;
				int xi = 0, yi = 0;
				const bool ok = map_coord(x0 - G::RA + c, a.nx, a.border, xi) && map_coord(y0 - R + r, a.ny, a.border, yi);
				const char* s = ok ? plane + xi * a.s_stride[0] + yi * a.s_stride[1] : a.src;
				cp_async4(dst + i, s, ok ? 4 : 0);
			}
		}
		cp_async_commit(); // one group per plane, empty for a zero-border plane outside
	};

	// thread roles
	const int xq = tid & 15, rg = tid >> 4;   // axis 0: 4 consecutive x of rows rg, rg + 16
	const int xp = tid & 31, yq = tid >> 5;   // axes 1, 2: x pair 2xp, y rows 2yq, 2yq + 1
	const int ox = x0 + 2 * xp;

	float2 win[2][K]; // axis-2 window: [row][plane slot]
#pragma unroll
	for (int j = 0; j < 2; ++j)
#pragma unroll
		for (int s = 0; s < K; ++s) win[j][s] = make_float2(0.0f, 0.0f);

	for (int p = 0; p < kNBuf - 1 && p < nplanes; ++p) issue(p);
	bool ok = true;

	// One plane: returns the axis-0/1 filtered 2x2 patch (zero for a zero-border plane).
	auto filter_plane = [&](int p, float2& c0, float2& c1) {
		int zi = 0;
		const bool present = tma || plane_of(p, zi);
		if (p + kNBuf - 1 < nplanes) issue(p + kNBuf - 1); // its buffer held plane p - 1
		if (tma) {
			if (ok && !mbar_wait_bounded(&bars[p % kNBuf], (p / kNBuf) & 1)) {
				ok = false;
				report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
			}
		} else {
			// groups committed after plane p's: planes p+1 .. min(p+3, last)
			const int newer = min(kNBuf - 1, nplanes - 1 - p);
			if (newer >= 3) {
				cp_async_wait<3>();
			} else if (newer == 2) {
				cp_async_wait<2>();
			} else if (newer == 1) {
				cp_async_wait<1>();
			} else {
				cp_async_wait<0>();
			}
		}
		if (fixup_of(p)) {
			// clamp / mirror: replace the zero-filled out-of-image halo cells by the cells the
			// border rule maps them to (inside this tile, else read from the image)
			const int y0 = y0_of(p);
			float* tile = A + (p % kNBuf) * G::A_FLOATS;
			int zi2 = 0;
			plane_of(p, zi2);
			const int gx0 = x0 - G::RA, gy0 = y0 - R;
			const int c_lo = max(0, -gx0), c_hi = min(G::AW, a.nx - gx0); // in-image columns [c_lo, c_hi)
			for (int r = tid >> 5; r < G::AH; r += kFThreads / 32) {
				const int gy = gy0 + r;
				const bool row_in = gy >= 0 && gy < a.ny;
				for (int c = tid & 31; c < G::AW; c += 32) {
					if (row_in && c >= c_lo && c < c_hi) continue;
					int mx = 0, my = 0;
					map_coord(gx0 + c, a.nx, a.border, mx);
					map_coord(gy, a.ny, a.border, my);
					const int lc = mx - gx0, lr = my - gy0;
					const bool in_image_cell = lc >= c_lo && lc < c_hi && lr >= 0 && lr < G::AH && my >= 0;
					tile[r * G::AW + c] = in_image_cell ? tile[lr * G::AW + lc]
						: *reinterpret_cast<const float*>(a.src + mx * a.s_stride[0] + my * a.s_stride[1] +
							zi2 * a.s_stride[2]);
				}
			}
		}
		__syncthreads(); // tile visible to all; B free
		if (present) {
			const float* tile = A + (p % kNBuf) * G::A_FLOATS;
#pragma unroll
			for (int k = 0; k < 2; ++k) {
				const int r = rg + 16 * k;
				if (r < G::AH) {
					float seg[G::SEG];
					const float4* srow = reinterpret_cast<const float4*>(tile + r * G::AW + 4 * xq);
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
						float s = 0.0f;
#pragma unroll
						for (int q = 0; q < K; ++q) s = fmaf(tx[q], seg[G::D + i + 2 * R - q], s);
						o[i] = s;
					}
					*reinterpret_cast<float4*>(B + r * kFX + 4 * xq) = make_float4(o[0], o[1], o[2], o[3]);
				}
			}
		}
		__syncthreads(); // B complete; this tile buffer is free for plane p + kNBuf
		c0 = make_float2(0.0f, 0.0f);
		c1 = make_float2(0.0f, 0.0f);
		if (present) {
			float2 col[2 + 2 * R];
#pragma unroll
			for (int m = 0; m < 2 + 2 * R; ++m) {
				col[m] = *reinterpret_cast<const float2*>(B + (2 * yq + m) * kFX + 2 * xp);
			}
#pragma unroll
			for (int q = 0; q < K; ++q) {
				const float2 t = tpair[q];
				c0 = __ffma2_rn(col[2 * R - q], t, c0);
				c1 = __ffma2_rn(col[1 + 2 * R - q], t, c1);
			}
		}
	};

	auto store = [&](int zo, int y0, const float2& v0, const float2& v1) {
#pragma unroll
		for (int j = 0; j < 2; ++j) {
			const int y = y0 + 2 * yq + j;
			const float2 v = j == 0 ? v0 : v1;
			if (y < a.ny) {
				char* row = a.dst + y * a.d_stride[1] + zo * a.d_stride[2];
				if (a.dst_pairs && ox + 1 < a.nx) {
					*reinterpret_cast<float2*>(row + ox * 4LL) = v;
				} else {
					if (ox < a.nx) *reinterpret_cast<float*>(row + ox * a.d_stride[0]) = v.x;
					if (ox + 1 < a.nx) *reinterpret_cast<float*>(row + (ox + 1) * a.d_stride[0]) = v.y;
				}
			}
		}
	};

	if constexpr (!Z) {
		for (int p = 0; p < nplanes; ++p) {
			float2 c0, c1;
			filter_plane(p, c0, c1);
			store(0, y0_of(p), c0, c1);
		}
	} else {
		for (int p = 0; p < nplanes; ++p) {
			float2 n0, n1;
			filter_plane(p, n0, n1);
#pragma unroll
			for (int q = 0; q < K - 1; ++q) {
				win[0][q] = win[0][q + 1];
				win[1][q] = win[1][q + 1];
			}
			win[0][K - 1] = n0;
			win[1][K - 1] = n1;
			if (p >= 2 * R) {
				// output plane zs + p - 2R uses planes p - 2R .. p; tap q meets plane p - q
				float2 o0 = make_float2(0.0f, 0.0f), o1 = make_float2(0.0f, 0.0f);
#pragma unroll
				for (int q = 0; q < K; ++q) {
					const float2 t = tpair[16 + q];
					o0 = __ffma2_rn(win[0][K - 1 - q], t, o0);
					o1 = __ffma2_rn(win[1][K - 1 - q], t, o1);
				}
				store(zs + p - 2 * R, y0_of(0), o0, o1);
			}
		}
	}
}

// Ring variant for radius <= 4 on 3-D volumes with a TMA-addressable source (the common
// case). Same tile and stages, with the per-plane overhead taken out:
//   * two planes per iteration: the 2 x (16 + 2R) x 16 axis-0 row segments of both are dealt
//     out over the 256 threads together (3 or 2 each instead of 2 or 1), and two block
//     barriers serve two planes;
//   * the axis-2 window lives in a thread-private ring in shared memory of L >= K + 1 slots
//     (a power of two: the slot of plane m is m & (L - 1)); K + 1 conflict-free 128-bit loads
//     give both planes' outputs. No register rotation;
//   * all taps are held in registers;
//   * the clamp/mirror fix-up of out-of-image halo cells is a list of (cell, source cell)
//     pairs built once per block -- the x/y geometry is the same for every plane. Only cells
//     within R of the image are listed (the others feed no stored output); for images of at
//     least 16 x 16 their source cells lie inside the tile;
//   * only the thread that issues a plane's TMA maps its z coordinate.
constexpr int kRBuf = 4; // tile buffers: the iteration's two planes and the next two

template<int R>
struct RingGeom {
	using G = SepGeom<R>;
	static constexpr int L = R == 1 ? 4 : (R <= 3 ? 8 : 16);   // ring slots, >= K + 1
	static constexpr int FIX = 2 * R * (G::AW + G::AH);        // out-of-image cells within R of the image
	static constexpr int SEGS = G::AH * (kFX / 4);              // axis-0 row segments of one plane
	static constexpr size_t BYTES = static_cast<size_t>(kRBuf * G::A_FLOATS + 2 * G::B_FLOATS) * 4 +
		static_cast<size_t>(L) * kFThreads * 16 + static_cast<size_t>(FIX) * 4 + kRBuf * 8 + 16;
};

template<int R>
__global__ void __launch_bounds__(kFThreads, R <= 3 ? 3 : 2) separable_ring_kernel(
	const __grid_constant__ CUtensorMap map, const SepFastArgs a)
{
	using G = SepGeom<R>;
	using RG = RingGeom<R>;
	constexpr int K = G::K;
	constexpr int L = RG::L;
	constexpr int FIX = RG::FIX;
	constexpr int SEGS = RG::SEGS;
	static_assert(L >= K + 1 && (L & (L - 1)) == 0, "ring length");
	extern __shared__ __align__(128) unsigned char smem_raw[];
	float* A = reinterpret_cast<float*>(smem_raw);                              // kRBuf tiles
	float* Bbuf = A + kRBuf * G::A_FLOATS;                                       // axis-0 results, 2 planes
	float4* ring = reinterpret_cast<float4*>(Bbuf + 2 * G::B_FLOATS);            // [L][threads]
	uint32_t* fix = reinterpret_cast<uint32_t*>(ring + L * kFThreads);           // (cell << 16) | source
	uint64_t* bars = reinterpret_cast<uint64_t*>(fix + FIX);
	int* nfix_s = reinterpret_cast<int*>(bars + kRBuf);

	const int tid = threadIdx.x;
	const int x0 = blockIdx.x * kFX, y0 = blockIdx.y * kFY;
	const int zs = blockIdx.z * a.zchunk;
	const int ze = min(zs + a.zchunk, a.nz);
	const int nplanes = (ze - zs) + 2 * R;
	const int npairs = (nplanes + 1) / 2;   // an odd count reads one extra plane, never stored
	const bool interior = x0 - G::RA >= 0 && x0 + kFX + G::RA <= a.nx && y0 - R >= 0 && y0 + kFY + R <= a.ny;
	const bool fixup = !interior && a.border != IANE_GB_BORDER_ZERO;

	auto tap = [&](int axis, int i) -> float {
		if (!a.tap_ptr[axis]) {
			return i == R ? 1.0f : 0.0f;
		}
		const int q = i - (R - a.k[axis] / 2);
		return q >= 0 && q < a.k[axis] ? *reinterpret_cast<const float*>(a.tap_ptr[axis] + q * a.tap_stride[axis])
			: 0.0f;
	};
	float tx[K];
	float2 ty2[K], tz2[K];
#pragma unroll
	for (int i = 0; i < K; ++i) {
		tx[i] = tap(0, i);
		const float t1 = tap(1, i), t2 = tap(2, i);
		ty2[i] = make_float2(t1, t1);
		tz2[i] = make_float2(t2, t2);
	}
	if (tid == 0) {
		*nfix_s = 0;
		for (int b = 0; b < kRBuf; ++b) mbar_init(&bars[b], 1);
		fence_barrier_init();
	}
	__syncthreads();
	if (fixup) {
		const int gx0 = x0 - G::RA, gy0 = y0 - R;
		for (int i = tid; i < G::AW * G::AH; i += kFThreads) {
			const int r = i / G::AW, c = i - r * G::AW;
			const int gx = gx0 + c, gy = gy0 + r;
			const int dx = gx < 0 ? -gx : (gx >= a.nx ? gx - a.nx + 1 : 0);
			const int dy = gy < 0 ? -gy : (gy >= a.ny ? gy - a.ny + 1 : 0);
			if ((dx == 0 && dy == 0) || dx > R || dy > R) continue;
			int mx = 0, my = 0;
			map_coord(gx, a.nx, a.border, mx);
			map_coord(gy, a.ny, a.border, my);
			const int lc = mx - gx0, lr = my - gy0;
			if (lc < 0 || lc >= G::AW || lr < 0 || lr >= G::AH) continue; // cannot happen for images >= 16 x 16
			const int k = atomicAdd(nfix_s, 1);
			if (k < FIX) fix[k] = (static_cast<uint32_t>(i) << 16) | static_cast<uint32_t>(lr * G::AW + lc);
		}
	}
	__syncthreads();
	const int nfix = min(*nfix_s, FIX);

	// plane m of the sequence is input plane zs - R + m, in tile buffer m % kRBuf; thread 0 issues
	auto issue = [&](int m) {
		const int b = m % kRBuf;
		const int z = zs - R + m;
		int zi = 0;
		const bool present = map_coord(z, a.nz, a.border, zi);
		if (fixup) {
			// order this buffer's earlier generic-proxy writes (the fix-up) before the TMA
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
		}
		mbar_arrive_expect_tx(&bars[b], static_cast<uint32_t>(G::AW * G::AH * 4));
		tma_load_3d(A + b * G::A_FLOATS, &map, x0 - G::RA, y0 - R, present ? zi : z, &bars[b]);
	};
	if (tid == 0) {
		for (int m = 0; m < kRBuf && m < 2 * npairs; ++m) issue(m);
	}
	bool ok = true;
	auto wait_fix = [&](int m) {
		const int b = m % kRBuf;
		if (ok && !mbar_wait_bounded(&bars[b], (m / kRBuf) & 1)) {
			ok = false;
			report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
		}
		float* tile = A + b * G::A_FLOATS;
		for (int k = tid; k < nfix; k += kFThreads) {
			const uint32_t e = fix[k];
			tile[e >> 16] = tile[e & 0xFFFFu];
		}
	};

	const int xp = tid & 31, yq = tid >> 5;   // axes 1, 2: x pair 2xp, y rows 2yq, 2yq + 1
	const int ox = x0 + 2 * xp, oy = y0 + 2 * yq;
	const bool pairs = a.dst_pairs && ox + 1 < a.nx;
	char* row0 = a.dst + oy * a.d_stride[1] + ox * a.d_stride[0];
	char* row1 = row0 + a.d_stride[1];
	const bool y0_in = oy < a.ny, y1_in = oy + 1 < a.ny, x0_in = ox < a.nx, x1_in = ox + 1 < a.nx;
	float4* my_ring = ring + tid;

	auto store = [&](int zo, const float2& o0, const float2& o1) {
		const long long zoff = static_cast<long long>(zo) * a.d_stride[2];
		if (pairs) {
			if (y0_in) *reinterpret_cast<float2*>(row0 + zoff) = o0;
			if (y1_in) *reinterpret_cast<float2*>(row1 + zoff) = o1;
		} else {
			if (y0_in && x0_in) *reinterpret_cast<float*>(row0 + zoff) = o0.x;
			if (y0_in && x1_in) *reinterpret_cast<float*>(row0 + zoff + a.d_stride[0]) = o0.y;
			if (y1_in && x0_in) *reinterpret_cast<float*>(row1 + zoff) = o1.x;
			if (y1_in && x1_in) *reinterpret_cast<float*>(row1 + zoff + a.d_stride[0]) = o1.y;
		}
	};

	for (int pp = 0; pp < npairs; ++pp) {
		const int p = 2 * pp; // planes p and p + 1
		// planes p + 2 and p + 3 are in flight while p and p + 1 are filtered
		wait_fix(p);
		wait_fix(p + 1);
		if (nfix > 0) __syncthreads(); // fixed tiles visible to all
		// axis 0 of both planes into B[0], B[1]: segment it = (plane, row, 4-column group);
		// B's last readers (axis 1 of the previous iteration) finished before its second barrier
		for (int it = tid; it < 2 * SEGS; it += kFThreads) {
			const int pl = it >= SEGS ? 1 : 0;
			const int rem = it - pl * SEGS;
			const int r = rem >> 4, xq = rem & 15;
			const float* tile = A + ((p + pl) % kRBuf) * G::A_FLOATS;
			float seg[G::SEG];
			const float4* srow = reinterpret_cast<const float4*>(tile + r * G::AW + 4 * xq);
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
				for (int q = 0; q < K; ++q) acc = fmaf(tx[q], seg[G::D + i + 2 * R - q], acc);
				o[i] = acc;
			}
			*reinterpret_cast<float4*>(Bbuf + pl * G::B_FLOATS + r * kFX + 4 * xq) = make_float4(o[0], o[1], o[2], o[3]);
		}
		__syncthreads(); // B complete; the tiles of planes p, p + 1 are free
		// planes p + 4 and p + 5 go to their buffers, just released. Only planes this block waits
		// for are issued: no copy may still be in flight when the block exits.
		if (tid == 0) {
			if (p + 4 < 2 * npairs) issue(p + 4);
			if (p + 5 < 2 * npairs) issue(p + 5);
		}
#pragma unroll
		for (int pl = 0; pl < 2; ++pl) {
			const float* B = Bbuf + pl * G::B_FLOATS;
			float2 c0 = make_float2(0.0f, 0.0f), c1 = make_float2(0.0f, 0.0f);
			float2 col[2 + 2 * R];
#pragma unroll
			for (int m = 0; m < 2 + 2 * R; ++m) {
				col[m] = *reinterpret_cast<const float2*>(B + (2 * yq + m) * kFX + 2 * xp);
			}
#pragma unroll
			for (int q = 0; q < K; ++q) {
				c0 = __ffma2_rn(col[2 * R - q], ty2[q], c0);
				c1 = __ffma2_rn(col[1 + 2 * R - q], ty2[q], c1);
			}
			my_ring[((p + pl) & (L - 1)) * kFThreads] = make_float4(c0.x, c0.y, c1.x, c1.y);
		}
		__syncthreads(); // both B buffers read: the next iteration may overwrite them
		if (p + 1 >= 2 * R) {
			// output planes zs + p - 2R and zs + p + 1 - 2R; tap q meets planes p - q, p + 1 - q
			float2 a0 = make_float2(0.0f, 0.0f), a1 = make_float2(0.0f, 0.0f);   // plane p + 1's output
			float2 b0 = make_float2(0.0f, 0.0f), b1 = make_float2(0.0f, 0.0f);   // plane p's output
#pragma unroll
			for (int j = 0; j <= K; ++j) {
				const float4 v = my_ring[((p + 1 - j) & (L - 1)) * kFThreads]; // plane p + 1 - j
				if (j < K) {
					a0 = __ffma2_rn(make_float2(v.x, v.y), tz2[j], a0);
					a1 = __ffma2_rn(make_float2(v.z, v.w), tz2[j], a1);
				}
				if (j >= 1) {
					b0 = __ffma2_rn(make_float2(v.x, v.y), tz2[j - 1], b0);
					b1 = __ffma2_rn(make_float2(v.z, v.w), tz2[j - 1], b1);
				}
			}
			const int zo = zs + p - 2 * R;
			if (p >= 2 * R && zo < ze) store(zo, b0, b1);
			if (zo + 1 < ze) store(zo + 1, a0, a1);
		}
	}
}

template<int R>
int launch_radius(const DevView& src, const DevView* taps, const DevView& dst, int border, cudaStream_t stream)
{
	using G = SepGeom<R>;
	SepFastArgs a{};
	a.src = src.ptr;
	a.dst = dst.ptr;
	for (int i = 0; i < 3; ++i) {
		a.s_stride[i] = src.stride[i];
		a.d_stride[i] = dst.stride[i];
	}
	a.nx = src.ext[0];
	a.ny = src.ext[1];
	a.nz = src.ext[2];
	a.border = border;
	a.status = device_status_ptr();
	if (!a.status) return IANE_GB_CUDA_ERROR;
	for (int axis = 0; axis < 3; ++axis) {
		a.tap_ptr[axis] = taps[axis].ptr;
		a.tap_stride[axis] = taps[axis].stride[0];
		a.k[axis] = taps[axis].ext[0];
	}
	const bool z3 = src.ext[2] > 1 || taps[2].ext[0] > 1;
	// TMA wants positive, 16-byte multiple pitches that do not make rows or planes overlap.
	a.use_tma = (rows_aligned16(src) && (src.ext[1] <= 1 || src.stride[1] >= 4LL * src.ext[0]) &&
		(src.ext[2] <= 1 || (src.stride[2] > 0 && src.stride[2] >= (src.ext[1] > 1 ? src.stride[1] : 4LL * src.ext[0]) *
			src.ext[1]))) ? 1 : 0;
	a.dst_pairs = (dst.stride[0] == 4 && reinterpret_cast<uintptr_t>(dst.ptr) % 8 == 0 &&
		(dst.ext[1] <= 1 || dst.stride[1] % 8 == 0) && (dst.ext[2] <= 1 || dst.stride[2] % 8 == 0)) ? 1 : 0;
	CUtensorMap map{};
	if (a.use_tma) {
		const long long row = src.ext[1] > 1 ? src.stride[1] : ((static_cast<long long>(src.ext[0]) * 4 + 15) & ~15LL);
		const long long plane = src.ext[2] > 1 ? src.stride[2] : row * src.ext[1];
		const int status = encode_tensor_map_f32(&map, src.ptr, src.ext[0], src.ext[1], src.ext[2], row, plane, G::AW,
			G::AH);
		if (status) return status;
	}
	const long long columns = static_cast<long long>((a.nx + kFX - 1) / kFX) * ((a.ny + kFY - 1) / kFY);
	int chunk = a.nz;
	const int sms = device_sm_count();
	while (z3 && chunk > 4 * G::K && columns * ((a.nz + chunk - 1) / chunk) < 8LL * sms) {
		chunk = (chunk + 1) / 2;
	}
	a.zchunk = chunk;
	const size_t smem = (kNBuf * G::A_FLOATS + G::B_FLOATS) * sizeof(float) + 2 * 16 * sizeof(float2) +
		kNBuf * sizeof(uint64_t);
	const dim3 grid((a.nx + kFX - 1) / kFX, (a.ny + kFY - 1) / kFY, z3 ? (a.nz + chunk - 1) / chunk : 1);
	if constexpr (R <= 4) {
		if (z3 && a.use_tma && a.nx >= 16 && a.ny >= 16) {
			const size_t rsmem = RingGeom<R>::BYTES;
			IANE_GB_CUDA(cudaFuncSetAttribute(separable_ring_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
				static_cast<int>(rsmem)), "separable: set shared memory size");
			// z chunks per column: the count that maximises the busy fraction of the last wave
			// times the share of planes that are not the chunk's 2R halo, from at least one wave
			int per_sm = 1;
			cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, separable_ring_kernel<R>, kFThreads, rsmem);
			const double slots = static_cast<double>(std::max(per_sm, 1)) * sms;
			int best_chunk = chunk;
			double best = -1.0;
			for (int c = 1; c <= a.nz && c <= 256; ++c) {
				const int len = (a.nz + c - 1) / c;
				if (len < 2 * G::K) break;
				const double waves = static_cast<double>(columns) * c / slots;
				if (waves < 1.0) continue;
				const double score = waves / std::ceil(waves) * len / (len + 2.0 * R);
				if (score > best) {
					best = score;
					best_chunk = len;
				}
			}
			a.zchunk = best_chunk;
			const dim3 rgrid(grid.x, grid.y, (a.nz + best_chunk - 1) / best_chunk);
			separable_ring_kernel<R><<<rgrid, kFThreads, rsmem, stream>>>(map, a);
			IANE_GB_CUDA(cudaGetLastError(), "separable: launch");
			return IANE_GB_OK;
		}
	}
	if (z3) {
		IANE_GB_CUDA(cudaFuncSetAttribute(separable_fast_kernel<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			static_cast<int>(smem)), "separable: set shared memory size");
		separable_fast_kernel<R, true><<<grid, kFThreads, smem, stream>>>(map, a);
	} else {
		auto kernel = separable_fast_kernel<R, false>;
		IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
			"separable: set shared memory size");
		// 2-D: blocks stream eight tile rows each (when that still gives several blocks per SM),
		// so a tile's load overlaps the previous tile's filtering
		dim3 g2 = grid;
		const unsigned int streamed = (grid.y + 7) / 8;
		if (static_cast<long long>(grid.x) * streamed >= 8LL * sms) g2.y = streamed;
		kernel<<<g2, kFThreads, smem, stream>>>(map, a);
	}
	IANE_GB_CUDA(cudaGetLastError(), "separable: launch");
	return IANE_GB_OK;
}

}  // namespace

int launch_conv_separable_fast(const DevView& src, const DevView* taps, const DevView& dst, int border,
	cudaStream_t stream)
{
	int r = 0;
	for (int i = 0; i < 3; ++i) r = max(r, taps[i].ext[0] / 2);
	if (src.stride[0] != 4 || r > 7 || src.ext[1] > 65535 * kFY || src.ext[2] > 65535 * 64) {
		return IANE_GB_UNSUPPORTED;
	}
	// large 2-D images stream down row strips (separable_rows.cu)
	const int rows = launch_separable_rows(src, taps, dst, border, stream);
	if (rows != IANE_GB_UNSUPPORTED) {
		return rows;
	}
	switch (r) {
	case 0:
	case 1: return launch_radius<1>(src, taps, dst, border, stream);
	case 2: return launch_radius<2>(src, taps, dst, border, stream);
	case 3: return launch_radius<3>(src, taps, dst, border, stream);
	case 4: return launch_radius<4>(src, taps, dst, border, stream);
	case 5: return launch_radius<5>(src, taps, dst, border, stream);
	case 6: return launch_radius<6>(src, taps, dst, border, stream);
	case 7: return launch_radius<7>(src, taps, dst, border, stream);
	default: return IANE_GB_UNSUPPORTED;
	}
}

}  // namespace iane_gb
