// Flat morphology: erosion, dilation and the prepared opening / closing of the reference's
// include/iane/algorithms/morphology/morphology.hpp (rank 1-3 here).
//
// erode(p)  = min over footprint offsets o of sample(p + o)
// dilate(p) = max over footprint offsets o of sample(p - o)
// with o = position - radius for positions in [0, 2 r] in raster order (axis 0 fastest), the
// border rule applied per axis (a zero-border sample is the value 0 and takes part), and the
// reference's update rule `value < result` (`>` for dilation) starting from +inf / -inf (the
// type's max / lowest for integers): NaN never replaces the running value, an all-NaN
// neighbourhood stays at the start value, and among equal values (-0 and +0) the first in
// scan order wins (morphology.hpp:44-71).
//
// Box footprints run separably -- x then y in shared memory per plane, then z over a ring of
// plane results in the same kernel (a second kernel for very deep z windows) -- in the same
// order per axis as the reference's raster scan (reversed for
// dilation, whose samples run p + r down to p - r). The first extreme of the raster scan is
// the first extreme along z of the first along y of the first along x, so the separable
// result is bit-identical, signed zeros included. Masked footprints (any subset of the box)
// take the direct kernel, which scans the footprint in raster order.
#include "common.cuh"
#include "kernels.h"

#include <limits>
#include <string>
#include <type_traits>

namespace iane_gb {
namespace {

constexpr int kTX = 32;  // box kernel: outputs per block along x
constexpr int kTY = 32;  //             and along y (8 rows of threads, 4 outputs each)

template<class T> __device__ __forceinline__ T start_value(bool dilate)
{
	if constexpr (std::is_floating_point_v<T>) {
		return dilate ? -std::numeric_limits<T>::infinity() : std::numeric_limits<T>::infinity();
	} else {
		return dilate ? std::numeric_limits<T>::lowest() : std::numeric_limits<T>::max();
	}
}

template<bool DILATE, class T> __device__ __forceinline__ void take(T v, T& r)
{
	if (DILATE ? v > r : v < r) r = v;
}

// The reference's scan of 2 r + 1 taps from p with stride `step` (negative for dilation).
template<bool DILATE, class T>
__device__ __forceinline__ T scan(const T* p, int taps, int step)
{
	T m = start_value<T>(DILATE);
#pragma unroll 4
	for (int o = 0; o < taps; ++o, p += step) take<DILATE>(*p, m);
	return m;
}

template<class T> __device__ __forceinline__ T sample(const DevView& v, int x, int y, int z, int border)
{
	int xi = 0, yi = 0, zi = 0;
	if (map_coord(x, v.ext[0], border, xi) && map_coord(y, v.ext[1], border, yi) && map_coord(z, v.ext[2], border, zi)) {
		return *element_ptr<T>(v, xi, yi, zi);
	}
	return T(0);
}

// Stage the (32 + 2 rx) x (32 + 2 ry) tile of plane zm (zok false: the zero plane) whose
// corner is (x0 - rx, y0 - ry): one row per warp step, the row's y mapped once, interior rows
// without per-element border mapping. 256 threads as 8 rows of 32.
template<class T>
__device__ __forceinline__ void load_tile(const DevView& src, T* tile, int x0, int y0, int rx, int ry, int zm, bool zok,
	int border)
{
	const int tw = kTX + 2 * rx, th = kTY + 2 * ry;
	const int gx0 = x0 - rx;
	const bool x_inside = gx0 >= 0 && gx0 + tw <= src.ext[0];
	for (int r = threadIdx.y; r < th; r += 8) {
		int yi = 0;
		const bool yok = zok && map_coord(y0 - ry + r, src.ext[1], border, yi);
		const char* row = src.ptr + yi * src.stride[1] + zm * src.stride[2];
		T* out = tile + r * tw;
		if (!yok) {
			for (int c = threadIdx.x; c < tw; c += 32) out[c] = T(0);
		} else if (x_inside) {
			for (int c = threadIdx.x; c < tw; c += 32) out[c] = *reinterpret_cast<const T*>(row + (gx0 + c) * src.stride[0]);
		} else {
			for (int c = threadIdx.x; c < tw; c += 32) {
				int xi = 0;
				out[c] = map_coord(gx0 + c, src.ext[0], border, xi) ? *reinterpret_cast<const T*>(row + xi * src.stride[0])
					: T(0);
			}
		}
	}
}

// Box footprint, x then y, for one 32x32 output tile of plane blockIdx.z. Shared memory: the
// (32 + 2 rx) x (32 + 2 ry) input tile, then the 32 x (32 + 2 ry) x-pass results.
template<class T, bool DILATE>
__global__ void __launch_bounds__(256) morph_box_xy_kernel(DevView src, DevView dst, int rx, int ry, int border)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int tw = kTX + 2 * rx, th = kTY + 2 * ry;
	T* tile = reinterpret_cast<T*>(smem_raw);
	T* xbuf = tile + tw * th;
	const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY, z = blockIdx.z;
	load_tile<T>(src, tile, x0, y0, rx, ry, z, true, border);
	__syncthreads();
	for (int r = threadIdx.y; r < th; r += 8) {
		xbuf[r * kTX + threadIdx.x] =
			scan<DILATE>(tile + r * tw + threadIdx.x + (DILATE ? 2 * rx : 0), 2 * rx + 1, DILATE ? -1 : 1);
	}
	__syncthreads();
	const int x = x0 + threadIdx.x;
	if (x >= dst.ext[0]) return;
	for (int k = 0; k < kTY / 8; ++k) {
		const int r = threadIdx.y + 8 * k;
		const int y = y0 + r;
		if (y >= dst.ext[1]) break;
		*const_cast<T*>(element_ptr<T>(dst, x, y, z)) = scan<DILATE>(
			xbuf + (r + (DILATE ? 2 * ry : 0)) * kTX + threadIdx.x, 2 * ry + 1, DILATE ? -kTX : kTX);
	}
}

// Box footprint in 3-D, fused: the block owns a 32x32 column of planes [z0, z0 + zc). Each
// input plane of [z0 - rz, z0 + zc + rz) is staged, reduced along x then y into a ring of
// 2 rz + 1 xy-results in shared memory, and every output plane whose z window is complete is
// reduced over the ring in scan order (increasing z for erosion, decreasing for dilation):
// one read of each input plane per chunk (plus 2 rz halo planes) and one write per output.
template<class T, bool DILATE>
__global__ void __launch_bounds__(256) morph_box_3d_kernel(DevView src, DevView dst, int rx, int ry, int rz, int zc,
	int border)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int tw = kTX + 2 * rx, th = kTY + 2 * ry;
	const int depth = 2 * rz + 1;
	T* ring = reinterpret_cast<T*>(smem_raw);      // depth x 32 x 32
	T* tile = ring + depth * kTX * kTY;            // tw x th
	T* xbuf = tile + tw * th;                      // 32 x th
	const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
	const int z0 = blockIdx.z * zc;
	const int z1 = min(dst.ext[2], z0 + zc);
	const int nz = src.ext[2];
	int slot_new = 0; // ring slot of plane zi: (zi - (z0 - rz)) mod depth
	for (int zi = z0 - rz; zi < z1 + rz; ++zi, slot_new = slot_new + 1 == depth ? 0 : slot_new + 1) {
		int zm = 0;
		const bool zok = map_coord(zi, nz, border, zm);
		load_tile<T>(src, tile, x0, y0, rx, ry, zm, zok, border);
		__syncthreads();
		for (int r = threadIdx.y; r < th; r += 8) {
			xbuf[r * kTX + threadIdx.x] =
				scan<DILATE>(tile + r * tw + threadIdx.x + (DILATE ? 2 * rx : 0), 2 * rx + 1, DILATE ? -1 : 1);
		}
		__syncthreads();
		T* slot = ring + slot_new * (kTX * kTY);
		for (int k = 0; k < kTY / 8; ++k) {
			const int r = threadIdx.y + 8 * k;
			slot[r * kTX + threadIdx.x] = scan<DILATE>(
				xbuf + (r + (DILATE ? 2 * ry : 0)) * kTX + threadIdx.x, 2 * ry + 1, DILATE ? -kTX : kTX);
		}
		__syncthreads();
		const int zo = zi - rz; // the output plane whose window ends at zi
		if (zo >= z0) {
			const int x = x0 + threadIdx.x;
			if (x < dst.ext[0]) {
				for (int k = 0; k < kTY / 8; ++k) {
					const int r = threadIdx.y + 8 * k;
					const int y = y0 + r;
					if (y >= dst.ext[1]) break;
					// the window zo - rz .. zo + rz = the ring's planes, the oldest in slot_new + 1
					T m = start_value<T>(DILATE);
					int sl = DILATE ? slot_new : (slot_new + 1 == depth ? 0 : slot_new + 1);
					for (int o = 0; o <= 2 * rz; ++o) {
						take<DILATE>(ring[sl * (kTX * kTY) + r * kTX + threadIdx.x], m);
						sl = DILATE ? (sl == 0 ? depth - 1 : sl - 1) : (sl + 1 == depth ? 0 : sl + 1);
					}
					*const_cast<T*>(element_ptr<T>(dst, x, y, zo)) = m;
				}
			}
		}
		// the next plane's y pass overwrites the oldest ring slot only after the barriers of
		// its tile and x passes, which every thread reaches after this reduction
	}
}

// The y pass of the cube kernel for one thread's OY consecutive outputs: col[q] is the x-pass
// result of tile row OY * ty + q, and output k takes rows k .. k + 2 R in the reference's order
// (increasing for erosion, decreasing for dilation). For 2 R >= OY every window holds rows OY - 1
// and OY, so it splits there into a part inside rows [0, OY) and a part inside [OY, k + 2 R];
// the two parts' first extremes are running values shared by the outputs, and combining them
// in scan order gives the first extreme of the whole window (the reference's `value < result`
// rule is associative over consecutive runs of the scan). Erosion scans the lower part first,
// so its partials are extended towards lower rows keeping ties (<=) and the upper partial
// towards higher rows replacing only on <; dilation mirrors this (upper part first, extended
// towards higher rows keeping ties (>=), lower part replacing only on >).
template<class T, bool DILATE, int R, int OY>
__device__ __forceinline__ void cube_y_pass(const T (&col)[OY + 2 * R], T (&m)[OY])
{
	if constexpr (2 * R >= OY) {
		T part[OY];
		T run = start_value<T>(DILATE);
#pragma unroll
		for (int k = OY - 1; k >= 0; --k) {
			const T v = col[k];
			if (DILATE ? v > run : v <= run) run = v;
			part[k] = run;
		}
		T edge = start_value<T>(DILATE);
#pragma unroll
		for (int j = OY; j < OY + 2 * R; ++j) {
			const T v = col[j];
			if (DILATE ? v >= edge : v < edge) edge = v;
			const int k = j - 2 * R;
			if (k >= 0) {
				if constexpr (DILATE) {
					m[k] = part[k] > edge ? part[k] : edge;
				} else {
					m[k] = edge < part[k] ? edge : part[k];
				}
			}
		}
	} else {
#pragma unroll
		for (int k = 0; k < OY; ++k) {
			T v = start_value<T>(DILATE);
#pragma unroll
			for (int o = 0; o <= 2 * R; ++o) take<DILATE>(col[k + (DILATE ? 2 * R - o : o)], v);
			m[k] = v;
		}
	}
}

// Cube footprints of radius R = 1, 2 or 3 in 3-D (the common case), fused like
// morph_box_3d_kernel with the scans fully unrolled. Thread (tx, ty) owns the outputs
// (x0 + tx, y0 + 4 ty + k), k < 4, of every plane of the chunk and keeps the xy results of the
// last 2 R + 1 input planes for them in registers. The 256 threads stage the tile's cells
// linearly (cell tid + 256 m), the same cells in every input plane, so their in-plane byte
// offsets and border rule are worked out once per block, and the next plane's cells are
// loaded into registers while the current plane is scanned. Same scan order as the reference
// (erosion: x, y and z increasing; dilation: decreasing).
template<class T, bool DILATE, int R>
__global__ void __launch_bounds__(256, sizeof(T) == 8 || R == 3 ? 2 : 3) morph_cube_kernel(DevView src, DevView dst, int zc, int border)
{
	constexpr int K = 2 * R + 1;
	constexpr int TW = kTX + 2 * R, TH = kTY + 2 * R;
	constexpr int NCELL = TW * TH;
	constexpr int M = (NCELL + 255) / 256; // staged cells per thread
	constexpr int OY = kTY / 8;            // consecutive output rows per thread
	extern __shared__ __align__(16) unsigned char smem_raw[];
	T* tile = reinterpret_cast<T*>(smem_raw); // TW x TH
	T* xbuf = tile + NCELL;                   // 32 x TH
	const int tx = threadIdx.x, ty = threadIdx.y;
	const int tid = ty * 32 + tx;
	const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
	const int z0 = blockIdx.z * zc;
	const int z1 = min(dst.ext[2], z0 + zc);
	const int nz = src.ext[2];

	// In-plane byte offsets of the staged cells (32-bit: the launcher sends views whose plane
	// spans more than 2^31 bytes elsewhere); bit m of `live` marks a cell that holds a sample
	// (a cell of the tile with its bit clear is a zero-border 0)
	int off[M];
	unsigned live = 0;
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int c = tid + 256 * m;
		const int r = c / TW, q = c - r * TW;
		int xi = 0, yi = 0;
		if (c < NCELL && map_coord(x0 - R + q, src.ext[0], border, xi) && map_coord(y0 - R + r, src.ext[1], border, yi)) {
			live |= 1u << m;
		}
		off[m] = xi * static_cast<int>(src.stride[0]) + yi * static_cast<int>(src.stride[1]);
	}
	T cell[M];
	auto fetch = [&](int zi) {
		int zm = 0;
		const bool zok = map_coord(zi, nz, border, zm);
		const char* base = src.ptr + static_cast<long long>(zm) * src.stride[2];
#pragma unroll
		for (int m = 0; m < M; ++m) cell[m] = zok && (live >> m & 1u) ? *reinterpret_cast<const T*>(base + off[m]) : T(0);
	};

	const int x = x0 + tx;
	const int yb = y0 + OY * ty;
	const int rows_out = x < dst.ext[0] ? min(OY, dst.ext[1] - yb) : 0;
	const int out_row = static_cast<int>(dst.stride[1]);
	char* const out_base = dst.ptr + (rows_out > 0 ? x * static_cast<int>(dst.stride[0]) + yb * out_row : 0);
	T win[OY][K]; // [k][slot], slot K - 1 the newest plane
#pragma unroll
	for (int k = 0; k < OY; ++k)
#pragma unroll
		for (int s = 0; s < K; ++s) win[k][s] = start_value<T>(DILATE);
	fetch(z0 - R);
	for (int zi = z0 - R; zi < z1 + R; ++zi) {
#pragma unroll
		for (int m = 0; m < M; ++m) {
			if (m + 1 < M || tid + 256 * m < NCELL) tile[tid + 256 * m] = cell[m];
		}
		if (zi + 1 < z1 + R) fetch(zi + 1); // in flight while this plane is scanned
		__syncthreads();
#pragma unroll
		for (int i = 0; i < (TH + 7) / 8; ++i) {
			const int r = ty + 8 * i;
			if (r < TH) {
				const T* row = tile + r * TW + tx;
				T v = start_value<T>(DILATE);
#pragma unroll
				for (int o = 0; o < K; ++o) take<DILATE>(row[DILATE ? 2 * R - o : o], v);
				xbuf[r * kTX + tx] = v;
			}
		}
		__syncthreads();
		T col[OY + 2 * R];
#pragma unroll
		for (int q = 0; q < OY + 2 * R; ++q) col[q] = xbuf[(OY * ty + q) * kTX + tx];
		T ym[OY];
		cube_y_pass<T, DILATE, R, OY>(col, ym);
#pragma unroll
		for (int k = 0; k < OY; ++k) {
#pragma unroll
			for (int s = 0; s < K - 1; ++s) win[k][s] = win[k][s + 1];
			win[k][K - 1] = ym[k];
		}
		const int zo = zi - R; // the output plane whose window ends at zi
		if (zo >= z0) {
			char* const out = out_base + static_cast<long long>(zo) * dst.stride[2];
#pragma unroll
			for (int k = 0; k < OY; ++k) {
				if (k < rows_out) {
					T v = start_value<T>(DILATE);
#pragma unroll
					for (int o = 0; o < K; ++o) take<DILATE>(win[k][DILATE ? K - 1 - o : o], v);
					*reinterpret_cast<T*>(out + k * out_row) = v;
				}
			}
		}
		// the next plane's staging and x pass come after this thread's y pass: both of its
		// barriers follow every thread's reads of tile and xbuf
	}
}

// Box footprint along z (after the xy pass): one output per thread.
template<class T, bool DILATE>
__global__ void __launch_bounds__(256) morph_box_z_kernel(DevView src, DevView dst, int rz, int border)
{
	const int x = blockIdx.x * 32 + threadIdx.x;
	const int y = blockIdx.y * 8 + threadIdx.y;
	const int z = blockIdx.z;
	if (x >= dst.ext[0] || y >= dst.ext[1]) return;
	T m = start_value<T>(DILATE);
	for (int o = 0; o <= 2 * rz; ++o) {
		int zi = 0;
		const int zs = DILATE ? z + rz - o : z - rz + o;
		const T v = map_coord(zs, src.ext[2], border, zi) ? *element_ptr<T>(src, x, y, zi) : T(0);
		take<DILATE>(v, m);
	}
	*const_cast<T*>(element_ptr<T>(dst, x, y, z)) = m;
}

// Any flat footprint (mask of (2r+1) per axis, raster order, nonzero = contained): one output
// per thread, the footprint scanned in raster order.
template<class T, bool DILATE>
__global__ void __launch_bounds__(256) morph_direct_kernel(DevView src, DevView dst, int rx, int ry, int rz,
	const uint8_t* __restrict__ mask, int border)
{
	const int x = blockIdx.x * 32 + threadIdx.x;
	const int y = blockIdx.y * 8 + threadIdx.y;
	const int z = blockIdx.z;
	if (x >= dst.ext[0] || y >= dst.ext[1]) return;
	T m = start_value<T>(DILATE);
	int q = 0;
	for (int pz = 0; pz <= 2 * rz; ++pz) {
		for (int py = 0; py <= 2 * ry; ++py) {
			for (int px = 0; px <= 2 * rx; ++px, ++q) {
				if (mask && !mask[q]) continue;
				const int ox = px - rx, oy = py - ry, oz = pz - rz;
				const T v = DILATE ? sample<T>(src, x - ox, y - oy, z - oz, border) : sample<T>(src, x + ox, y + oy, z + oz, border);
				take<DILATE>(v, m);
			}
		}
	}
	*const_cast<T*>(element_ptr<T>(dst, x, y, z)) = m;
}

// Whether every in-plane byte offset of the view fits in an int (the cube kernel's offsets).
bool plane_offsets_fit(const DevView& v)
{
	constexpr long long kMax = std::numeric_limits<int>::max();
	long long span = 0;
	for (int a = 0; a < 2; ++a) {
		if (v.ext[a] <= 1) continue;
		const long long st = v.stride[a] < 0 ? -v.stride[a] : v.stride[a];
		if (st > kMax) return false;
		span += static_cast<long long>(v.ext[a] - 1) * st;
	}
	return span <= kMax;
}

size_t box_xy_smem(int rx, int ry, int esize)
{
	return static_cast<size_t>((kTX + 2 * rx) * (kTY + 2 * ry) + kTX * (kTY + 2 * ry)) * esize;
}

size_t box_3d_smem(int rx, int ry, int rz, int esize)
{
	return box_xy_smem(rx, ry, esize) + static_cast<size_t>(2 * rz + 1) * kTX * kTY * esize;
}

template<class T, bool DILATE>
int launch_op(const DevView& s, const DevView& d, const int* r, const uint8_t* mask, int border, void* temp,
	cudaStream_t st)
{
	const dim3 g8((d.ext[0] + 31) / 32, (d.ext[1] + 7) / 8, d.ext[2]);
	if (mask) {
		morph_direct_kernel<T, DILATE><<<g8, dim3(32, 8), 0, st>>>(s, d, r[0], r[1], r[2], mask, border);
		IANE_GB_CUDA(cudaGetLastError(), "morphology: launch");
		return IANE_GB_OK;
	}
	const size_t smem = box_xy_smem(r[0], r[1], sizeof(T));
	if (smem > 200 * 1024) {
		morph_direct_kernel<T, DILATE><<<g8, dim3(32, 8), 0, st>>>(s, d, r[0], r[1], r[2], nullptr, border);
		IANE_GB_CUDA(cudaGetLastError(), "morphology: launch");
		return IANE_GB_OK;
	}
	auto xy = morph_box_xy_kernel<T, DILATE>;
	IANE_GB_CUDA(cudaFuncSetAttribute(xy, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
		"morphology: shared memory");
	const dim3 gt((d.ext[0] + kTX - 1) / kTX, (d.ext[1] + kTY - 1) / kTY, d.ext[2]);
	if (r[2] == 0) {
		xy<<<gt, dim3(32, 8), smem, st>>>(s, d, r[0], r[1], border);
		IANE_GB_CUDA(cudaGetLastError(), "morphology: launch");
		return IANE_GB_OK;
	}
	if (r[0] == r[1] && r[1] == r[2] && r[0] >= 1 && r[0] <= 3 && plane_offsets_fit(s) && plane_offsets_fit(d)) {
		// cube footprint: the unrolled kernel with the z window in registers
		const long long tiles = static_cast<long long>(gt.x) * gt.y;
		int zc = 32;
		while (zc > 4 && tiles * ((d.ext[2] + zc - 1) / zc) < 8LL * device_sm_count()) zc /= 2;
		const dim3 g3(gt.x, gt.y, (d.ext[2] + zc - 1) / zc);
		const size_t sm = box_xy_smem(r[0], r[0], sizeof(T));
		if (r[0] == 1) {
			morph_cube_kernel<T, DILATE, 1><<<g3, dim3(32, 8), sm, st>>>(s, d, zc, border);
		} else if (r[0] == 2) {
			morph_cube_kernel<T, DILATE, 2><<<g3, dim3(32, 8), sm, st>>>(s, d, zc, border);
		} else {
			morph_cube_kernel<T, DILATE, 3><<<g3, dim3(32, 8), sm, st>>>(s, d, zc, border);
		}
		IANE_GB_CUDA(cudaGetLastError(), "morphology: launch");
		return IANE_GB_OK;
	}
	const size_t smem3 = box_3d_smem(r[0], r[1], r[2], sizeof(T));
	if (smem3 <= 100 * 1024) {
		// fused 3-D box: chunks of zc output planes per block, enough blocks to fill the GPU
		const long long tiles = static_cast<long long>(gt.x) * gt.y;
		int zc = 32;
		while (zc > 4 && tiles * ((d.ext[2] + zc - 1) / zc) < 8LL * device_sm_count()) zc /= 2;
		auto k3 = morph_box_3d_kernel<T, DILATE>;
		IANE_GB_CUDA(cudaFuncSetAttribute(k3, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem3)),
			"morphology: shared memory");
		const dim3 g3(gt.x, gt.y, (d.ext[2] + zc - 1) / zc);
		k3<<<g3, dim3(32, 8), smem3, st>>>(s, d, r[0], r[1], r[2], zc, border);
		IANE_GB_CUDA(cudaGetLastError(), "morphology: launch");
		return IANE_GB_OK;
	}
	// 3-D box with a deep z window: xy into a packed temporary, then z into the destination
	DevView t{};
	t.ptr = static_cast<char*>(temp);
	t.dtype = d.dtype;
	t.rank = d.rank;
	for (int i = 0; i < 3; ++i) t.ext[i] = d.ext[i];
	t.stride[0] = sizeof(T);
	t.stride[1] = t.stride[0] * t.ext[0];
	t.stride[2] = t.stride[1] * t.ext[1];
	xy<<<gt, dim3(32, 8), smem, st>>>(s, t, r[0], r[1], border);
	morph_box_z_kernel<T, DILATE><<<g8, dim3(32, 8), 0, st>>>(t, d, r[2], border);
	IANE_GB_CUDA(cudaGetLastError(), "morphology: launch");
	return IANE_GB_OK;
}

template<class T>
int launch_typed(const DevView& s, const DevView& d, const int* r, const uint8_t* mask, int op, int border,
	void* temp, cudaStream_t st)
{
	return op == IANE_GB_DILATE ? launch_op<T, true>(s, d, r, mask, border, temp, st)
		: launch_op<T, false>(s, d, r, mask, border, temp, st);
}

int launch_any(const DevView& s, const DevView& d, const int* r, const uint8_t* mask, int op, int border, void* temp,
	cudaStream_t st)
{
	switch (s.dtype) {
	case IANE_GB_U8: return launch_typed<uint8_t>(s, d, r, mask, op, border, temp, st);
	case IANE_GB_I8: return launch_typed<int8_t>(s, d, r, mask, op, border, temp, st);
	case IANE_GB_U16: return launch_typed<uint16_t>(s, d, r, mask, op, border, temp, st);
	case IANE_GB_I16: return launch_typed<int16_t>(s, d, r, mask, op, border, temp, st);
	case IANE_GB_I32: return launch_typed<int32_t>(s, d, r, mask, op, border, temp, st);
	case IANE_GB_U32: return launch_typed<uint32_t>(s, d, r, mask, op, border, temp, st);
	case IANE_GB_F32: return launch_typed<float>(s, d, r, mask, op, border, temp, st);
	case IANE_GB_F64: return launch_typed<double>(s, d, r, mask, op, border, temp, st);
	default: return fail(IANE_GB_UNSUPPORTED, "morphology: element type (u8, i8, u16, i16, i32, u32, f32, f64)");
	}
}

// Shared argument checks; fills r[3] (unused axes 0).
int check_args(const iane_gb_view* src, const iane_gb_view* dst, const int32_t* radius, int border, DevView& s,
	DevView& d, int r[3])
{
	int status = normalise_view(src, "morphology source", &s);
	if (status) return status;
	status = normalise_view(dst, "morphology destination", &d);
	if (status) return status;
	if (!radius) return fail(IANE_GB_INVALID_ARGUMENT, "morphology: null radius");
	if (s.rank != d.rank) return fail(IANE_GB_INVALID_ARGUMENT, "morphology: source and destination need the same rank");
	if (s.dtype != d.dtype) {
		return fail(IANE_GB_INVALID_ARGUMENT, "morphology: source and destination need the same element type");
	}
	for (int i = 0; i < 3; ++i) {
		if (s.ext[i] != d.ext[i]) {
			return fail(IANE_GB_INVALID_ARGUMENT, "Source and destination require matching nonnegative dimensions");
		}
		r[i] = i < s.rank ? radius[i] : 0;
		// morphology.hpp:76-88
		if (r[i] < 0 || r[i] > 1 << 14) {
			return fail(IANE_GB_INVALID_ARGUMENT, "Morphology requires a nonnegative radius with representable width");
		}
	}
	if (border < IANE_GB_BORDER_CLAMP || border > IANE_GB_BORDER_MIRROR) {
		return fail(IANE_GB_INVALID_ARGUMENT, "morphology: unknown border mode");
	}
	if (s.ext[1] > 65535 * 8 || s.ext[2] > 65535) {
		return fail(IANE_GB_UNSUPPORTED, "morphology: image too large along axis 1 or 2 for the grid");
	}
	return IANE_GB_OK;
}

// The direct kernel scans the whole footprint per output: bound its work.
int check_direct(const int r[3], const uint8_t* mask, int esize)
{
	const bool direct = mask || box_xy_smem(r[0], r[1], esize) > 200 * 1024;
	const long long cells = static_cast<long long>(2 * r[0] + 1) * (2 * r[1] + 1) * (2 * r[2] + 1);
	if (direct && cells > (1LL << 20)) {
		return fail(IANE_GB_UNSUPPORTED, "morphology: footprint too large for the direct kernel (over 2^20 cells)");
	}
	return IANE_GB_OK;
}

size_t packed_bytes(const DevView& d)
{
	return (static_cast<size_t>(element_count(d)) * dtype_size(d.dtype) + 255) & ~size_t(255);
}

}  // namespace
}  // namespace iane_gb

using namespace iane_gb;

extern "C" {

int iane_gb_morphology(const iane_gb_view* src, const iane_gb_view* dst, const int32_t* radius,
	const uint8_t* footprint, int op, int border, void* stream)
{
	DevView s{}, d{};
	int r[3];
	int status = check_args(src, dst, radius, border, s, d, r);
	if (status) return status;
	if (op != IANE_GB_ERODE && op != IANE_GB_DILATE) {
		return fail(IANE_GB_INVALID_ARGUMENT, "morphology: op must be IANE_GB_ERODE or IANE_GB_DILATE");
	}
	if (element_count(s) == 0) return IANE_GB_OK;
	status = check_direct(r, footprint, dtype_size(d.dtype));
	if (status) return status;
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	void* temp = nullptr;
	const bool needs_temp = !footprint && r[2] > 0 && box_xy_smem(r[0], r[1], dtype_size(d.dtype)) <= 200 * 1024 &&
		box_3d_smem(r[0], r[1], r[2], dtype_size(d.dtype)) > 100 * 1024;
	if (needs_temp) {
		IANE_GB_CUDA(cudaMallocAsync(&temp, packed_bytes(d), st), "morphology: temporary");
	}
	status = launch_any(s, d, r, footprint, op, border, temp, st);
	if (temp) cudaFreeAsync(temp, st);
	return status;
}

size_t iane_gb_morphology_scratch_bytes(int dtype, int rank, const int32_t* extent)
{
	if (!extent || rank < 1 || rank > 3 || dtype_size(dtype) == 0) return 0;
	size_t count = 1;
	for (int i = 0; i < rank; ++i) count *= extent[i] > 0 ? static_cast<size_t>(extent[i]) : 0;
	// the intermediate image, and the temporary of a 3-D box pass
	return 2 * ((count * dtype_size(dtype) + 255) & ~size_t(255));
}

int iane_gb_morphology_compound(const iane_gb_view* src, const iane_gb_view* dst, const int32_t* radius,
	const uint8_t* footprint, int op, int border, void* scratch, size_t scratch_bytes, void* stream)
{
	DevView s{}, d{};
	int r[3];
	int status = check_args(src, dst, radius, border, s, d, r);
	if (status) return status;
	if (op != IANE_GB_OPENING && op != IANE_GB_CLOSING) {
		return fail(IANE_GB_INVALID_ARGUMENT, "morphology: op must be IANE_GB_OPENING or IANE_GB_CLOSING");
	}
	if (element_count(s) == 0) return IANE_GB_OK;
	status = check_direct(r, footprint, dtype_size(d.dtype));
	if (status) return status;
	const size_t image = packed_bytes(d);
	if (!scratch || scratch_bytes < 2 * image) {
		return fail(IANE_GB_LENGTH_ERROR, "morphology: scratch smaller than iane_gb_morphology_scratch_bytes");
	}
	// morphology.hpp:118-125: the first pass into a packed intermediate, the second into dst
	DevView mid = d;
	mid.ptr = static_cast<char*>(scratch);
	mid.stride[0] = dtype_size(d.dtype);
	mid.stride[1] = mid.stride[0] * d.ext[0];
	mid.stride[2] = mid.stride[1] * d.ext[1];
	void* temp = static_cast<char*>(scratch) + image;
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	const int first = op == IANE_GB_OPENING ? IANE_GB_ERODE : IANE_GB_DILATE;
	const int second = op == IANE_GB_OPENING ? IANE_GB_DILATE : IANE_GB_ERODE;
	status = launch_any(s, mid, r, footprint, first, border, temp, st);
	if (status) return status;
	return launch_any(mid, d, r, footprint, second, border, temp, st);
}

}  // extern "C"
