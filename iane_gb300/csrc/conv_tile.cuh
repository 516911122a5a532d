// Register-tiled FP32 direct convolution core, shared by iane_gb_convolve's fast path and
// the two fused Richardson-Lucy passes.
//
// Geometry (one output plane z per block, kernel planes streamed through shared memory):
//   * a warp is 4 (x) x 8 (y) lanes; each lane owns kRX=8 consecutive x by kRY=4
//     consecutive y outputs, so a warp covers 32x32 and a block of WX x WY warps covers
//     (32 WX) x (32 WY) outputs;
//   * for each kernel plane qz the input halo tile of that plane, (TX + 2 rx) x (TY + 2 ry)
//     floats, is staged in shared memory -- by one TMA (cp.async.bulk.tensor, zero fill
//     outside the image; for clamp and mirror borders, tiles at the image edge then rewrite
//     their out-of-image cells from the cells the rule maps them to) when the buffer is
//     TMA-addressable (STAGE kTileTma; for 8- and 16-bit integer images, kTileTmaNarrow, the
//     TMA lands the tile's raw elements in a byte staging buffer and the block converts them
//     to floats), else element by element with the border rule applied (kTileCopy: 4-byte
//     cp.async for f32, batched loads and conversion for other element types and textures) --
//     double buffered, so the next plane lands while this one is consumed;
//   * a lane walks the RY + 2 ry input rows it needs; each row segment (8 + 2 rx floats) is
//     read once with 128-bit shared loads into registers and feeds every (output row j,
//     kernel row b) pair that uses it: 8 x KX FMAs per (j, b) against a kernel row that is
//     read as a warp-uniform broadcast (packed f32x2 FMAs were measured slower here: half
//     the taps need operand pairs at odd offsets, and the register moves that build them
//     cost more issue slots than the packing saves);
//   * only the current and next kernel planes' taps are held in shared memory, so four
//     64x64-tile blocks fit per SM.
// A second lane geometry (template RX = 16, RY = 2: 2 x 16 lanes, each 16 x by 2 y outputs)
// covers the same 32 x 32 per warp and reads the same tile (its width does not depend on RX):
// per kernel row it loads the taps once for 16 x 2 = 32 FMAs per tap instead of twice, and
// the interior input rows, which feed both output rows, run without the kernel-row checks.
// The persistent RL kernel and the 3-D fast convolve up to 15 wide use it; the sums are the
// same bits in either geometry (each output's taps are added in the same order).
// Per kernel plane each output accumulates its ky*kx taps into a plane partial that is
// added to the total afterwards (two-level FP32 summation), which keeps the rounding error
// of a 1575-tap sum near 1e-6 relative. Single-plane kernels (SINGLE) sum straight into the
// total: the same bits (the total would be +0 + the plane partial, and a sum that starts at
// +0 is never -0) with 32 fewer live registers, so more blocks fit per SM.
//
// Coordinates follow the reference's convolution_filter (include/iane/algorithms/
// convolution.hpp:37-45): out[p] = sum_q K[q] * in[p + size/2 - q].
#pragma once

#include "common.cuh"

namespace iane_gb {

constexpr int kRX = 8;
constexpr int kRY = 4;

template<int KX>
struct TileGeom {
	static constexpr int rx = KX / 2;
	static constexpr int RXA = (rx + 3) & ~3;              // x halo rounded to a 16-byte boundary
	static constexpr int D = RXA - rx;                      // segment lead-in
	static constexpr int SEGN = (D + kRX + KX - 1 + 3) & ~3; // floats per row segment (multiple of 4)
	static constexpr int KXP = (KX + 3) & ~3;               // padded kernel row in shared memory
};

template<int KX, int WX>
struct TileWidth {
	static constexpr int TX = 32 * WX;
	static constexpr int W = TX - kRX + TileGeom<KX>::SEGN;  // columns read
	static constexpr int P = (W % 8 == 0) ? W + 4 : W;        // pitch, = 4 mod 8 floats
};

// How halo tiles reach shared memory (the STAGE template argument).
constexpr int kTileCopy = 0;       // element by element (TileArgs::stage says how)
constexpr int kTileTma = 1;        // one TMA of f32 elements
constexpr int kTileTmaNarrow = 2;  // one TMA of 8- or 16-bit integers, converted in shared memory

// Narrow TMA boxes start 16 elements left of the tile (a 16-byte-aligned x for 1- and 2-byte
// elements) and cover the float tile's W columns from G::RXA left of it.
template<int KX, int WX>
__host__ __device__ constexpr int narrow_box_elems(int esize)
{
	return (((16 - TileGeom<KX>::RXA + TileWidth<KX, WX>::W) * esize + 15) & ~15) / esize;
}
template<int KX, int WX, int WY>
__host__ __device__ inline size_t narrow_stage_bytes(int ky, int esize)
{
	const int H = 32 * WY + 2 * (ky / 2);
	return (static_cast<size_t>(narrow_box_elems<KX, WX>(esize)) * esize * H + 127) & ~size_t(127);
}

// How the element-by-element path stages a halo tile.
enum TileStage : int {
	kStageF32 = 0,     // f32 source, 4-byte cp.async
	kStageConvert = 1, // any element type (TileArgs::src_dtype), converted to float while loading
	kStageTexture = 2, // texels of TileArgs::tex, converted to float
};

struct TileArgs {
	// source of the halo tiles, used by the non-TMA path (the TMA path reads the tensor map)
	const char* src;
	long long s_stride[3];
	int nx, ny, nz;
	int stage;     // TileStage
	int src_dtype; // kStageConvert: element type of src
	TexSource tex; // kStageTexture: the texture and the view's origin
	// kernel: kx is the template KX; f32 device view
	int ky, kz;
	const char* kernel;
	long long k_stride[3];
	int border;
	int* status; // device status word for bounded waits
};

// Halo-tile and tap buffers: two (double buffering across kernel planes) for 3-D kernels,
// one for single-plane kernels, which have nothing to double-buffer.
__host__ __device__ inline int tile_buffers(int kz) { return kz > 1 ? 2 : 1; }

// Shared memory bytes of one launch: float tiles and taps, the two tile mbarriers and, for
// kTileTmaNarrow (esize = element bytes), the staging buffers 128 bytes after the barriers.
template<int KX, int WX, int WY>
inline size_t tile_smem_bytes(int ky, int kz, int stage = kTileCopy, int esize = 0)
{
	const int H = 32 * WY + 2 * (ky / 2);
	const size_t plane = (static_cast<size_t>(TileWidth<KX, WX>::P) * H * 4 + 127) & ~size_t(127);
	const size_t psf = (static_cast<size_t>(ky) * TileGeom<KX>::KXP * 4 + 127) & ~size_t(127);
	const size_t base = tile_buffers(kz) * (plane + psf);
	if (stage == kTileTmaNarrow) {
		return base + 128 + tile_buffers(kz) * narrow_stage_bytes<KX, WX, WY>(ky, esize);
	}
	return base + 16;
}

// Element-by-element staging for element types other than f32 and for textures: batches of
// loads are issued before any is stored so that their latencies overlap; integer and bf16
// elements are loaded raw by size and converted afterwards.
template<int W, int P, int NT>
__device__ __forceinline__ void stage_elements(const TileArgs& a, float* dst, int gx0, int gy0, int H, int zi, bool zok)
{
	constexpr int kBatch = 8;
	const int tid = threadIdx.x;
	const int n = W * H;
	const char* plane = a.src + zi * a.s_stride[2];
	const bool texture = a.stage == kStageTexture;
	const int esize = a.src_dtype == IANE_GB_U8 || a.src_dtype == IANE_GB_I8 ? 1 :
		(a.src_dtype == IANE_GB_U16 || a.src_dtype == IANE_GB_I16 || a.src_dtype == IANE_GB_BF16 ? 2 : 4);
	for (int base = tid; base < n; base += NT * kBatch) {
		uint32_t raw[kBatch]; // element bits, or a texel's float bits
		uint32_t in = 0;      // bit u: sample u lies in the image (else it is the zero value)
#pragma unroll
		for (int u = 0; u < kBatch; ++u) {
			const int i = base + u * NT;
			raw[u] = 0;
			if (i < n) {
				const int r = i / W, c = i - (i / W) * W;
				int xi = 0, yi = 0;
				if (zok && map_coord(gx0 + c, a.nx, a.border, xi) && map_coord(gy0 + r, a.ny, a.border, yi)) {
					in |= 1u << u;
					if (texture) {
						raw[u] = __float_as_uint(texel_as_float(a.tex.tex, a.tex.dtype, a.tex.rank, a.tex.origin[0] + xi,
							a.tex.origin[1] + yi, a.tex.origin[2] + zi));
					} else {
						const char* q = plane + xi * a.s_stride[0] + yi * a.s_stride[1];
						raw[u] = esize == 1 ? static_cast<uint32_t>(*reinterpret_cast<const uint8_t*>(q))
							: esize == 2 ? static_cast<uint32_t>(*reinterpret_cast<const uint16_t*>(q))
							: *reinterpret_cast<const uint32_t*>(q);
					}
				}
			}
		}
#pragma unroll
		for (int u = 0; u < kBatch; ++u) {
			const int i = base + u * NT;
			if (i >= n) break;
			float v = 0.0f;
			if (in & (1u << u)) {
				const int dt = texture ? IANE_GB_F32 : a.src_dtype;
				switch (dt) {
				case IANE_GB_U8: case IANE_GB_U16: case IANE_GB_U32: v = static_cast<float>(raw[u]); break;
				case IANE_GB_I8: v = static_cast<float>(static_cast<int8_t>(raw[u])); break;
				case IANE_GB_I16: v = static_cast<float>(static_cast<int16_t>(raw[u])); break;
				case IANE_GB_I32: v = static_cast<float>(static_cast<int32_t>(raw[u])); break;
				case IANE_GB_BF16: v = __uint_as_float(raw[u] << 16); break;
				default: v = __uint_as_float(raw[u]); break; // f32 bits
				}
			}
			const int r = i / W, c = i - (i / W) * W;
			dst[r * P + c] = v;
		}
	}
}

// kTileTmaNarrow: convert the raw staged box (row pitch `pitch` bytes) into the float tile,
// four cells at a time: OFF = 16 - RXA and W are multiples of 4, so each group of four is one
// 4-byte (8-bit types) or 8-byte (16-bit) load from the staging row and one 16-byte store.
template<int W, int P, int NT, int OFF>
__device__ __forceinline__ void convert_narrow(const unsigned char* sg, float* t, int H, int pitch, int dtype)
{
	static_assert(W % 4 == 0 && OFF % 4 == 0 && P % 4 == 0, "vector conversion");
	constexpr int G4 = W / 4; // groups of four cells per row
	const int tid = threadIdx.x;
	for (int i = tid; i < G4 * H; i += NT) {
		const int r = i / G4, g = i - r * G4;
		float4 v;
		if (dtype == IANE_GB_U8 || dtype == IANE_GB_I8) {
			const uint32_t w = *reinterpret_cast<const uint32_t*>(sg + r * pitch + OFF + 4 * g);
			if (dtype == IANE_GB_U8) {
				v = make_float4(static_cast<float>(w & 0xffu), static_cast<float>((w >> 8) & 0xffu),
					static_cast<float>((w >> 16) & 0xffu), static_cast<float>(w >> 24));
			} else {
				v = make_float4(static_cast<float>(static_cast<int8_t>(w & 0xffu)),
					static_cast<float>(static_cast<int8_t>((w >> 8) & 0xffu)),
					static_cast<float>(static_cast<int8_t>((w >> 16) & 0xffu)), static_cast<float>(static_cast<int8_t>(w >> 24)));
			}
		} else {
			const uint2 w = *reinterpret_cast<const uint2*>(sg + r * pitch + 2 * (OFF + 4 * g));
			if (dtype == IANE_GB_U16) {
				v = make_float4(static_cast<float>(w.x & 0xffffu), static_cast<float>(w.x >> 16),
					static_cast<float>(w.y & 0xffffu), static_cast<float>(w.y >> 16));
			} else {
				v = make_float4(static_cast<float>(static_cast<int16_t>(w.x & 0xffffu)),
					static_cast<float>(static_cast<int16_t>(w.x >> 16)), static_cast<float>(static_cast<int16_t>(w.y & 0xffffu)),
					static_cast<float>(static_cast<int16_t>(w.y >> 16)));
			}
		}
		*reinterpret_cast<float4*>(t + r * P + 4 * g) = v;
	}
}

// Input row r of the lane's window: read its segment once and apply it to every output row j
// whose kernel row b = j + 2 ry - r exists (CHECK false: the caller knows all of them do).
template<int KX, int P, int RX, int RY, bool CHECK>
__device__ __forceinline__ void row_sums(float (&sum)[RY][RX], const float* tile, const float* kplane, int ry, int ky,
	int r)
{
	using G = TileGeom<KX>;
	constexpr int SEGN = (G::D + RX + KX - 1 + 3) & ~3;
	float seg[SEGN];
	const float4* srow = reinterpret_cast<const float4*>(tile + r * P);
#pragma unroll
	for (int m = 0; m < SEGN / 4; ++m) {
		const float4 v = srow[m];
		seg[4 * m + 0] = v.x;
		seg[4 * m + 1] = v.y;
		seg[4 * m + 2] = v.z;
		seg[4 * m + 3] = v.w;
	}
#pragma unroll
	for (int j = 0; j < RY; ++j) {
		const int b = j + 2 * ry - r;
		if (!CHECK || (b >= 0 && b < ky)) {
			const float4* krow = reinterpret_cast<const float4*>(kplane + b * G::KXP);
			float k[G::KXP];
#pragma unroll
			for (int m = 0; m < G::KXP / 4; ++m) {
				const float4 v = krow[m];
				k[4 * m + 0] = v.x;
				k[4 * m + 1] = v.y;
				k[4 * m + 2] = v.z;
				k[4 * m + 3] = v.w;
			}
#pragma unroll
			for (int q = 0; q < KX; ++q) {
#pragma unroll
				for (int i = 0; i < RX; ++i) {
					sum[j][i] = fmaf(k[q], seg[G::D + i + 2 * G::rx - q], sum[j][i]);
				}
			}
		}
	}
}

template<int KX, int P, int RX = kRX, int RY = kRY>
__device__ __forceinline__ void plane_sums(float (&sum)[RY][RX], const float* tile, const float* kplane, int ry, int ky)
{
	const int rows = RY + 2 * ry;
	if constexpr (RX == kRX) {
#pragma unroll 1
		for (int r = 0; r < rows; ++r) row_sums<KX, P, RX, RY, true>(sum, tile, kplane, ry, ky, r);
	} else {
		// rows RY - 1 .. 2 ry feed all RY output rows; the first and last RY - 1 rows feed some
		const int lo = RY - 1 < 2 * ry + 1 ? RY - 1 : 2 * ry + 1;
		const int hi = 2 * ry + 1 > lo ? 2 * ry + 1 : lo;
#pragma unroll 1
		for (int r = 0; r < lo; ++r) row_sums<KX, P, RX, RY, true>(sum, tile, kplane, ry, ky, r);
#pragma unroll 1
		for (int r = lo; r < hi; ++r) row_sums<KX, P, RX, RY, false>(sum, tile, kplane, ry, ky, r);
#pragma unroll 1
		for (int r = hi; r < rows; ++r) row_sums<KX, P, RX, RY, true>(sum, tile, kplane, ry, ky, r);
	}
}

// The sums of one output tile (x0, y0, z) of the tiled convolution: acc[j][i] is the output
// at (xo + i, yo + j, z) with (xo, yo) from tile_origin(). Persistent kernels call it once per
// work item; `phases` carries the parity of the next wait on each tile buffer's mbarrier
// (bit b for buffer b) from one call to the next, and `bars` are the two tile mbarriers (TMA
// stages), initialised by the caller. The caller applies its epilogue to acc afterwards, so
// none of the epilogue's state is live during the sums.
// taps_resident: a single-plane caller's previous call left this kernel's taps in shared memory.
template<int KX, int WX, int WY, int STAGE, bool SINGLE = false, int RX = kRX, int RY = kRY>
__device__ __forceinline__ void conv_tile_sums(const CUtensorMap* tmap_ptr, const TileArgs& a, int x0, int y0, int z,
	uint32_t& phases, uint64_t* bars, float (&acc)[RY][RX], bool taps_resident = false)
{
	static_assert(RX % 4 == 0 && RX * RY == kRX * kRY && 32 % RX == 0, "a lane owns 32 outputs of a 32 x 32 warp tile");
	constexpr int LX = 32 / RX; // lanes along x in a warp
	using G = TileGeom<KX>;
	constexpr int TX = 32 * WX;
	constexpr int TY = 32 * WY;
	constexpr int P = TileWidth<KX, WX>::P;
	constexpr int W = TileWidth<KX, WX>::W;
	constexpr int NT = 32 * WX * WY;
	extern __shared__ __align__(128) unsigned char smem_raw[];

	const int ky = a.ky, kz = a.kz;
	const int ry = ky / 2, rz = kz / 2;
	const int H = TY + 2 * ry;
	const int plane_floats = ((P * H + 31) & ~31);
	float* tiles = reinterpret_cast<float*>(smem_raw);
	float* psf_s = tiles + tile_buffers(kz) * plane_floats; // taps of one or two kernel planes
	const int psf_floats = ((ky * G::KXP + 31) & ~31);

	const int tid = threadIdx.x;
	const int lane = tid & 31, warp = tid >> 5;
	// kTileTmaNarrow: raw boxes of narrow_pitch bytes per row, 128 bytes after the barriers
	unsigned char* narrow = reinterpret_cast<unsigned char*>(bars) + 128;
	const int esize = (a.src_dtype == IANE_GB_U8 || a.src_dtype == IANE_GB_I8) ? 1 : 2;
	const int narrow_pitch = narrow_box_elems<KX, WX>(esize) * esize;
	const int narrow_buf = static_cast<int>(narrow_stage_bytes<KX, WX, WY>(ky, esize));
	const int tx_b = (warp % WX) * LX + (lane % LX);
	const int ty_b = (warp / WX) * (32 / LX) + (lane / LX);
	// a warp whose 32 x 32 outputs all lie outside the image (the ragged last tiles) skips the
	// sums: the epilogue stores nothing there, so no result changes
	const bool warp_active = x0 + 32 * (warp % WX) < a.nx && y0 + 32 * (warp / WX) < a.ny;

	// Kernel planes that touch the image: all of them except, for a zero border, planes
	// whose input plane lies outside (those contribute only zero samples).
	int qz_lo = 0, qz_hi = kz - 1;
	if (a.border == IANE_GB_BORDER_ZERO) {
		qz_lo = max(0, z + rz - (a.nz - 1));
		qz_hi = min(kz - 1, z + rz);
	}
	const int nplanes = qz_hi - qz_lo + 1;

	// Taps of kernel plane qz_lo + p into tap buffer p & 1.
	auto load_taps = [&](int p) {
		const int qz = qz_lo + p;
		float* dst = psf_s + (p & 1) * psf_floats;
		for (int i = tid; i < ky * G::KXP; i += NT) {
			const int qx = i % G::KXP, qy = i / G::KXP;
			float v = 0.0f;
			if (qx < KX) {
				v = *reinterpret_cast<const float*>(a.kernel + qx * a.k_stride[0] + qy * a.k_stride[1] +
					qz * a.k_stride[2]);
			}
			dst[i] = v;
		}
	};
	if (nplanes > 0 && !(SINGLE && taps_resident)) load_taps(0);
	if (nplanes > 1) load_taps(1);
	__syncthreads(); // taps visible; every lane is done with the previous tile's buffers

	auto issue = [&](int p) {
		float* dst = tiles + (p & 1) * plane_floats;
		const int qz = qz_lo + p;
		if constexpr (STAGE != kTileCopy) {
			if (tid == 0) {
				// zero border: an out-of-volume plane is never issued (qz range above); clamp
				// and mirror: the plane the rule maps to
				int zi = z + rz - qz;
				if (a.border != IANE_GB_BORDER_ZERO) map_coord(z + rz - qz, a.nz, a.border, zi);
				// order earlier generic-proxy use of this buffer before the async-proxy write
				asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
				if constexpr (STAGE == kTileTma) {
					mbar_arrive_expect_tx(&bars[p & 1], static_cast<uint32_t>(P * H * 4));
					tma_load_3d(dst, tmap_ptr, x0 - G::RXA, y0 - ry, zi, &bars[p & 1]);
				} else {
					mbar_arrive_expect_tx(&bars[p & 1], static_cast<uint32_t>(narrow_pitch * H));
					tma_load_3d(narrow + (p & 1) * narrow_buf, tmap_ptr, x0 - 16, y0 - ry, zi, &bars[p & 1]);
				}
			}
		} else {
			int zi = 0;
			const bool zok = map_coord(z + rz - qz, a.nz, a.border, zi);
			const char* plane = a.src + zi * a.s_stride[2];
			if (a.stage == kStageF32) {
				for (int i = tid; i < W * H; i += NT) {
					const int col = i % W, row = i / W;
					int xi = 0, yi = 0;
					const bool ok = zok && map_coord(x0 - G::RXA + col, a.nx, a.border, xi) &&
						map_coord(y0 - ry + row, a.ny, a.border, yi);
					const char* src = ok ? plane + xi * a.s_stride[0] + yi * a.s_stride[1] : a.src;
					cp_async4(dst + row * P + col, src, ok ? 4 : 0);
				}
			} else {
				// plain loads and stores; the wait and barrier before the tile is read order them
				stage_elements<W, P, NT>(a, dst, x0 - G::RXA, y0 - ry, H, zi, zok);
			}
			cp_async_commit();
		}
	};


#pragma unroll
	for (int j = 0; j < RY; ++j)
#pragma unroll
		for (int i = 0; i < RX; ++i) acc[j][i] = 0.0f;

	bool ok = true;
	// TMA with a clamp or mirror border: a tile that reaches outside the image gets its
	// out-of-image cells within (rx, ry) of the image -- the only ones stored outputs read --
	// from the in-image cells the rule maps them to. Those lie inside the tile whenever
	// nx > rx and ny > ry (the launcher's condition); any other cell keeps the TMA's zeros.
	const bool fix_tile = STAGE != kTileCopy && a.border != IANE_GB_BORDER_ZERO &&
		!(x0 - G::RXA >= 0 && x0 - G::RXA + W <= a.nx && y0 - ry >= 0 && y0 + TY + ry <= a.ny);
	if (nplanes > 0) issue(0);
	if (nplanes > 1) issue(1);
	for (int p = 0; p < nplanes; ++p) {
		if constexpr (STAGE != kTileCopy) {
			const uint32_t bit = 1u << (p & 1);
			if (ok && !mbar_wait_bounded(&bars[p & 1], (phases & bit) ? 1u : 0u)) {
				ok = false;
				report_device_status(a.status, IANE_GB_DEVICE_TIMEOUT);
			}
			phases ^= bit;
			if constexpr (STAGE == kTileTmaNarrow) {
				convert_narrow<W, P, NT, 16 - G::RXA>(narrow + (p & 1) * narrow_buf, tiles + (p & 1) * plane_floats, H,
					narrow_pitch, a.src_dtype);
				__syncthreads(); // converted tile visible to all lanes
			}
			if (fix_tile) {
				float* t = tiles + (p & 1) * plane_floats;
				const int gx0 = x0 - G::RXA, gy0 = y0 - ry;
				for (int i = tid; i < W * H; i += NT) {
					const int r = i / W, c = i - r * W;
					const int gx = gx0 + c, gy = gy0 + r;
					const int dx = gx < 0 ? -gx : (gx >= a.nx ? gx - a.nx + 1 : 0);
					const int dy = gy < 0 ? -gy : (gy >= a.ny ? gy - a.ny + 1 : 0);
					if ((dx == 0 && dy == 0) || dx > G::rx || dy > ry) continue;
					int mx = 0, my = 0;
					map_coord(gx, a.nx, a.border, mx);
					map_coord(gy, a.ny, a.border, my);
					const int lc = mx - gx0, lr = my - gy0;
					if (lc < 0 || lc >= W || lr < 0 || lr >= H) continue;
					t[r * P + c] = t[lr * P + lc];
				}
				__syncthreads(); // fixed tile visible to all lanes
			}
		} else {
			if (p + 1 < nplanes) {
				cp_async_wait<1>();
			} else {
				cp_async_wait<0>();
			}
			__syncthreads();
		}
		const float* tile = tiles + (p & 1) * plane_floats + (RY * ty_b) * P + RX * tx_b;
		const float* kplane = psf_s + (p & 1) * psf_floats;
		if (!warp_active) {
			// nothing to sum
		} else if constexpr (SINGLE) {
			plane_sums<KX, P, RX, RY>(acc, tile, kplane, ry, ky);
		} else {
			float part[RY][RX];
#pragma unroll
			for (int j = 0; j < RY; ++j)
#pragma unroll
				for (int i = 0; i < RX; ++i) part[j][i] = 0.0f;
			plane_sums<KX, P, RX, RY>(part, tile, kplane, ry, ky);
#pragma unroll
			for (int j = 0; j < RY; ++j)
#pragma unroll
				for (int i = 0; i < RX; ++i) acc[j][i] += part[j][i];
		}


		__syncthreads(); // every lane is done with this plane's tile and taps
		if (p + 2 < nplanes) {
			issue(p + 2);
			load_taps(p + 2);
		}
	}
}

// Origin of this thread's RX x RY outputs within the tile at (x0, y0) of a WX-warp-wide block.
template<int WX, int RX = kRX, int RY = kRY>
__device__ __forceinline__ void tile_origin(int x0, int y0, int& xo, int& yo)
{
	constexpr int LX = 32 / RX;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	xo = x0 + RX * ((warp % WX) * LX + (lane % LX));
	yo = y0 + RY * ((warp / WX) * (32 / LX) + (lane / LX));
}

// Shared memory bytes of the tile barriers (after the tiles and taps of conv_tile_sums).
template<int KX, int WX, int WY>
__device__ __forceinline__ uint64_t* tile_barriers(int ky, int kz)
{
	extern __shared__ __align__(128) unsigned char smem_raw[];
	const int H = 32 * WY + 2 * (ky / 2);
	const int plane_floats = ((TileWidth<KX, WX>::P * H + 31) & ~31);
	const int psf_floats = ((ky * TileGeom<KX>::KXP + 31) & ~31);
	return reinterpret_cast<uint64_t*>(reinterpret_cast<float*>(smem_raw) +
		tile_buffers(kz) * (plane_floats + psf_floats));
}

template<int KX, int WX, int WY, int STAGE, class Epi, bool SINGLE, int RX, int RY>
__global__ void __launch_bounds__(32 * WX * WY)
	conv_tile_kernel(const __grid_constant__ CUtensorMap tmap, const TileArgs a, const __grid_constant__ Epi epi_in)
{
	if constexpr (STAGE != kTileCopy) {
		if (threadIdx.x == 0) {
			uint64_t* bars = tile_barriers<KX, WX, WY>(a.ky, a.kz);
			mbar_init(&bars[0], 1);
			mbar_init(&bars[1], 1);
			fence_barrier_init();
		}
	}
	uint32_t phases = 0;
	const int x0 = blockIdx.x * 32 * WX, y0 = blockIdx.y * 32 * WY;
	float acc[RY][RX];
	conv_tile_sums<KX, WX, WY, STAGE, SINGLE, RX, RY>(&tmap, a, x0, y0, blockIdx.z, phases,
		tile_barriers<KX, WX, WY>(a.ky, a.kz), acc);
	// the epilogue's state (pointers, Kahan sums) comes to life only after the sums
	Epi epi = epi_in;
	int xo = 0, yo = 0;
	tile_origin<WX, RX, RY>(x0, y0, xo, yo);
#pragma unroll
	for (int j = 0; j < RY; ++j) {
		epi.row(xo, yo + j, blockIdx.z, acc[j]);
	}
	epi.finish();
}

// Launch helper: grid = tiles over (x, y) and one block per output plane; RX x RY outputs per lane.
template<int KX, int WX, int WY, int STAGE, bool SINGLE = false, int RX = kRX, int RY = kRY, class Epi>
int launch_tile(const CUtensorMap& map, const TileArgs& a, const Epi& epi, cudaStream_t stream)
{
	auto kernel = conv_tile_kernel<KX, WX, WY, STAGE, Epi, SINGLE, RX, RY>;
	const int esize = (a.src_dtype == IANE_GB_U8 || a.src_dtype == IANE_GB_I8) ? 1 : 2;
	const size_t smem = tile_smem_bytes<KX, WX, WY>(a.ky, a.kz, STAGE, esize);
	IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
		"tiled convolution: set shared memory size");
	const dim3 grid((a.nx + 32 * WX - 1) / (32 * WX), (a.ny + 32 * WY - 1) / (32 * WY), a.nz);
	kernel<<<grid, 32 * WX * WY, smem, stream>>>(map, a, epi);
	IANE_GB_CUDA(cudaGetLastError(), "tiled convolution: launch");
	return IANE_GB_OK;
}

// Store epilogue for iane_gb_convolve: f32 destinations directly (16-byte stores where rows
// allow), other element types through the reference's conversion of the sum.
struct EpiStoreF32 {
	char* dst;
	long long stride[3];
	int nx, ny;
	int vec4;   // rows start 16-byte aligned and axis 0 is packed
	int dtype;  // destination element type (0 or IANE_GB_F32: f32)

	// N outputs of one row starting at xo (N 8 or 16; xo a multiple of N)
	template<int N>
	__device__ __forceinline__ void row(int xo, int y, int z, const float (&v)[N]) const
	{
		static_assert(N == 8 || N == 16, "8 or 16 outputs per lane row");
		if (y >= ny) {
			return;
		}
		char* base = dst + y * stride[1] + z * stride[2];
		if (dtype != 0 && dtype != IANE_GB_F32) {
			if (dtype == IANE_GB_U8 && vec4 && xo + N <= nx) {
				// packed rows: the lane's N bytes in one N-byte store
				uint32_t w[N / 4] = {};
#pragma unroll
				for (int i = 0; i < N; ++i) w[i >> 2] |= static_cast<uint32_t>(convert_f32_u8(v[i])) << (8 * (i & 3));
				if constexpr (N == 8) {
					*reinterpret_cast<uint2*>(base + xo) = make_uint2(w[0], w[1]);
				} else {
					*reinterpret_cast<uint4*>(base + xo) = make_uint4(w[0], w[1], w[2], w[3]);
				}
				return;
			}
#pragma unroll
			for (int i = 0; i < N; ++i) {
				if (xo + i < nx) {
					store_converted_f32(base + (xo + i) * stride[0], dtype, v[i]);
				}
			}
			return;
		}
		if (vec4 && xo + N <= nx) {
			float4* p = reinterpret_cast<float4*>(base + xo * 4LL);
#pragma unroll
			for (int m = 0; m < N / 4; ++m) p[m] = make_float4(v[4 * m], v[4 * m + 1], v[4 * m + 2], v[4 * m + 3]);
			return;
		}
#pragma unroll
		for (int i = 0; i < N; ++i) {
			if (xo + i < nx) {
				*reinterpret_cast<float*>(base + (xo + i) * stride[0]) = v[i];
			}
		}
	}
	__device__ __forceinline__ void finish() const {}
};

}  // namespace iane_gb
