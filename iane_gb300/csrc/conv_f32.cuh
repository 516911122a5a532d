// iane_gb_convolve's FP32 fast path: the register-tiled kernel of conv_tile.cuh, with the halo
// tiles staged by TMA when the source is a TMA-addressable f32 view (clamp and mirror edges
// fixed up in shared memory), by 4-byte cp.async with the border rule applied per element for
// other f32 views, and by converting loads for other element types and texture sources.
#pragma once

#include "conv_tile.cuh"

namespace iane_gb {

template<int KX>
int launch_f32_kx(const DevView& src, const DevView& kernel, const DevView& dst, int border, int stage,
	const TexSource* tex, cudaStream_t stream)
{
	TileArgs a{};
	a.src = src.ptr;
	for (int i = 0; i < 3; ++i) {
		a.s_stride[i] = src.stride[i];
		a.k_stride[i] = kernel.stride[i];
	}
	a.nx = src.ext[0];
	a.ny = src.ext[1];
	a.nz = src.ext[2];
	a.ky = kernel.ext[1];
	a.kz = kernel.ext[2];
	a.kernel = kernel.ptr;
	a.border = border;
	a.src_dtype = src.dtype;
	if (tex) {
		a.stage = kStageTexture;
		a.tex = *tex;
	} else {
		a.stage = src.dtype == IANE_GB_F32 ? kStageF32 : kStageConvert;
	}
	a.status = device_status_ptr();
	if (!a.status) {
		return IANE_GB_CUDA_ERROR;
	}
	EpiStoreF32 epi{};
	epi.dst = dst.ptr;
	for (int i = 0; i < 3; ++i) epi.stride[i] = dst.stride[i];
	epi.nx = dst.ext[0];
	epi.ny = dst.ext[1];
	epi.vec4 = rows_aligned16(dst) ? 1 : 0;
	epi.dtype = dst.dtype;
	// Large images use 64x64 tiles; small ones 32x32 so that the grid still fills the GPU.
	const long long big_tiles = static_cast<long long>((a.nx + 63) / 64) * ((a.ny + 63) / 64) * a.nz;
	const bool big = big_tiles >= 2LL * device_sm_count();
	CUtensorMap map{};
	if (stage == kTileTmaNarrow) {
		// the raw staging buffers come on top of the float tiles: element staging instead where
		// they would not fit (16-bit images with the widest and tallest kernels)
		const int es = dtype_size(src.dtype);
		const size_t need = big ? tile_smem_bytes<KX, 2, 2>(a.ky, a.kz, kTileTmaNarrow, es)
			: tile_smem_bytes<KX, 1, 1>(a.ky, a.kz, kTileTmaNarrow, es);
		if (need > 227u * 1024u) stage = kTileCopy;
	}
	// single-plane kernels on large images: direct summation (fewer registers, more blocks)
	const bool single = big && a.kz == 1;
	if (stage == kTileCopy) {
		return single ? launch_tile<KX, 2, 2, kTileCopy, true>(map, a, epi, stream)
			: big ? launch_tile<KX, 2, 2, kTileCopy>(map, a, epi, stream)
			: launch_tile<KX, 1, 1, kTileCopy>(map, a, epi, stream);
	}
	// box = one halo tile at the shared-memory pitch (f32) or the raw narrow box
	const int esize = dtype_size(src.dtype);
	const long long row = src.ext[1] > 1 ? src.stride[1] : ((static_cast<long long>(src.ext[0]) * esize + 15) & ~15LL);
	const long long plane = src.ext[2] > 1 ? src.stride[2] : row * src.ext[1];
	const int box_h = (big ? 64 : 32) + 2 * (a.ky / 2);
	if (stage == kTileTma) {
		const int box_w = big ? TileWidth<KX, 2>::P : TileWidth<KX, 1>::P;
		const int status =
			encode_tensor_map_f32(&map, src.ptr, src.ext[0], src.ext[1], src.ext[2], row, plane, box_w, box_h);
		if (status) return status;
		// 3-D kernels up to 15 wide take 16 x 2 outputs per lane: fewer kernel-row loads and checks
		// per FMA, the same sums. Wider ones keep 8 x 4, whose row segment needs fewer registers,
		// and so do single-plane kernels: 16 x 2 costs them the seventh block per SM, and held to
		// 72 registers it still measured slower (8192^2 7x7 mirror: 0.166 -> 0.176 / 0.192 ms).
		constexpr int RX = KX <= 15 ? 16 : kRX, RY = KX <= 15 ? 2 : kRY;
		return single ? launch_tile<KX, 2, 2, kTileTma, true>(map, a, epi, stream)
			: big ? launch_tile<KX, 2, 2, kTileTma, false, RX, RY>(map, a, epi, stream)
			: launch_tile<KX, 1, 1, kTileTma>(map, a, epi, stream);
	}
	const int box_w = big ? narrow_box_elems<KX, 2>(esize) : narrow_box_elems<KX, 1>(esize);
	const int status = encode_tensor_map(&map, esize == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16,
		src.ptr, src.ext[0], src.ext[1], src.ext[2], row, plane, box_w, box_h);
	if (status) return status;
	return single ? launch_tile<KX, 2, 2, kTileTmaNarrow, true>(map, a, epi, stream)
		: big ? launch_tile<KX, 2, 2, kTileTmaNarrow>(map, a, epi, stream)
		: launch_tile<KX, 1, 1, kTileTmaNarrow>(map, a, epi, stream);
}

// The instantiations for kernel widths K1 and K2, one pair per translation unit
// (conv_f32_k*.cu) so that they compile in parallel.
#define IANE_GB_F32_WIDTHS(NAME, K1, K2)                                                                      \
	int NAME(int kx, const DevView& src, const DevView& kernel, const DevView& dst, int border, int stage,    \
		const TexSource* tex, cudaStream_t stream)                                                           \
	{                                                                                                         \
		if (kx == K1) return launch_f32_kx<K1>(src, kernel, dst, border, stage, tex, stream);                 \
		if (kx == K2) return launch_f32_kx<K2>(src, kernel, dst, border, stage, tex, stream);                 \
		return IANE_GB_UNSUPPORTED;                                                                           \
	}

using LaunchF32Widths = int (*)(int, const DevView&, const DevView&, const DevView&, int, int, const TexSource*,
	cudaStream_t);
int launch_f32_k1_3(int, const DevView&, const DevView&, const DevView&, int, int, const TexSource*, cudaStream_t);
int launch_f32_k5_7(int, const DevView&, const DevView&, const DevView&, int, int, const TexSource*, cudaStream_t);
int launch_f32_k9_11(int, const DevView&, const DevView&, const DevView&, int, int, const TexSource*, cudaStream_t);
int launch_f32_k13_15(int, const DevView&, const DevView&, const DevView&, int, int, const TexSource*, cudaStream_t);
int launch_f32_k17_19(int, const DevView&, const DevView&, const DevView&, int, int, const TexSource*, cudaStream_t);
int launch_f32_k21_23(int, const DevView&, const DevView&, const DevView&, int, int, const TexSource*, cudaStream_t);
int launch_f32_k25_27(int, const DevView&, const DevView&, const DevView&, int, int, const TexSource*, cudaStream_t);
int launch_f32_k29_31(int, const DevView&, const DevView&, const DevView&, int, int, const TexSource*, cudaStream_t);

}  // namespace iane_gb
