// iane_gb_convolve's FP32 fast path: the register-tiled kernel of conv_tile.cuh, with the halo
// tiles staged by TMA when the source is a TMA-addressable f32 view (clamp and mirror edges
// fixed up in shared memory), by 4-byte cp.async with the border rule applied per element for
// other f32 views, and by converting loads for other element types and texture sources.
#pragma once

#include "conv_tile.cuh"

namespace iane_gb {

template<int KX>
int launch_f32_kx(const DevView& src, const DevView& kernel, const DevView& dst, int border, bool tma, const TexSource* tex,
	cudaStream_t stream)
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
	if (tex) {
		a.stage = kStageTexture;
		a.tex = *tex;
	} else {
		a.stage = src.dtype == IANE_GB_F32 ? kStageF32 : kStageConvert;
		a.src_dtype = src.dtype;
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
	if (!tma) {
		return big ? launch_tile<KX, 2, 2, false>(map, a, epi, stream) : launch_tile<KX, 1, 1, false>(map, a, epi, stream);
	}
	// box = one halo tile at the shared-memory pitch, as the RL passes load theirs
	const long long row = src.ext[1] > 1 ? src.stride[1] : ((static_cast<long long>(src.ext[0]) * 4 + 15) & ~15LL);
	const long long plane = src.ext[2] > 1 ? src.stride[2] : row * src.ext[1];
	const int box_w = big ? TileWidth<KX, 2>::P : TileWidth<KX, 1>::P;
	const int box_h = (big ? 64 : 32) + 2 * (a.ky / 2);
	const int status = encode_tensor_map_f32(&map, src.ptr, src.ext[0], src.ext[1], src.ext[2], row, plane, box_w, box_h);
	if (status) return status;
	return big ? launch_tile<KX, 2, 2, true>(map, a, epi, stream) : launch_tile<KX, 1, 1, true>(map, a, epi, stream);
}

// Kernel widths 1..15 (conv_f32.cu) and 17..31 (conv_f32_wide.cu).
int launch_f32_narrow(int kx, const DevView& src, const DevView& kernel, const DevView& dst, int border, bool tma, const TexSource* tex,
	cudaStream_t stream);
int launch_f32_wide(int kx, const DevView& src, const DevView& kernel, const DevView& dst, int border, bool tma, const TexSource* tex,
	cudaStream_t stream);

}  // namespace iane_gb
