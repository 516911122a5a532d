// iane_gb_convolve's FP32 fast path: dispatch, and the instantiations for kernel widths 1..15.
#include "conv_f32.cuh"
#include "kernels.h"

namespace iane_gb {

int launch_f32_narrow(int kx, const DevView& src, const DevView& kernel, const DevView& dst, int border, bool tma, const TexSource* tex,
	cudaStream_t stream)
{
	switch (kx) {
	case 1: return launch_f32_kx<1>(src, kernel, dst, border, tma, tex, stream);
	case 3: return launch_f32_kx<3>(src, kernel, dst, border, tma, tex, stream);
	case 5: return launch_f32_kx<5>(src, kernel, dst, border, tma, tex, stream);
	case 7: return launch_f32_kx<7>(src, kernel, dst, border, tma, tex, stream);
	case 9: return launch_f32_kx<9>(src, kernel, dst, border, tma, tex, stream);
	case 11: return launch_f32_kx<11>(src, kernel, dst, border, tma, tex, stream);
	case 13: return launch_f32_kx<13>(src, kernel, dst, border, tma, tex, stream);
	case 15: return launch_f32_kx<15>(src, kernel, dst, border, tma, tex, stream);
	default: return IANE_GB_UNSUPPORTED;
	}
}

int launch_conv_f32_tiled(const DevView& src, const DevView& kernel, const DevView& dst, int border,
	cudaStream_t stream, const TexSource* tex)
{
	const int kx = kernel.ext[0], ky = kernel.ext[1], kz = kernel.ext[2];
	// FP32 sums of f32 taps: the fast mode's arithmetic for every source type but f64 (whose
	// fast mode sums in FP64) and integer kernels (int64 sums)
	if (kernel.dtype != IANE_GB_F32 || src.dtype == IANE_GB_F64 || src.dtype == IANE_GB_RGB8 ||
	    dst.dtype == IANE_GB_BF16 || dst.dtype == IANE_GB_RGB8) {
		return IANE_GB_UNSUPPORTED;
	}
	if (ky > 63 || src.ext[1] > 65535 * 32 || src.ext[2] > 65535) {
		return IANE_GB_UNSUPPORTED;
	}
	// Shared memory holds one or two kernel planes' taps (ky x 32 floats at most) next to the
	// halo tiles; the planes stream through it, so kz has no limit here.
	(void)kz;
	// TMA staging when the source is a TMA-addressable f32 view (16-byte aligned rows and
	// planes that do not overlap) and, for clamp and mirror, wider than the kernel radius on x
	// and y (the edge fix-up takes its sources from inside the tile); else per-element staging.
	const bool tma = !tex && src.dtype == IANE_GB_F32 && rows_aligned16(src) &&
		(src.ext[1] <= 1 || src.stride[1] >= 4LL * src.ext[0]) &&
		(src.ext[2] <= 1 || (src.stride[2] > 0 && src.stride[2] >= (src.ext[1] > 1 ? src.stride[1] : 4LL * src.ext[0]) *
			src.ext[1])) &&
		(border == IANE_GB_BORDER_ZERO || (src.ext[0] > kx / 2 && src.ext[1] > ky / 2));
	return kx <= 15 ? launch_f32_narrow(kx, src, kernel, dst, border, tma, tex, stream)
		: launch_f32_wide(kx, src, kernel, dst, border, tma, tex, stream);
}

}  // namespace iane_gb
