// iane_gb_convolve's FP32 fast path: dispatch, and the instantiations for kernel widths 1..15.
#include "conv_f32.cuh"
#include "kernels.h"

namespace iane_gb {

int launch_f32_narrow(int kx, const DevView& src, const DevView& kernel, const DevView& dst, int border, bool tma,
	cudaStream_t stream)
{
	switch (kx) {
	case 1: return launch_f32_kx<1>(src, kernel, dst, border, tma, stream);
	case 3: return launch_f32_kx<3>(src, kernel, dst, border, tma, stream);
	case 5: return launch_f32_kx<5>(src, kernel, dst, border, tma, stream);
	case 7: return launch_f32_kx<7>(src, kernel, dst, border, tma, stream);
	case 9: return launch_f32_kx<9>(src, kernel, dst, border, tma, stream);
	case 11: return launch_f32_kx<11>(src, kernel, dst, border, tma, stream);
	case 13: return launch_f32_kx<13>(src, kernel, dst, border, tma, stream);
	case 15: return launch_f32_kx<15>(src, kernel, dst, border, tma, stream);
	default: return IANE_GB_UNSUPPORTED;
	}
}

int launch_conv_f32_tiled(const DevView& src, const DevView& kernel, const DevView& dst, int border,
	cudaStream_t stream)
{
	const int kx = kernel.ext[0], ky = kernel.ext[1], kz = kernel.ext[2];
	if (src.dtype != IANE_GB_F32 || kernel.dtype != IANE_GB_F32 || dst.dtype != IANE_GB_F32) {
		return IANE_GB_UNSUPPORTED;
	}
	if (ky > 63 || src.ext[1] > 65535 * 32 || src.ext[2] > 65535) {
		return IANE_GB_UNSUPPORTED;
	}
	// Shared memory holds one or two kernel planes' taps (ky x 32 floats at most) next to the
	// halo tiles; the planes stream through it, so kz has no limit here.
	(void)kz;
	// TMA staging when the source is TMA-addressable (16-byte aligned rows and planes that do
	// not overlap) and, for clamp and mirror, wider than the kernel radius on x and y (the
	// edge fix-up takes its sources from inside the tile); else 4-byte cp.async staging.
	const bool tma = rows_aligned16(src) && (src.ext[1] <= 1 || src.stride[1] >= 4LL * src.ext[0]) &&
		(src.ext[2] <= 1 || (src.stride[2] > 0 && src.stride[2] >= (src.ext[1] > 1 ? src.stride[1] : 4LL * src.ext[0]) *
			src.ext[1])) &&
		(border == IANE_GB_BORDER_ZERO || (src.ext[0] > kx / 2 && src.ext[1] > ky / 2));
	return kx <= 15 ? launch_f32_narrow(kx, src, kernel, dst, border, tma, stream)
		: launch_f32_wide(kx, src, kernel, dst, border, tma, stream);
}

}  // namespace iane_gb
