// iane_gb_convolve's FP32 fast path: eligibility, staging choice and dispatch by kernel width.
#include "conv_f32.cuh"
#include "kernels.h"

namespace iane_gb {

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
	// large 2-D f32 images with kernels up to 7 x 7: the row-strip kernel (same sums)
	if (!tex) {
		const int rows = launch_direct_rows(src, kernel, dst, border, stream);
		if (rows != IANE_GB_UNSUPPORTED) return rows;
	}
	// Small single-plane jobs (too few 64x64 tiles for every SM, and under 5e7 tap-products):
	// the one-warp blocks of 32x32 tiles are latency-bound there, and the generic kernel (one
	// output per thread, 256-thread blocks, FP32 sums) with many times the warps per SM is
	// faster -- measured on GB300: 512^2 7x7 16.5 -> 9.9 us, 256^2 15x15 27.8 -> 8.9 us,
	// 384x640 11x11 23.5 -> 14.4 us; 1024^2 9x9 (8.5e7) and 512^2 31x31 stay tiled.
	const long long big_tiles = static_cast<long long>((src.ext[0] + 63) / 64) * ((src.ext[1] + 63) / 64) * src.ext[2];
	const double work = static_cast<double>(element_count(src)) * kx * ky;
	if (kz == 1 && big_tiles < 2LL * device_sm_count() && work < 5e7) {
		return IANE_GB_UNSUPPORTED;
	}
	// Shared memory holds one or two kernel planes' taps (ky x 32 floats at most) next to the
	// halo tiles; the planes stream through it, so kz has no limit here.
	(void)kz;
	// TMA staging when the source is a TMA-addressable f32 or 8/16-bit integer view (16-byte
	// aligned rows and planes that do not overlap) and, for clamp and mirror, wider than the
	// kernel radius on x and y (the edge fix-up takes its sources from inside the tile); else
	// element-by-element staging.
	const bool narrow = src.dtype == IANE_GB_U8 || src.dtype == IANE_GB_I8 || src.dtype == IANE_GB_U16 ||
		src.dtype == IANE_GB_I16;
	const long long row_bytes = static_cast<long long>(dtype_size(src.dtype)) * src.ext[0];
	const bool tma = !tex && (src.dtype == IANE_GB_F32 || narrow) && rows_aligned16(src) &&
		(src.ext[1] <= 1 || src.stride[1] >= row_bytes) &&
		(src.ext[2] <= 1 || (src.stride[2] > 0 && src.stride[2] >= (src.ext[1] > 1 ? src.stride[1] : row_bytes) *
			src.ext[1])) &&
		(border == IANE_GB_BORDER_ZERO || (src.ext[0] > kx / 2 && src.ext[1] > ky / 2));
	const int stage = !tma ? kTileCopy : (narrow ? kTileTmaNarrow : kTileTma);
	static const LaunchF32Widths by_width[8] = {launch_f32_k1_3, launch_f32_k5_7, launch_f32_k9_11, launch_f32_k13_15,
		launch_f32_k17_19, launch_f32_k21_23, launch_f32_k25_27, launch_f32_k29_31};
	if (kx < 1 || kx > 31) {
		return IANE_GB_UNSUPPORTED;
	}
	return by_width[(kx - 1) / 4](kx, src, kernel, dst, border, stage, tex, stream);
}

}  // namespace iane_gb
