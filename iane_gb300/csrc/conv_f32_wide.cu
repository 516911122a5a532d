// iane_gb_convolve's FP32 fast path: instantiations for kernel widths 17..31.
#include "conv_f32.cuh"

namespace iane_gb {

int launch_f32_wide(int kx, const DevView& src, const DevView& kernel, const DevView& dst, int border, bool tma, const TexSource* tex,
	cudaStream_t stream)
{
	switch (kx) {
	case 17: return launch_f32_kx<17>(src, kernel, dst, border, tma, tex, stream);
	case 19: return launch_f32_kx<19>(src, kernel, dst, border, tma, tex, stream);
	case 21: return launch_f32_kx<21>(src, kernel, dst, border, tma, tex, stream);
	case 23: return launch_f32_kx<23>(src, kernel, dst, border, tma, tex, stream);
	case 25: return launch_f32_kx<25>(src, kernel, dst, border, tma, tex, stream);
	case 27: return launch_f32_kx<27>(src, kernel, dst, border, tma, tex, stream);
	case 29: return launch_f32_kx<29>(src, kernel, dst, border, tma, tex, stream);
	case 31: return launch_f32_kx<31>(src, kernel, dst, border, tma, tex, stream);
	default: return IANE_GB_UNSUPPORTED;
	}
}

}  // namespace iane_gb
