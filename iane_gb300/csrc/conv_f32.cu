// iane_gb_convolve's FP32 fast path: the register-tiled kernel of conv_tile.cuh with the
// border rule applied by 4-byte cp.async staging (any border, any f32 strides).
#include "conv_tile.cuh"
#include "kernels.h"

namespace iane_gb {
namespace {

template<int KX>
int launch_for_kx(const DevView& src, const DevView& kernel, const DevView& dst, int border, cudaStream_t stream)
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
	CUtensorMap unused{};
	// Large images use 64x64 tiles; small ones 32x32 so that the grid still fills the GPU.
	const long long big_tiles = static_cast<long long>((a.nx + 63) / 64) * ((a.ny + 63) / 64) * a.nz;
	if (big_tiles >= 2LL * device_sm_count()) {
		return launch_tile<KX, 2, 2, false>(unused, a, epi, stream);
	}
	return launch_tile<KX, 1, 1, false>(unused, a, epi, stream);
}

}  // namespace

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
	// The kernel planes live in shared memory next to two halo tiles.
	if (static_cast<long long>(kz) * ky * ((kx + 3) & ~3) * 4 > 96 * 1024) {
		return IANE_GB_UNSUPPORTED;
	}
	switch (kx) {
	case 1: return launch_for_kx<1>(src, kernel, dst, border, stream);
	case 3: return launch_for_kx<3>(src, kernel, dst, border, stream);
	case 5: return launch_for_kx<5>(src, kernel, dst, border, stream);
	case 7: return launch_for_kx<7>(src, kernel, dst, border, stream);
	case 9: return launch_for_kx<9>(src, kernel, dst, border, stream);
	case 11: return launch_for_kx<11>(src, kernel, dst, border, stream);
	case 13: return launch_for_kx<13>(src, kernel, dst, border, stream);
	case 15: return launch_for_kx<15>(src, kernel, dst, border, stream);
	case 17: return launch_for_kx<17>(src, kernel, dst, border, stream);
	case 19: return launch_for_kx<19>(src, kernel, dst, border, stream);
	case 21: return launch_for_kx<21>(src, kernel, dst, border, stream);
	case 23: return launch_for_kx<23>(src, kernel, dst, border, stream);
	case 25: return launch_for_kx<25>(src, kernel, dst, border, stream);
	case 27: return launch_for_kx<27>(src, kernel, dst, border, stream);
	case 29: return launch_for_kx<29>(src, kernel, dst, border, stream);
	case 31: return launch_for_kx<31>(src, kernel, dst, border, stream);
	default: return IANE_GB_UNSUPPORTED;
	}
}

}  // namespace iane_gb
