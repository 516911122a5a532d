// Richardson-Lucy pass instantiations for kernel widths 17, 19, 21, 23, 25, 27, 29, 31.
#include "rl.cuh"

namespace iane_gb {

int launch_rl_pass_a_hi(int kx, bool small, const CUtensorMap& map, const TileArgs& a, const EpiRatio& e,
	cudaStream_t stream)
{
	switch (kx) {
	case 17: return small ? launch_tile<17, 1, 1, true>(map, a, e, stream) : launch_tile<17, 2, 2, true>(map, a, e, stream);
	case 19: return small ? launch_tile<19, 1, 1, true>(map, a, e, stream) : launch_tile<19, 2, 2, true>(map, a, e, stream);
	case 21: return small ? launch_tile<21, 1, 1, true>(map, a, e, stream) : launch_tile<21, 2, 2, true>(map, a, e, stream);
	case 23: return small ? launch_tile<23, 1, 1, true>(map, a, e, stream) : launch_tile<23, 2, 2, true>(map, a, e, stream);
	case 25: return small ? launch_tile<25, 1, 1, true>(map, a, e, stream) : launch_tile<25, 2, 2, true>(map, a, e, stream);
	case 27: return small ? launch_tile<27, 1, 1, true>(map, a, e, stream) : launch_tile<27, 2, 2, true>(map, a, e, stream);
	case 29: return small ? launch_tile<29, 1, 1, true>(map, a, e, stream) : launch_tile<29, 2, 2, true>(map, a, e, stream);
	case 31: return small ? launch_tile<31, 1, 1, true>(map, a, e, stream) : launch_tile<31, 2, 2, true>(map, a, e, stream);
	default: return fail(IANE_GB_UNSUPPORTED, "Richardson-Lucy: unsupported PSF width");
	}
}

int launch_rl_pass_b_hi(int kx, bool small, const CUtensorMap& map, const TileArgs& a, const EpiUpdate& e,
	cudaStream_t stream)
{
	switch (kx) {
	case 17: return small ? launch_tile<17, 1, 1, true>(map, a, e, stream) : launch_tile<17, 2, 2, true>(map, a, e, stream);
	case 19: return small ? launch_tile<19, 1, 1, true>(map, a, e, stream) : launch_tile<19, 2, 2, true>(map, a, e, stream);
	case 21: return small ? launch_tile<21, 1, 1, true>(map, a, e, stream) : launch_tile<21, 2, 2, true>(map, a, e, stream);
	case 23: return small ? launch_tile<23, 1, 1, true>(map, a, e, stream) : launch_tile<23, 2, 2, true>(map, a, e, stream);
	case 25: return small ? launch_tile<25, 1, 1, true>(map, a, e, stream) : launch_tile<25, 2, 2, true>(map, a, e, stream);
	case 27: return small ? launch_tile<27, 1, 1, true>(map, a, e, stream) : launch_tile<27, 2, 2, true>(map, a, e, stream);
	case 29: return small ? launch_tile<29, 1, 1, true>(map, a, e, stream) : launch_tile<29, 2, 2, true>(map, a, e, stream);
	case 31: return small ? launch_tile<31, 1, 1, true>(map, a, e, stream) : launch_tile<31, 2, 2, true>(map, a, e, stream);
	default: return fail(IANE_GB_UNSUPPORTED, "Richardson-Lucy: unsupported PSF width");
	}
}

}  // namespace iane_gb
