// Richardson-Lucy pass instantiations for kernel widths 1, 3, 5, 7, 9, 11, 13, 15.
#include "rl.cuh"

namespace iane_gb {

int launch_rl_pass_a_lo(int kx, bool small, const CUtensorMap& map, const TileArgs& a, const EpiRatio& e,
	cudaStream_t stream)
{
	switch (kx) {
	case 1: return small ? launch_tile<1, 1, 1, true>(map, a, e, stream) : launch_tile<1, 2, 2, true>(map, a, e, stream);
	case 3: return small ? launch_tile<3, 1, 1, true>(map, a, e, stream) : launch_tile<3, 2, 2, true>(map, a, e, stream);
	case 5: return small ? launch_tile<5, 1, 1, true>(map, a, e, stream) : launch_tile<5, 2, 2, true>(map, a, e, stream);
	case 7: return small ? launch_tile<7, 1, 1, true>(map, a, e, stream) : launch_tile<7, 2, 2, true>(map, a, e, stream);
	case 9: return small ? launch_tile<9, 1, 1, true>(map, a, e, stream) : launch_tile<9, 2, 2, true>(map, a, e, stream);
	case 11: return small ? launch_tile<11, 1, 1, true>(map, a, e, stream) : launch_tile<11, 2, 2, true>(map, a, e, stream);
	case 13: return small ? launch_tile<13, 1, 1, true>(map, a, e, stream) : launch_tile<13, 2, 2, true>(map, a, e, stream);
	case 15: return small ? launch_tile<15, 1, 1, true>(map, a, e, stream) : launch_tile<15, 2, 2, true>(map, a, e, stream);
	default: return fail(IANE_GB_UNSUPPORTED, "Richardson-Lucy: unsupported PSF width");
	}
}

int launch_rl_pass_b_lo(int kx, bool small, const CUtensorMap& map, const TileArgs& a, const EpiUpdate& e,
	cudaStream_t stream)
{
	switch (kx) {
	case 1: return small ? launch_tile<1, 1, 1, true>(map, a, e, stream) : launch_tile<1, 2, 2, true>(map, a, e, stream);
	case 3: return small ? launch_tile<3, 1, 1, true>(map, a, e, stream) : launch_tile<3, 2, 2, true>(map, a, e, stream);
	case 5: return small ? launch_tile<5, 1, 1, true>(map, a, e, stream) : launch_tile<5, 2, 2, true>(map, a, e, stream);
	case 7: return small ? launch_tile<7, 1, 1, true>(map, a, e, stream) : launch_tile<7, 2, 2, true>(map, a, e, stream);
	case 9: return small ? launch_tile<9, 1, 1, true>(map, a, e, stream) : launch_tile<9, 2, 2, true>(map, a, e, stream);
	case 11: return small ? launch_tile<11, 1, 1, true>(map, a, e, stream) : launch_tile<11, 2, 2, true>(map, a, e, stream);
	case 13: return small ? launch_tile<13, 1, 1, true>(map, a, e, stream) : launch_tile<13, 2, 2, true>(map, a, e, stream);
	case 15: return small ? launch_tile<15, 1, 1, true>(map, a, e, stream) : launch_tile<15, 2, 2, true>(map, a, e, stream);
	default: return fail(IANE_GB_UNSUPPORTED, "Richardson-Lucy: unsupported PSF width");
	}
}

}  // namespace iane_gb
