// Persistent Richardson-Lucy kernel instantiations for kernel widths 1, 3, 5, 7, 9, 11, 13, 15.
#include "rl_persist.cuh"

namespace iane_gb {

int launch_rl_persist_lo(int kx, const RlPersistArgs& p, cudaStream_t stream)
{
	switch (kx) {
	case 1: return launch_rl_persist_kx<1>(p, stream);
	case 3: return launch_rl_persist_kx<3>(p, stream);
	case 5: return launch_rl_persist_kx<5>(p, stream);
	case 7: return launch_rl_persist_kx<7>(p, stream);
	case 9: return launch_rl_persist_kx<9>(p, stream);
	case 11: return launch_rl_persist_kx<11>(p, stream);
	case 13: return launch_rl_persist_kx<13>(p, stream);
	case 15: return launch_rl_persist_kx<15>(p, stream);
	default: return fail(IANE_GB_UNSUPPORTED, "Richardson-Lucy: unsupported PSF width");
	}
}

}  // namespace iane_gb
