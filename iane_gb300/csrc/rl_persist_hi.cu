// Persistent Richardson-Lucy kernel instantiations for kernel widths 17, 19, 21, 23, 25, 27, 29, 31.
#include "rl_persist.cuh"

namespace iane_gb {

int launch_rl_persist_hi(int kx, const RlPersistArgs& p, cudaStream_t stream)
{
	switch (kx) {
	case 17: return launch_rl_persist_kx<17>(p, stream);
	case 19: return launch_rl_persist_kx<19>(p, stream);
	case 21: return launch_rl_persist_kx<21>(p, stream);
	case 23: return launch_rl_persist_kx<23>(p, stream);
	case 25: return launch_rl_persist_kx<25>(p, stream);
	case 27: return launch_rl_persist_kx<27>(p, stream);
	case 29: return launch_rl_persist_kx<29>(p, stream);
	case 31: return launch_rl_persist_kx<31>(p, stream);
	default: return fail(IANE_GB_UNSUPPORTED, "Richardson-Lucy: unsupported PSF width");
	}
}

}  // namespace iane_gb
