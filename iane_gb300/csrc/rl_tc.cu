// Launchers of the BF16 tensor-core Richardson-Lucy passes.
#include "rl_tcz.cuh"

namespace iane_gb {
namespace {

template<class Epi>
int launch(const CUtensorMap& map, const TcArgs& a, const Epi& e, cudaStream_t stream)
{
	auto kernel = tc_conv_kernel<Epi>;
	IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, a.smem_bytes),
		"tensor-core convolution: set shared memory size");
	const dim3 grid((a.nx + kTcN - 1) / kTcN, (a.ny + kTcM - 1) / kTcM, a.nz);
	kernel<<<grid, 128, a.smem_bytes, stream>>>(map, a, e);
	IANE_GB_CUDA(cudaGetLastError(), "tensor-core convolution: launch");
	return IANE_GB_OK;
}

template<class Epi>
int launch_z(const CUtensorMap& map, const TcArgs& a, const Epi& e, cudaStream_t stream)
{
	auto kernel = tcz_conv_kernel<Epi>;
	IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, a.smem_bytes),
		"tensor-core convolution: set shared memory size");
	const dim3 grid((a.nx + 15) / 16, (a.ny + kTcM - 1) / kTcM, (a.nz + kTczZ - 1) / kTczZ);
	kernel<<<grid, kTczThreads, a.smem_bytes, stream>>>(map, a, e);
	IANE_GB_CUDA(cudaGetLastError(), "tensor-core convolution: launch");
	return IANE_GB_OK;
}

}  // namespace

bool tcz_supported(int kx, int ky, int kz)
{
	return kx <= 17 && ky <= 17 && kz <= 31 && tcz_smem_bytes(ky, kz) <= 227 * 1024;
}

int launch_tcz_pass_a(const CUtensorMap& map, const TcArgs& a, const EpiRatioTc& e, cudaStream_t stream)
{
	return launch_z(map, a, e, stream);
}

int launch_tcz_pass_b(const CUtensorMap& map, const TcArgs& a, const EpiUpdateTc& e, cudaStream_t stream)
{
	return launch_z(map, a, e, stream);
}

int launch_tc_pass_a(const CUtensorMap& map, const TcArgs& a, const EpiRatioTc& e, cudaStream_t stream)
{
	return launch(map, a, e, stream);
}

int launch_tc_pass_b(const CUtensorMap& map, const TcArgs& a, const EpiUpdateTc& e, cudaStream_t stream)
{
	return launch(map, a, e, stream);
}

}  // namespace iane_gb
