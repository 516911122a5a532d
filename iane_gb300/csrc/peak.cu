// FP32 throughput probe: the denominator of the FP32-pipe roofline, measured on the device
// that runs the convolutions instead of derived from a clock and a lane count.
//
// Every thread runs CHAINS independent fused multiply-add chains (enough to cover the FMA
// latency at full occupancy), unrolled 16 deep per loop trip, with a multiplier just below
// one and a small addend so the values stay finite. The paired form issues the packed
// fma.rn.f32x2 instruction of sm_100-class GPUs (two FMAs per lane per instruction); the
// scalar form issues one FFMA per FMA. The result is the larger rate seen over a few
// launches; it is a throughput ceiling for FP32 FMA work, like a STREAM copy is for HBM.
#include "common.cuh"

#include <cuda_runtime.h>

namespace iane_gb {
namespace {

constexpr int kChains = 8;
constexpr int kUnroll = 16;

__global__ void __launch_bounds__(256) fp32_peak_scalar_kernel(float* sink, int trips, float a, float b)
{
	float acc[kChains];
#pragma unroll
	for (int i = 0; i < kChains; ++i) acc[i] = static_cast<float>(threadIdx.x + i) * 1e-3f;
	for (int t = 0; t < trips; ++t) {
#pragma unroll
		for (int u = 0; u < kUnroll; ++u) {
#pragma unroll
			for (int i = 0; i < kChains; ++i) acc[i] = fmaf(acc[i], a, b);
		}
	}
	float s = 0.0f;
#pragma unroll
	for (int i = 0; i < kChains; ++i) s += acc[i];
	if (s == -1.0f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;  // never true; keeps the chains live
}

__global__ void __launch_bounds__(256) fp32_peak_paired_kernel(float* sink, int trips, float a, float b)
{
	unsigned long long acc[kChains];
	const float2 av = make_float2(a, a), bv = make_float2(b, b);
	const unsigned long long a2 = *reinterpret_cast<const unsigned long long*>(&av);
	const unsigned long long b2 = *reinterpret_cast<const unsigned long long*>(&bv);
#pragma unroll
	for (int i = 0; i < kChains; ++i) {
		const float2 v = make_float2(static_cast<float>(threadIdx.x + i) * 1e-3f, static_cast<float>(i));
		acc[i] = *reinterpret_cast<const unsigned long long*>(&v);
	}
	for (int t = 0; t < trips; ++t) {
#pragma unroll
		for (int u = 0; u < kUnroll; ++u) {
#pragma unroll
			for (int i = 0; i < kChains; ++i) {
				asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(acc[i]) : "l"(a2), "l"(b2));
			}
		}
	}
	float s = 0.0f;
#pragma unroll
	for (int i = 0; i < kChains; ++i) {
		const float2 v = *reinterpret_cast<const float2*>(&acc[i]);
		s += v.x + v.y;
	}
	if (s == -1.0f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace iane_gb

using namespace iane_gb;

extern "C" int iane_gb_fp32_peak_probe(int paired, double* tflops, void* stream)
{
	if (!tflops || (paired != 0 && paired != 1)) {
		return fail(IANE_GB_INVALID_ARGUMENT, "fp32_peak_probe: null result or paired not 0/1");
	}
	*tflops = 0.0;
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	const int sms = device_sm_count();
	const int blocks = sms * 8;  // 8 blocks of 256 threads: 64 warps per SM
	const int threads = 256;
	const int trips = 4096;
	float* sink = nullptr;  // never written (the guarded store is unreachable); a null base is fine
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	IANE_GB_CUDA(cudaEventCreate(&e0), "fp32_peak_probe: event");
	if (cudaEventCreate(&e1) != cudaSuccess) {
		cudaEventDestroy(e0);
		return fail(IANE_GB_CUDA_ERROR, "fp32_peak_probe: event");
	}
	double best = 0.0;
	int status = IANE_GB_OK;
	for (int rep = 0; rep < 4 && status == IANE_GB_OK; ++rep) {
		cudaEventRecord(e0, st);
		if (paired) {
			fp32_peak_paired_kernel<<<blocks, threads, 0, st>>>(sink, trips, 0.9999999f, 1e-7f);
		} else {
			fp32_peak_scalar_kernel<<<blocks, threads, 0, st>>>(sink, trips, 0.9999999f, 1e-7f);
		}
		cudaEventRecord(e1, st);
		if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
			status = fail(IANE_GB_CUDA_ERROR, "fp32_peak_probe: launch");
			break;
		}
		float ms = 0.0f;
		cudaEventElapsedTime(&ms, e0, e1);
		const double fmas = static_cast<double>(blocks) * threads * trips * kUnroll * kChains * (paired ? 2 : 1);
		const double rate = 2.0 * fmas / (ms * 1e-3) / 1e12;
		if (rep > 0 && rate > best) best = rate;  // the first launch is a warm-up
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	*tflops = best;
	return status;
}
