// Wiener deconvolution as a prepared operation: the reference's examples/wiener/main.cu:44-83
// (2-D there; rank 1 to 3 here).
//
// prepare: the PSF is placed in an image-sized real buffer with its centre (extent / 2 per
// axis) at the origin, wrapped periodically (main.cu:112-120), transformed (FP32 real-to-
// complex; the reference's complex transform of a real image gives the same spectrum), and
// the filter G = conj(H) / (|H|^2 + noise) is formed once, in FP64 from the FP32 spectrum and
// rounded to FP32 (the reference forms the same quotient per run, main.cu:21-31).
// run: observed -> real buffer (any element type, any strides), R2C, multiply by G, C2R, and
// the result times 1 / N encoded into the destination: to_gray8 for u8
// (examples/common/deconvolution.hpp:43-55), the plain value for f32. The transforms use
// cuFFT with their work area in the caller's scratch, as the reference's FFT plans do
// (include/iane/algorithms/fft/fft.hpp:160-172); the pad, filter, multiply and encode
// kernels are this library's.
#include "common.cuh"
#include "kernels.h"

#include <cufft.h>

#include <cmath>
#include <string>

struct iane_gb_wiener_plan {
	int rank;
	int ext[3];        // image extents, axis 0 fastest (unused axes 1)
	long long n;       // real cells
	long long nc;      // complex cells of the half spectrum ((ext0 / 2 + 1) * ext1 * ext2)
	cufftHandle r2c;
	cufftHandle c2r;
	size_t work_bytes; // cuFFT work area, the larger of the two plans'
	float2* filter;    // G, nc entries
	int device;
};

namespace iane_gb {
namespace {

constexpr size_t kAlign = 256;
size_t align_up(size_t v) { return (v + kAlign - 1) & ~(kAlign - 1); }

int grid_for(long long n)
{
	const long long b = (n + 255) / 256;
	const long long cap = 16LL * device_sm_count();
	return static_cast<int>(b < 1 ? 1 : (b > cap ? cap : b));
}

// Cell p of the padded PSF: tap x with x - e/2 = p (mod n) per axis, if any.
__device__ __forceinline__ bool psf_source(int p, int n, int e, int& x)
{
	if (p < e - e / 2) {
		x = p + e / 2;
		return true;
	}
	if (p >= n - e / 2) {
		x = p - n + e / 2;
		return true;
	}
	return false;
}

__global__ void wiener_pad_psf(DevView psf, int n0, int n1, int n2, float* out)
{
	const long long total = static_cast<long long>(n0) * n1 * n2;
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int p0 = static_cast<int>(i % n0);
		const int p1 = static_cast<int>((i / n0) % n1);
		const int p2 = static_cast<int>(i / (static_cast<long long>(n0) * n1));
		int x = 0, y = 0, z = 0;
		float v = 0.0f;
		if (psf_source(p0, n0, psf.ext[0], x) && psf_source(p1, n1, psf.ext[1], y) && psf_source(p2, n2, psf.ext[2], z)) {
			v = *element_ptr<float>(psf, x, y, z);
		}
		out[i] = v;
	}
}

__global__ void wiener_make_filter(float2* h, long long nc, double noise)
{
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < nc;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const double re = h[i].x, im = h[i].y;
		const double den = re * re + im * im + noise;
		h[i] = make_float2(static_cast<float>(re / den), static_cast<float>(-im / den));
	}
}

__global__ void wiener_load(DevView src, float* out)
{
	const long long total = element_count(src);
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int x = static_cast<int>(i % src.ext[0]);
		const int y = static_cast<int>((i / src.ext[0]) % src.ext[1]);
		const int z = static_cast<int>(i / (static_cast<long long>(src.ext[0]) * src.ext[1]));
		out[i] = load_as_float(src.ptr + x * src.stride[0] + y * src.stride[1] + z * src.stride[2], src.dtype);
	}
}

__global__ void wiener_apply(float2* spec, const float2* __restrict__ g, long long nc)
{
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < nc;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const float2 o = spec[i], w = g[i];
		spec[i] = make_float2(o.x * w.x - o.y * w.y, o.x * w.y + o.y * w.x);
	}
}

__global__ void wiener_store(const float* __restrict__ real, float scale, DevView dst)
{
	const long long total = element_count(dst);
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int x = static_cast<int>(i % dst.ext[0]);
		const int y = static_cast<int>((i / dst.ext[0]) % dst.ext[1]);
		const int z = static_cast<int>(i / (static_cast<long long>(dst.ext[0]) * dst.ext[1]));
		store_converted_f32(dst.ptr + x * dst.stride[0] + y * dst.stride[1] + z * dst.stride[2], dst.dtype,
			real[i] * scale);
	}
}

#define IANE_GB_CUFFT_OK(call, what)                                                                        \
	do {                                                                                                    \
		const cufftResult r_ = (call);                                                                      \
		if (r_ != CUFFT_SUCCESS) {                                                                          \
			return fail(IANE_GB_CUDA_ERROR, std::string(what) + ": cuFFT error " + std::to_string(static_cast<int>(r_))); \
		}                                                                                                   \
	} while (0)

int make_plans(iane_gb_wiener_plan* p)
{
	int dims[3];
	for (int i = 0; i < p->rank; ++i) dims[i] = p->ext[p->rank - 1 - i]; // slowest first
	size_t w1 = 0, w2 = 0;
	IANE_GB_CUFFT_OK(cufftCreate(&p->r2c), "wiener: FFT plan");
	IANE_GB_CUFFT_OK(cufftCreate(&p->c2r), "wiener: FFT plan");
	IANE_GB_CUFFT_OK(cufftSetAutoAllocation(p->r2c, 0), "wiener: FFT plan");
	IANE_GB_CUFFT_OK(cufftSetAutoAllocation(p->c2r, 0), "wiener: FFT plan");
	IANE_GB_CUFFT_OK(cufftMakePlanMany(p->r2c, p->rank, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_R2C, 1, &w1),
		"wiener: FFT plan");
	IANE_GB_CUFFT_OK(cufftMakePlanMany(p->c2r, p->rank, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_C2R, 1, &w2),
		"wiener: FFT plan");
	p->work_bytes = w1 > w2 ? w1 : w2;
	return IANE_GB_OK;
}

void destroy_plan(iane_gb_wiener_plan* p)
{
	if (!p) return;
	if (p->r2c) cufftDestroy(p->r2c);
	if (p->c2r) cufftDestroy(p->c2r);
	if (p->filter) cudaFree(p->filter);
	delete p;
}

size_t scratch_of(const iane_gb_wiener_plan* p)
{
	return align_up(static_cast<size_t>(p->n) * sizeof(float)) + align_up(static_cast<size_t>(p->nc) * sizeof(float2)) +
		align_up(p->work_bytes);
}

}  // namespace
}  // namespace iane_gb

using namespace iane_gb;

extern "C" {

int iane_gb_wiener_prepare(const iane_gb_view* psf, int rank, const int32_t* extent, float noise, void* stream,
	iane_gb_wiener_plan** plan)
{
	if (!plan || !extent) {
		return fail(IANE_GB_INVALID_ARGUMENT, "wiener prepare: null argument");
	}
	*plan = nullptr;
	// examples/wiener/main.cu:93-96, 101-104
	if (!std::isfinite(noise) || !(noise > 0.0f)) {
		return fail(IANE_GB_INVALID_ARGUMENT, "Noise must be finite and positive");
	}
	DevView k{};
	int status = normalise_view(psf, "wiener psf", &k);
	if (status) return status;
	if (k.dtype != IANE_GB_F32) {
		return fail(IANE_GB_UNSUPPORTED, "wiener prepare: the PSF is f32");
	}
	if (rank < 1 || rank > 3 || k.rank != rank) {
		return fail(IANE_GB_INVALID_ARGUMENT, "wiener prepare: the PSF needs the image's rank (1..3)");
	}
	auto* p = new iane_gb_wiener_plan{};
	p->rank = rank;
	p->n = 1;
	for (int i = 0; i < 3; ++i) {
		p->ext[i] = i < rank ? extent[i] : 1;
		if (p->ext[i] <= 0) {
			delete p;
			return fail(IANE_GB_INVALID_ARGUMENT, "wiener prepare: image extents must be positive");
		}
		if (k.ext[i] > p->ext[i] || k.ext[i] <= 0) {
			delete p;
			return fail(IANE_GB_INVALID_ARGUMENT, "PSF must fit inside the input image");
		}
		p->n *= p->ext[i];
	}
	p->nc = p->n / p->ext[0] * (p->ext[0] / 2 + 1);
	cudaGetDevice(&p->device);
	status = make_plans(p);
	if (status) {
		destroy_plan(p);
		return status;
	}
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p->filter), static_cast<size_t>(p->nc) * sizeof(float2));
	if (e != cudaSuccess) {
		destroy_plan(p);
		return cuda_fail(e, "wiener prepare: filter");
	}
	// the PSF's spectrum, through a temporary real buffer and work area
	char* tmp = nullptr;
	const size_t real_bytes = align_up(static_cast<size_t>(p->n) * sizeof(float));
	const cudaError_t e2 = cudaMallocAsync(reinterpret_cast<void**>(&tmp), real_bytes + align_up(p->work_bytes), st);
	if (e2 != cudaSuccess) {
		destroy_plan(p);
		return cuda_fail(e2, "wiener prepare: buffers");
	}
	float* real = reinterpret_cast<float*>(tmp);
	wiener_pad_psf<<<grid_for(p->n), 256, 0, st>>>(k, p->ext[0], p->ext[1], p->ext[2], real);
	status = IANE_GB_OK;
	if (cufftSetStream(p->r2c, st) != CUFFT_SUCCESS || cufftSetWorkArea(p->r2c, tmp + real_bytes) != CUFFT_SUCCESS ||
	    cufftExecR2C(p->r2c, real, reinterpret_cast<cufftComplex*>(p->filter)) != CUFFT_SUCCESS) {
		status = fail(IANE_GB_CUDA_ERROR, "wiener prepare: PSF transform");
	}
	if (!status) {
		wiener_make_filter<<<grid_for(p->nc), 256, 0, st>>>(p->filter, p->nc, static_cast<double>(noise));
		const cudaError_t e3 = cudaGetLastError();
		if (e3 != cudaSuccess) status = cuda_fail(e3, "wiener prepare: filter kernel");
	}
	cudaFreeAsync(tmp, st);
	if (!status) {
		const cudaError_t e4 = cudaStreamSynchronize(st);
		if (e4 != cudaSuccess) status = cuda_fail(e4, "wiener prepare");
	}
	if (status) {
		destroy_plan(p);
		return status;
	}
	*plan = p;
	return IANE_GB_OK;
}

size_t iane_gb_wiener_scratch_bytes(const iane_gb_wiener_plan* plan)
{
	return plan ? scratch_of(plan) : 0;
}

int iane_gb_wiener_run(iane_gb_wiener_plan* plan, const iane_gb_view* observed, const iane_gb_view* restored,
	void* scratch, size_t scratch_bytes, void* stream)
{
	if (!plan) {
		return fail(IANE_GB_INVALID_ARGUMENT, "wiener run: null plan");
	}
	DevView s{}, d{};
	int status = normalise_view(observed, "wiener observed", &s);
	if (status) return status;
	status = normalise_view(restored, "wiener restored", &d);
	if (status) return status;
	if (s.rank != plan->rank || d.rank != plan->rank) {
		return fail(IANE_GB_INVALID_ARGUMENT, "wiener run: views need the prepared rank");
	}
	for (int i = 0; i < 3; ++i) {
		if (s.ext[i] != plan->ext[i] || d.ext[i] != plan->ext[i]) {
			return fail(IANE_GB_INVALID_ARGUMENT, "wiener run: views must match the prepared shape");
		}
	}
	if (s.dtype == IANE_GB_F64 || s.dtype == IANE_GB_RGB8 || d.dtype == IANE_GB_BF16 || d.dtype == IANE_GB_RGB8) {
		return fail(IANE_GB_UNSUPPORTED, "wiener run: observed u8/i8/u16/i16/i32/u32/bf16/f32, restored scalar");
	}
	if (!scratch || scratch_bytes < scratch_of(plan)) {
		return fail(IANE_GB_LENGTH_ERROR, "wiener run: scratch smaller than iane_gb_wiener_scratch_bytes");
	}
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	char* base = static_cast<char*>(scratch);
	float* real = reinterpret_cast<float*>(base);
	base += align_up(static_cast<size_t>(plan->n) * sizeof(float));
	cufftComplex* spec = reinterpret_cast<cufftComplex*>(base);
	base += align_up(static_cast<size_t>(plan->nc) * sizeof(float2));
	void* work = base;
	wiener_load<<<grid_for(plan->n), 256, 0, st>>>(s, real);
	if (cufftSetStream(plan->r2c, st) != CUFFT_SUCCESS || cufftSetStream(plan->c2r, st) != CUFFT_SUCCESS ||
	    cufftSetWorkArea(plan->r2c, work) != CUFFT_SUCCESS || cufftSetWorkArea(plan->c2r, work) != CUFFT_SUCCESS ||
	    cufftExecR2C(plan->r2c, real, spec) != CUFFT_SUCCESS) {
		return fail(IANE_GB_CUDA_ERROR, "wiener run: forward transform");
	}
	wiener_apply<<<grid_for(plan->nc), 256, 0, st>>>(reinterpret_cast<float2*>(spec), plan->filter, plan->nc);
	if (cufftExecC2R(plan->c2r, spec, real) != CUFFT_SUCCESS) {
		return fail(IANE_GB_CUDA_ERROR, "wiener run: inverse transform");
	}
	// main.cu:74: scale = 1 / (w h) in double, rounded to float
	const float scale = static_cast<float>(1.0 / static_cast<double>(plan->n));
	wiener_store<<<grid_for(plan->n), 256, 0, st>>>(real, scale, d);
	IANE_GB_CUDA(cudaGetLastError(), "wiener run: kernels");
	return IANE_GB_OK;
}

int iane_gb_wiener_destroy(iane_gb_wiener_plan* plan)
{
	destroy_plan(plan);
	return IANE_GB_OK;
}

}  // extern "C"
