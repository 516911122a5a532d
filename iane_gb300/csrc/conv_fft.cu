// Spectral (FFT) convolution for large kernels, behind iane_gb_convolve.
//
// out[p] = sum_q K[q] in[p + c - q] (c = size / 2 per axis, the border rule applied to in)
// is computed as a circular convolution of length L >= n + k - 1 per axis:
//   P[j] = in[j - c] for j in [0, n + k - 1) (the border rule gives the halo), 0 beyond;
//   Kp[q] = K[q] at the origin, 0 beyond;
//   R = IFFT(FFT(P) FFT(Kp)) / L_total;   out[p] = R[p + k - 1]
// (no wrap-around: every index p + k - 1 - q lies in [0, L)). The transforms are cuFFT
// real-to-complex / complex-to-real in FP64, so the result carries about 1e-13 of relative
// error before the final cast -- inside the per-element bar of the FP32 direct path -- while
// the work grows as L log L instead of n x taps. L per axis is the next size with prime
// factors 2, 3, 5, 7. Plans are cached per (L, rank, device); buffers come from the stream-
// ordered allocator.
#include "common.cuh"
#include "kernels.h"

#include <cufft.h>

#include <cmath>
#include <map>
#include <mutex>
#include <tuple>

namespace iane_gb {
namespace {

int good_size(int n)
{
	for (int m = n;; ++m) {
		int r = m;
		for (int p : {2, 3, 5, 7}) {
			while (r % p == 0) r /= p;
		}
		if (r == 1) return m;
	}
}

struct FftPlans {
	cufftHandle fwd = 0, inv = 0;
};

std::mutex& plan_mutex()
{
	static std::mutex m;
	return m;
}

std::map<std::tuple<int, int, int, int, int>, FftPlans>& plan_cache()
{
	static std::map<std::tuple<int, int, int, int, int>, FftPlans> cache;
	return cache;
}

template<class TS>
__global__ void pad_source_kernel(DevView src, int border, int c0, int c1, int c2, int l0, int l1, int l2, int m0, int m1,
	int m2, double* out)
{
	// m = n + k - 1: the padded extent that carries data; indices beyond it are zeros
	const long long total = static_cast<long long>(l0) * l1 * l2;
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int j0 = static_cast<int>(i % l0);
		const int j1 = static_cast<int>((i / l0) % l1);
		const int j2 = static_cast<int>(i / (static_cast<long long>(l0) * l1));
		double v = 0.0;
		if (j0 < m0 && j1 < m1 && j2 < m2) {
			int x = 0, y = 0, z = 0;
			if (map_coord(j0 - c0, src.ext[0], border, x) && map_coord(j1 - c1, src.ext[1], border, y) &&
			    map_coord(j2 - c2, src.ext[2], border, z)) {
				v = to_double(*element_ptr<TS>(src, x, y, z));
			}
		}
		out[i] = v;
	}
}

template<class TK>
__global__ void pad_kernel_kernel(DevView k, int l0, int l1, int l2, double* out)
{
	const long long total = static_cast<long long>(l0) * l1 * l2;
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int j0 = static_cast<int>(i % l0);
		const int j1 = static_cast<int>((i / l0) % l1);
		const int j2 = static_cast<int>(i / (static_cast<long long>(l0) * l1));
		double v = 0.0;
		if (j0 < k.ext[0] && j1 < k.ext[1] && j2 < k.ext[2]) v = to_double(*element_ptr<TK>(k, j0, j1, j2));
		out[i] = v;
	}
}

__global__ void spectral_product_kernel(cufftDoubleComplex* a, const cufftDoubleComplex* b, long long n, double scale)
{
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const cufftDoubleComplex u = a[i], w = b[i];
		a[i] = make_cuDoubleComplex((u.x * w.x - u.y * w.y) * scale, (u.x * w.y + u.y * w.x) * scale);
	}
}

template<class TD>
__global__ void crop_kernel(const double* r, int l0, int l1, int o0, int o1, int o2, DevView dst)
{
	const long long total = static_cast<long long>(dst.ext[0]) * dst.ext[1] * dst.ext[2];
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int x = static_cast<int>(i % dst.ext[0]);
		const int y = static_cast<int>((i / dst.ext[0]) % dst.ext[1]);
		const int z = static_cast<int>(i / (static_cast<long long>(dst.ext[0]) * dst.ext[1]));
		const double v = r[(static_cast<long long>(z + o2) * l1 + (y + o1)) * l0 + (x + o0)];
		*const_cast<TD*>(element_ptr<TD>(dst, x, y, z)) = convert_sum<TD>(v);
	}
}

int grid_of(long long n)
{
	const long long b = (n + 255) / 256;
	const long long cap = 32LL * device_sm_count();
	return static_cast<int>(b < 1 ? 1 : (b > cap ? cap : b));
}

#define IANE_GB_CUFFT(call, what)                                                      \
	do {                                                                                \
		const cufftResult r_ = (call);                                                  \
		if (r_ != CUFFT_SUCCESS) {                                                      \
			return fail(IANE_GB_CUDA_ERROR, std::string(what) + ": cuFFT error " + std::to_string(static_cast<int>(r_))); \
		}                                                                               \
	} while (0)

}  // namespace

// Padded transform extents for a source of extents n and a kernel of extents k (axis 0
// fastest; unused axes 1).
void fft_extents(const DevView& s, const DevView& k, int (&l)[3])
{
	for (int i = 0; i < 3; ++i) l[i] = i < s.rank ? good_size(s.ext[i] + k.ext[i] - 1) : 1;
}

// Predicted seconds of the direct FP32 path and of the FFT path on one GB300. Constants from
// measurements on the 256x256x64 volume: the direct tiled kernel sustains about 50 TFLOP/s
// on large kernels (2.40 ms for 14415 taps); the three FP64 transforms of a 288x288x80 grid
// plus padding, product and crop take 2.68 ms, i.e. about 0.45 TFLOP/s of FFT arithmetic
// (5/2 L log2 L per real transform).
void conv_cost_model(const DevView& s, const DevView& k, double& direct_s, double& fft_s)
{
	const double voxels = static_cast<double>(element_count(s));
	const double taps = static_cast<double>(element_count(k));
	direct_s = std::max(voxels * taps * 2.0 / 50e12, voxels * 8.0 / 3.0e12) + 6e-6;
	int l[3];
	fft_extents(s, k, l);
	const double lt = static_cast<double>(l[0]) * l[1] * l[2];
	// two transforms over the data, one over the kernel, plus padding, product and crop
	fft_s = 3.0 * 2.5 * lt * std::log2(std::max(2.0, lt)) / 0.45e12 + lt * 8.0 * 6.0 / 3.0e12 + 60e-6;
}

bool conv_fft_supported(const DevView& s, const DevView& k, const DevView& d)
{
	auto fp = [](int t) { return t == IANE_GB_F32 || t == IANE_GB_F64; };
	return fp(s.dtype) && fp(k.dtype) && fp(d.dtype) && s.rank >= 1 && s.rank <= 3;
}

int launch_conv_fft(const DevView& s, const DevView& k, const DevView& d, int border, cudaStream_t st)
{
	if (!conv_fft_supported(s, k, d)) {
		return fail(IANE_GB_UNSUPPORTED, "convolve: the FFT path takes f32/f64 source, kernel and destination");
	}
	int l[3];
	fft_extents(s, k, l);
	const long long lt = static_cast<long long>(l[0]) * l[1] * l[2];
	const long long lc = static_cast<long long>(l[2]) * l[1] * (l[0] / 2 + 1);  // complex half-spectrum
	if (lt > (1LL << 31)) {
		return fail(IANE_GB_UNSUPPORTED, "convolve: FFT extents too large");
	}
	int device = 0;
	cudaGetDevice(&device);
	FftPlans plans;
	{
		const std::lock_guard<std::mutex> lock(plan_mutex());
		auto key = std::make_tuple(l[0], l[1], l[2], s.rank, device);
		auto it = plan_cache().find(key);
		if (it == plan_cache().end()) {
			// cuFFT dims are slowest first; the last one is contiguous
			int dims[3];
			for (int i = 0; i < s.rank; ++i) dims[i] = l[s.rank - 1 - i];
			FftPlans p;
			IANE_GB_CUFFT(cufftPlanMany(&p.fwd, s.rank, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_D2Z, 1),
				"convolve: FFT plan");
			if (cufftPlanMany(&p.inv, s.rank, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_Z2D, 1) != CUFFT_SUCCESS) {
				cufftDestroy(p.fwd);
				return fail(IANE_GB_CUDA_ERROR, "convolve: FFT plan");
			}
			it = plan_cache().emplace(key, p).first;
		}
		plans = it->second;
	}
	// buffers: padded source / result (real), padded kernel (real), two half-spectra
	char* base = nullptr;
	const size_t real_bytes = (static_cast<size_t>(lt) * sizeof(double) + 255) & ~size_t(255);
	const size_t cplx_bytes = (static_cast<size_t>(lc) * sizeof(cufftDoubleComplex) + 255) & ~size_t(255);
	IANE_GB_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&base), 2 * real_bytes + 2 * cplx_bytes, st),
		"convolve: FFT buffers");
	double* pr = reinterpret_cast<double*>(base);
	double* kr = reinterpret_cast<double*>(base + real_bytes);
	cufftDoubleComplex* pc = reinterpret_cast<cufftDoubleComplex*>(base + 2 * real_bytes);
	cufftDoubleComplex* kc = reinterpret_cast<cufftDoubleComplex*>(base + 2 * real_bytes + cplx_bytes);
	int status = IANE_GB_OK;
	const int c0 = k.ext[0] / 2, c1 = k.ext[1] / 2, c2 = k.ext[2] / 2;
	const int m0 = s.ext[0] + k.ext[0] - 1, m1 = s.ext[1] + k.ext[1] - 1, m2 = s.ext[2] + k.ext[2] - 1;
	const int g = grid_of(lt);
	if (s.dtype == IANE_GB_F32) {
		pad_source_kernel<float><<<g, 256, 0, st>>>(s, border, c0, c1, c2, l[0], l[1], l[2], m0, m1, m2, pr);
	} else {
		pad_source_kernel<double><<<g, 256, 0, st>>>(s, border, c0, c1, c2, l[0], l[1], l[2], m0, m1, m2, pr);
	}
	if (k.dtype == IANE_GB_F32) {
		pad_kernel_kernel<float><<<g, 256, 0, st>>>(k, l[0], l[1], l[2], kr);
	} else {
		pad_kernel_kernel<double><<<g, 256, 0, st>>>(k, l[0], l[1], l[2], kr);
	}
	{
		const std::lock_guard<std::mutex> lock(plan_mutex()); // a plan runs on one stream at a time
		if (cufftSetStream(plans.fwd, st) != CUFFT_SUCCESS || cufftSetStream(plans.inv, st) != CUFFT_SUCCESS ||
		    cufftExecD2Z(plans.fwd, pr, pc) != CUFFT_SUCCESS || cufftExecD2Z(plans.fwd, kr, kc) != CUFFT_SUCCESS) {
			status = fail(IANE_GB_CUDA_ERROR, "convolve: forward FFT");
		}
		if (!status) {
			spectral_product_kernel<<<grid_of(lc), 256, 0, st>>>(pc, kc, lc, 1.0 / static_cast<double>(lt));
			if (cufftExecZ2D(plans.inv, pc, pr) != CUFFT_SUCCESS) status = fail(IANE_GB_CUDA_ERROR, "convolve: inverse FFT");
		}
	}
	if (!status) {
		const int o0 = k.ext[0] - 1, o1 = k.ext[1] - 1, o2 = k.ext[2] - 1;
		const int gc = grid_of(element_count(d));
		if (d.dtype == IANE_GB_F32) {
			crop_kernel<float><<<gc, 256, 0, st>>>(pr, l[0], l[1], o0, o1, o2, d);
		} else {
			crop_kernel<double><<<gc, 256, 0, st>>>(pr, l[0], l[1], o0, o1, o2, d);
		}
		const cudaError_t e = cudaGetLastError();
		if (e != cudaSuccess) status = cuda_fail(e, "convolve: FFT kernels");
	}
	cudaFreeAsync(base, st);
	return status;
}

}  // namespace iane_gb
