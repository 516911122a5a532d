// Generic direct convolution for every supported element type, border and stride.
//
// One thread per output, 32x8 outputs per block. Each kernel plane's input halo tile is
// staged in shared memory with the border rule applied while loading; the kernel
// coefficients sit in shared memory in the accumulator type. Taps are visited in the
// reference's raster order (kernel axis 0 fastest, include/iane/math/index.hpp:53-64), so
// in exact mode -- FP64 fma starting from +0.0, every tap including zero-border ones --
// the result is bit-identical to the reference's convolution_filter
// (include/iane/algorithms/convolution.hpp:29-76). Fast mode accumulates in FP32 for float
// kernels and in int64 for integer sample/kernel pairs (exact while |sum| < 2^53, where the
// reference's double sum is exact too).
#include "common.cuh"
#include "kernels.h"

#include <type_traits>

namespace iane_gb {
namespace {

constexpr int kGX = 32;
constexpr int kGY = 8;

template<class TAcc> struct acc_ops;
template<> struct acc_ops<float> {
	template<class TS> static __device__ __forceinline__ float sample(TS v) { return to_float(v); }
	static __device__ __forceinline__ float coef(double k) { return static_cast<float>(k); }
	static __device__ __forceinline__ float mac(float s, float k, float acc) { return fmaf(s, k, acc); }
	static __device__ __forceinline__ double to_sum(float acc) { return static_cast<double>(acc); }
};
template<> struct acc_ops<double> {
	template<class TS> static __device__ __forceinline__ double sample(TS v) { return to_double(v); }
	static __device__ __forceinline__ double coef(double k) { return k; }
	static __device__ __forceinline__ double mac(double s, double k, double acc) { return fma(s, k, acc); }
	static __device__ __forceinline__ double to_sum(double acc) { return acc; }
};
template<> struct acc_ops<long long> {
	template<class TS> static __device__ __forceinline__ long long sample(TS v) { return static_cast<long long>(v); }
	static __device__ __forceinline__ long long coef(double k) { return static_cast<long long>(k); }
	static __device__ __forceinline__ long long mac(long long s, long long k, long long acc) { return acc + s * k; }
	static __device__ __forceinline__ double to_sum(long long acc) { return static_cast<double>(acc); }
};

template<class T> __device__ __forceinline__ T zero_value() { return T(0); }
template<> __device__ __forceinline__ __nv_bfloat16 zero_value<__nv_bfloat16>() { return __float2bfloat16(0.0f); }

__device__ __forceinline__ double load_coef(const char* p, int dtype)
{
	switch (dtype) {
	case IANE_GB_I32: return static_cast<double>(*reinterpret_cast<const int32_t*>(p));
	case IANE_GB_F32: return static_cast<double>(*reinterpret_cast<const float*>(p));
	case IANE_GB_F64: return *reinterpret_cast<const double*>(p);
	default: return 0.0;
	}
}

struct GenericArgs {
	DevView src;
	DevView kernel;
	DevView dst;
	int border;
	int staged;    // 1: halo tile in shared memory; 0: direct loads (tile too large)
	int use_tex;   // samples come from `tex` (src gives extents and the texel type only)
	TexSource tex;
};

template<class T> inline constexpr bool texel_type = std::is_same_v<T, uint8_t> || std::is_same_v<T, int8_t> ||
	std::is_same_v<T, uint16_t> || std::is_same_v<T, int16_t> || std::is_same_v<T, int32_t> ||
	std::is_same_v<T, uint32_t> || std::is_same_v<T, float>;

// Sample (xi, yi, zi) (in range) of the memory view or the texture.
template<class TS>
__device__ __forceinline__ TS load_sample(const GenericArgs& a, int xi, int yi, int zi)
{
	if constexpr (texel_type<TS>) {
		if (a.use_tex) {
			return texel<TS>(a.tex.tex, a.tex.rank, a.tex.origin[0] + xi, a.tex.origin[1] + yi, a.tex.origin[2] + zi);
		}
	}
	return *element_ptr<TS>(a.src, xi, yi, zi);
}

template<class TS, class TAcc>
__global__ void __launch_bounds__(kGX * kGY) conv_generic_kernel(GenericArgs a)
{
	using ops = acc_ops<TAcc>;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int kx = a.kernel.ext[0], ky = a.kernel.ext[1], kz = a.kernel.ext[2];
	const int cx = kx / 2, cy = ky / 2, cz = kz / 2;
	const int nx = a.src.ext[0], ny = a.src.ext[1], nz = a.src.ext[2];
	const int tid = threadIdx.y * kGX + threadIdx.x;
	const int x0 = blockIdx.x * kGX, y0 = blockIdx.y * kGY, z = blockIdx.z;
	const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
	const int taps = kx * ky * kz;

	TAcc* coef = reinterpret_cast<TAcc*>(smem_raw);
	for (int i = tid; i < taps; i += kGX * kGY) {
		const int qx = i % kx, qy = (i / kx) % ky, qz = i / (kx * ky);
		const char* p = a.kernel.ptr + qx * a.kernel.stride[0] + qy * a.kernel.stride[1] + qz * a.kernel.stride[2];
		coef[i] = ops::coef(load_coef(p, a.kernel.dtype));
	}
	const int tw = kGX + 2 * cx, th = kGY + 2 * cy;
	TS* tile = reinterpret_cast<TS*>(smem_raw + ((taps * sizeof(TAcc) + 15) & ~size_t(15)));
	TAcc acc = TAcc(0);
	const bool active = x < nx && y < ny;

	for (int qz = 0; qz < kz; ++qz) {
		int zi = 0;
		const bool plane_ok = map_coord(z + cz - qz, nz, a.border, zi);
		__syncthreads();
		if (a.staged && plane_ok) {
			for (int i = tid; i < tw * th; i += kGX * kGY) {
				const int col = i % tw, row = i / tw;
				int xi = 0, yi = 0;
				TS v = zero_value<TS>();
				if (map_coord(x0 - cx + col, nx, a.border, xi) && map_coord(y0 - cy + row, ny, a.border, yi)) {
					v = load_sample<TS>(a, xi, yi, zi);
				}
				tile[i] = v;
			}
		}
		__syncthreads();
		if (!active) {
			continue;
		}
		const TAcc* kp = coef + qz * kx * ky;
		if (!plane_ok) {
			// Every sample of this plane is the zero value; keep the reference's
			// fma(0, k, sum) so that non-finite coefficients propagate the same way.
			for (int q = 0; q < kx * ky; ++q) {
				acc = ops::mac(TAcc(0), kp[q], acc);
			}
			continue;
		}
		for (int qy = 0; qy < ky; ++qy) {
			for (int qx = 0; qx < kx; ++qx) {
				TAcc s;
				if (a.staged) {
					s = ops::sample(tile[(threadIdx.y + 2 * cy - qy) * tw + threadIdx.x + 2 * cx - qx]);
				} else {
					int xi = 0, yi = 0;
					s = TAcc(0);
					if (map_coord(x + cx - qx, nx, a.border, xi) && map_coord(y + cy - qy, ny, a.border, yi)) {
						s = ops::sample(load_sample<TS>(a, xi, yi, zi));
					}
				}
				acc = ops::mac(s, kp[qy * kx + qx], acc);
			}
		}
	}
	if (active) {
		char* out = a.dst.ptr + x * a.dst.stride[0] + y * a.dst.stride[1] + z * a.dst.stride[2];
		store_converted(out, a.dst.dtype, ops::to_sum(acc));
	}
}

template<class TS, class TAcc>
int launch_typed(const GenericArgs& args, cudaStream_t stream)
{
	const int kx = args.kernel.ext[0], ky = args.kernel.ext[1], kz = args.kernel.ext[2];
	const size_t coef_bytes = (static_cast<size_t>(kx) * ky * kz * sizeof(TAcc) + 15) & ~size_t(15);
	const size_t tile_bytes = static_cast<size_t>(kGX + kx - 1) * (kGY + ky - 1) * sizeof(TS);
	constexpr size_t kLimit = 200 * 1024;
	if (coef_bytes > kLimit) {
		return fail(IANE_GB_UNSUPPORTED, "convolve: kernel has too many taps for the generic path");
	}
	GenericArgs a = args;
	a.staged = coef_bytes + tile_bytes <= kLimit ? 1 : 0;
	const size_t smem = coef_bytes + (a.staged ? tile_bytes : 0);
	auto kernel = conv_generic_kernel<TS, TAcc>;
	IANE_GB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
		"convolve: set shared memory size");
	const dim3 grid((a.src.ext[0] + kGX - 1) / kGX, (a.src.ext[1] + kGY - 1) / kGY, a.src.ext[2]);
	kernel<<<grid, dim3(kGX, kGY), smem, stream>>>(a);
	IANE_GB_CUDA(cudaGetLastError(), "convolve: launch generic kernel");
	return IANE_GB_OK;
}

template<class TS>
int launch_for_source(const GenericArgs& args, bool exact, cudaStream_t stream)
{
	if (exact || args.src.dtype == IANE_GB_F64 || args.kernel.dtype == IANE_GB_F64) {
		return launch_typed<TS, double>(args, stream);
	}
	if constexpr (std::is_integral_v<TS>) {
		if (args.kernel.dtype == IANE_GB_I32) {
			return launch_typed<TS, long long>(args, stream);
		}
	}
	return launch_typed<TS, float>(args, stream);
}

}  // namespace

int launch_conv_generic(const DevView& src, const DevView& kernel, const DevView& dst, int border, bool exact,
	cudaStream_t stream, const TexSource* tex)
{
	GenericArgs a{};
	a.src = src;
	a.kernel = kernel;
	a.dst = dst;
	a.border = border;
	a.staged = 1;
	if (tex) {
		a.use_tex = 1;
		a.tex = *tex;
	}
	if (src.ext[1] > 65535 * kGY || src.ext[2] > 65535) {
		return fail(IANE_GB_UNSUPPORTED, "convolve: image too large along axis 1 or 2 for the grid");
	}
	switch (src.dtype) {
	case IANE_GB_U8: return launch_for_source<uint8_t>(a, exact, stream);
	case IANE_GB_U16: return launch_for_source<uint16_t>(a, exact, stream);
	case IANE_GB_I16: return launch_for_source<int16_t>(a, exact, stream);
	case IANE_GB_I32: return launch_for_source<int32_t>(a, exact, stream);
	case IANE_GB_F32: return launch_for_source<float>(a, exact, stream);
	case IANE_GB_F64: return launch_for_source<double>(a, exact, stream);
	case IANE_GB_BF16: return launch_for_source<__nv_bfloat16>(a, exact, stream);
	case IANE_GB_I8: return launch_for_source<int8_t>(a, exact, stream);
	case IANE_GB_U32: return launch_for_source<uint32_t>(a, exact, stream);
	default: return fail(IANE_GB_UNSUPPORTED, "convolve: unsupported source element type");
	}
}

}  // namespace iane_gb
