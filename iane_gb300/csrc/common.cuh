// Shared host/device helpers for the iane_gb kernels (sm_103a only).
#pragma once

#include "../../include/iane_gb/capi.h"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ != 1030)
#error "iane_gb kernels are written for sm_103a only"
#endif

namespace iane_gb {

// ------------------------------------------------------------------------------------
// host-side error state (one message per host thread, read by iane_gb_last_error)

void set_error(const std::string& message);
int fail(int status, const std::string& message);
int cuda_fail(cudaError_t error, const char* what);

#define IANE_GB_CUDA(call, what)                          \
	do {                                                  \
		const cudaError_t iane_gb_err_ = (call);          \
		if (iane_gb_err_ != cudaSuccess) {                \
			return ::iane_gb::cuda_fail(iane_gb_err_, what); \
		}                                                 \
	} while (0)

int dtype_size(int dtype);
const char* dtype_name(int dtype);

// ------------------------------------------------------------------------------------
// views

// A rank-3 normalised view: unused axes have extent 1 and stride 0.
struct DevView {
	char* ptr;
	int dtype;
	int rank;
	int ext[3];
	long long stride[3];
};

// Validate a C-ABI view and normalise it to rank 3. Returns 0 or a negative status.
int normalise_view(const iane_gb_view* view, const char* name, DevView* out);

__host__ __device__ inline long long element_count(const DevView& v)
{
	return static_cast<long long>(v.ext[0]) * v.ext[1] * v.ext[2];
}

// True when axis 0 is contiguous and rows/planes are packed with a pitch that is a
// multiple of 16 bytes and the base pointer is 16-byte aligned.
bool rows_aligned16(const DevView& v);

// ------------------------------------------------------------------------------------
// device-side element access

template<class T> struct dtype_of;
template<> struct dtype_of<uint8_t> { static constexpr int value = IANE_GB_U8; };
template<> struct dtype_of<uint16_t> { static constexpr int value = IANE_GB_U16; };
template<> struct dtype_of<int16_t> { static constexpr int value = IANE_GB_I16; };
template<> struct dtype_of<int32_t> { static constexpr int value = IANE_GB_I32; };
template<> struct dtype_of<float> { static constexpr int value = IANE_GB_F32; };
template<> struct dtype_of<double> { static constexpr int value = IANE_GB_F64; };
template<> struct dtype_of<__nv_bfloat16> { static constexpr int value = IANE_GB_BF16; };
template<> struct dtype_of<int8_t> { static constexpr int value = IANE_GB_I8; };
template<> struct dtype_of<uint32_t> { static constexpr int value = IANE_GB_U32; };

template<class T> __device__ __forceinline__ float to_float(T v) { return static_cast<float>(v); }
template<> __device__ __forceinline__ float to_float<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template<class T> __device__ __forceinline__ double to_double(T v) { return static_cast<double>(v); }
template<> __device__ __forceinline__ double to_double<__nv_bfloat16>(__nv_bfloat16 v)
{
	return static_cast<double>(__bfloat162float(v));
}

// The reference's conversion of an accumulated sum to the destination element
// (include/iane/algorithms/convolution.hpp:51-75): bytes round half up and saturate,
// other integers saturate with NaN -> 0, floating point is a plain cast.
template<class TD> __device__ __forceinline__ TD convert_sum(double sum);
template<> __device__ __forceinline__ uint8_t convert_sum<uint8_t>(double sum)
{
	if (!(sum > 0.0)) return 0;
	if (sum >= 255.0) return 255;
	const unsigned int integer = static_cast<unsigned int>(sum);
	return static_cast<uint8_t>(integer + (sum - integer >= 0.5));
}
template<class TI> __device__ __forceinline__ TI saturate_integral(double sum, double lo, double hi, TI lov, TI hiv)
{
	if (sum != sum) return TI(0);
	if (sum <= lo) return lov;
	if (sum >= hi) return hiv;
	return static_cast<TI>(sum);
}
template<> __device__ __forceinline__ uint16_t convert_sum<uint16_t>(double sum)
{
	return saturate_integral<uint16_t>(sum, 0.0, 65535.0, 0, 65535);
}
template<> __device__ __forceinline__ int16_t convert_sum<int16_t>(double sum)
{
	return saturate_integral<int16_t>(sum, -32768.0, 32767.0, -32768, 32767);
}
template<> __device__ __forceinline__ int32_t convert_sum<int32_t>(double sum)
{
	return saturate_integral<int32_t>(sum, -2147483648.0, 2147483647.0, INT32_MIN, INT32_MAX);
}
template<> __device__ __forceinline__ int8_t convert_sum<int8_t>(double sum)
{
	return saturate_integral<int8_t>(sum, -128.0, 127.0, -128, 127);
}
template<> __device__ __forceinline__ uint32_t convert_sum<uint32_t>(double sum)
{
	return saturate_integral<uint32_t>(sum, 0.0, 4294967295.0, 0u, 4294967295u);
}
template<> __device__ __forceinline__ float convert_sum<float>(double sum) { return static_cast<float>(sum); }
template<> __device__ __forceinline__ double convert_sum<double>(double sum) { return sum; }

// One element of a runtime element type as float (u8..u32, bf16 and f32 are exact for the
// 8- and 16-bit types; i32/u32 round as a float conversion does).
__device__ __forceinline__ float load_as_float(const char* p, int dtype)
{
	switch (dtype) {
	case IANE_GB_U8: return static_cast<float>(*reinterpret_cast<const uint8_t*>(p));
	case IANE_GB_I8: return static_cast<float>(*reinterpret_cast<const int8_t*>(p));
	case IANE_GB_U16: return static_cast<float>(*reinterpret_cast<const uint16_t*>(p));
	case IANE_GB_I16: return static_cast<float>(*reinterpret_cast<const int16_t*>(p));
	case IANE_GB_I32: return static_cast<float>(*reinterpret_cast<const int32_t*>(p));
	case IANE_GB_U32: return static_cast<float>(*reinterpret_cast<const uint32_t*>(p));
	case IANE_GB_BF16: return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(p));
	case IANE_GB_F32: return *reinterpret_cast<const float*>(p);
	default: return 0.0f;
	}
}

// Store a sum into a runtime destination element type with the reference's conversion.
__device__ __forceinline__ void store_converted(char* p, int dtype, double sum)
{
	switch (dtype) {
	case IANE_GB_U8: *reinterpret_cast<uint8_t*>(p) = convert_sum<uint8_t>(sum); break;
	case IANE_GB_I8: *reinterpret_cast<int8_t*>(p) = convert_sum<int8_t>(sum); break;
	case IANE_GB_U16: *reinterpret_cast<uint16_t*>(p) = convert_sum<uint16_t>(sum); break;
	case IANE_GB_I16: *reinterpret_cast<int16_t*>(p) = convert_sum<int16_t>(sum); break;
	case IANE_GB_I32: *reinterpret_cast<int32_t*>(p) = convert_sum<int32_t>(sum); break;
	case IANE_GB_U32: *reinterpret_cast<uint32_t*>(p) = convert_sum<uint32_t>(sum); break;
	case IANE_GB_F32: *reinterpret_cast<float*>(p) = convert_sum<float>(sum); break;
	case IANE_GB_F64: *reinterpret_cast<double*>(p) = sum; break;
	default: break;
	}
}

// The same conversions for an FP32 sum, in FP32 arithmetic. They equal convert_sum of the
// sum widened to double: v - (unsigned)v is exact for a float below 2^24, and a float
// compares with the saturation bounds as its double does once an upper bound that is not a
// float (2^31 - 1, 2^32 - 1) is replaced by the next float up (no float lies in between).
__device__ __forceinline__ uint8_t convert_f32_u8(float v)
{
	if (!(v > 0.0f)) return 0;
	if (v >= 255.0f) return 255;
	const unsigned int integer = static_cast<unsigned int>(v);
	return static_cast<uint8_t>(integer + (v - static_cast<float>(integer) >= 0.5f));
}
template<class TI>
__device__ __forceinline__ TI saturate_f32(float v, float lo, float hi, TI lov, TI hiv)
{
	if (v != v) return TI(0);
	if (v <= lo) return lov;
	if (v >= hi) return hiv;
	return static_cast<TI>(v);
}
__device__ __forceinline__ void store_converted_f32(char* p, int dtype, float v)
{
	switch (dtype) {
	case IANE_GB_U8: *reinterpret_cast<uint8_t*>(p) = convert_f32_u8(v); break;
	case IANE_GB_I8: *reinterpret_cast<int8_t*>(p) = saturate_f32<int8_t>(v, -128.0f, 127.0f, -128, 127); break;
	case IANE_GB_U16: *reinterpret_cast<uint16_t*>(p) = saturate_f32<uint16_t>(v, 0.0f, 65535.0f, 0, 65535); break;
	case IANE_GB_I16:
		*reinterpret_cast<int16_t*>(p) = saturate_f32<int16_t>(v, -32768.0f, 32767.0f, -32768, 32767);
		break;
	case IANE_GB_I32:
		*reinterpret_cast<int32_t*>(p) = saturate_f32<int32_t>(v, -2147483648.0f, 2147483648.0f, INT32_MIN, INT32_MAX);
		break;
	case IANE_GB_U32:
		*reinterpret_cast<uint32_t*>(p) = saturate_f32<uint32_t>(v, 0.0f, 4294967296.0f, 0u, 4294967295u);
		break;
	case IANE_GB_F32: *reinterpret_cast<float*>(p) = v; break;
	case IANE_GB_F64: *reinterpret_cast<double*>(p) = static_cast<double>(v); break;
	default: break;
	}
}

// A texel of a point-sampled texture with unnormalised coordinates, read at its centre as
// the reference's texture_image_view::operator[] does (texture_image_view.hpp:45-53).
template<class T>
__device__ __forceinline__ T texel(cudaTextureObject_t tex, int rank, int x, int y, int z)
{
	if (rank == 1) return tex1D<T>(tex, x + 0.5f);
	if (rank == 2) return tex2D<T>(tex, x + 0.5f, y + 0.5f);
	return tex3D<T>(tex, x + 0.5f, y + 0.5f, z + 0.5f);
}

// A texel as float (exact for the 8- and 16-bit types; i32/u32 round as a float conversion
// does).
__device__ __forceinline__ float texel_as_float(cudaTextureObject_t tex, int dtype, int rank, int x, int y, int z)
{
	switch (dtype) {
	case IANE_GB_U8: return static_cast<float>(texel<unsigned char>(tex, rank, x, y, z));
	case IANE_GB_I8: return static_cast<float>(texel<signed char>(tex, rank, x, y, z));
	case IANE_GB_U16: return static_cast<float>(texel<unsigned short>(tex, rank, x, y, z));
	case IANE_GB_I16: return static_cast<float>(texel<short>(tex, rank, x, y, z));
	case IANE_GB_I32: return static_cast<float>(texel<int>(tex, rank, x, y, z));
	case IANE_GB_U32: return static_cast<float>(texel<unsigned int>(tex, rank, x, y, z));
	case IANE_GB_F32: return texel<float>(tex, rank, x, y, z);
	default: return 0.0f;
	}
}

// Texture source of a convolution (a normalised iane_gb_texture_view).
struct TexSource {
	cudaTextureObject_t tex;
	int dtype;
	int rank;
	int origin[3];
};

// Border rule for one coordinate: returns false if the sample is the zero value.
// clamp/zero follow include/iane/locator/image_locator.hpp:44-52; mirror is half-sample
// symmetric with period 2n.
__device__ __forceinline__ bool map_coord(int c, int n, int border, int& out)
{
	if (c >= 0 && c < n) {
		out = c;
		return true;
	}
	if (border == IANE_GB_BORDER_ZERO) {
		return false;
	}
	if (border == IANE_GB_BORDER_CLAMP) {
		out = c < 0 ? 0 : n - 1;
		return true;
	}
	const int period = 2 * n;
	int m = c % period;
	if (m < 0) m += period;
	out = m < n ? m : period - 1 - m;
	return true;
}

template<class T>
__device__ __forceinline__ const T* element_ptr(const DevView& v, int x, int y, int z)
{
	return reinterpret_cast<const T*>(v.ptr + x * v.stride[0] + y * v.stride[1] + z * v.stride[2]);
}

// ------------------------------------------------------------------------------------
// device status word: bounded waits that give up record a code here instead of trapping

// `status` points at a library-owned device word (see device_status_ptr()).
__device__ __forceinline__ void report_device_status(int* status, int code)
{
	atomicCAS(status, 0, code);
}

// ------------------------------------------------------------------------------------
// TMA / mbarrier helpers (inline PTX, sm_90+ forms that sm_103a supports)

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
	return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init()
{
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
		: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
	uint32_t done;
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		"selp.u32 %0, 1, 0, p;\n\t}"
		: "=r"(done)
		: "r"(smem_addr(bar)), "r"(parity)
		: "memory");
	return done != 0;
}

// Nanoseconds of the GPU's global timer.
__device__ __forceinline__ uint64_t global_ns()
{
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// Acquire load of a completion counter that other CTAs release with a fence and an atomic.
__device__ __forceinline__ unsigned int load_acquire(const unsigned int* p)
{
	unsigned int v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ int load_volatile(const int* p)
{
	return *reinterpret_cast<const volatile int*>(p);
}

// Generic-proxy writes of this thread (epilogue stores) ordered against async-proxy (TMA)
// accesses to global memory: used after a tile's stores and before a dependent tile's loads.
__device__ __forceinline__ void fence_proxy_async_global()
{
	asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Bounded wait until *word >= need. False if the run was aborted or the wait gave up after
// `limit_ns` of global time (which it records in the status word and turns into an abort).
__device__ __forceinline__ bool wait_counter(const unsigned int* word, unsigned int need, int* abort, int* status,
	uint64_t limit_ns = 2000000000ull)
{
	if (load_acquire(word) >= need) {
		return true;
	}
	const uint64_t t0 = global_ns();
	for (uint32_t i = 1; i < (1u << 26); ++i) {
		if (load_acquire(word) >= need) {
			return true;
		}
		if (load_volatile(abort)) {
			return false;
		}
		if ((i & 63u) == 0 && global_ns() - t0 > limit_ns) {
			break;
		}
		__nanosleep(64);
	}
	report_device_status(status, IANE_GB_DEVICE_TIMEOUT);
	atomicExch(abort, 1);
	return false;
}

// Bounded wait on an mbarrier phase: gives up (returns false) after `limit_ns` of global time
// -- two seconds unless told otherwise -- or 2^26 tries, whichever comes first, so that a
// phase that never completes ends the kernel instead of hanging it. The caller records the
// timeout in the device status word and finishes.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns = 2000000000ull)
{
	if (mbar_try_wait(bar, parity)) {
		return true;
	}
	const uint64_t t0 = global_ns();
	for (uint32_t i = 1; i < (1u << 26); ++i) {
		if (mbar_try_wait(bar, parity)) {
			return true;
		}
		if ((i & 255u) == 0 && global_ns() - t0 > limit_ns) {
			return false;
		}
	}
	return false;
}

// 3-D tiled TMA load into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar)
{
	asm volatile(
		"cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
		::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
		: "memory");
}

// 5-D tiled TMA load into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
	uint64_t* bar)
{
	asm volatile(
		"cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
		::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4),
		"r"(smem_addr(bar))
		: "memory");
}

// 4-byte asynchronous global->shared copy; src_bytes = 0 writes zero.
__device__ __forceinline__ void cp_async4(void* dst, const void* src, int src_bytes)
{
	asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_addr(dst)), "l"(src), "r"(src_bytes)
		: "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template<int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// ------------------------------------------------------------------------------------
// host: tensor maps

// Encode a 3-D f32 tensor map over a packed-pitch buffer: dims (nx, ny, nz), byte pitches
// row_pitch (dim 1) and plane_pitch (dim 2), box (bx, by, 1), zero fill out of bounds.
int encode_tensor_map_f32(CUtensorMap* map, const void* base, int nx, int ny, int nz,
	long long row_pitch, long long plane_pitch, int bx, int by);
// The same for any CUtensorMapDataType (e.g. CU_TENSOR_MAP_DATA_TYPE_BFLOAT16).
int encode_tensor_map(CUtensorMap* map, int data_type, const void* base, int nx, int ny, int nz,
	long long row_pitch, long long plane_pitch, int bx, int by);
// Rank 1..5: dims[rank] elements, byte_strides[rank - 1] of dims 1.., box[rank] elements.
int encode_tensor_map_nd(CUtensorMap* map, int data_type, int rank, const void* base, const long long* dims,
	const long long* byte_strides, const int* box);

int device_sm_count();

// Device address of the status word of the current device (one int per device, zero while
// no bounded wait has given up). Null on failure, with the error recorded.
int* device_status_ptr();

}  // namespace iane_gb
