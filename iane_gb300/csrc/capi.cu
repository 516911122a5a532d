// C-ABI core: error state, view validation, tensor maps, device status, iane_gb_convolve
// and iane_gb_convolve_separable.
#include "common.cuh"
#include "kernels.h"

#include <cstring>
#include <mutex>
#include <string>

namespace iane_gb {

namespace {
thread_local std::string t_last_error;
}

void set_error(const std::string& message) { t_last_error = message; }

int fail(int status, const std::string& message)
{
	set_error(message);
	return status;
}

int cuda_fail(cudaError_t error, const char* what)
{
	set_error(std::string(what) + ": " + cudaGetErrorString(error));
	return error == cudaErrorMemoryAllocation ? IANE_GB_OUT_OF_MEMORY : IANE_GB_CUDA_ERROR;
}

int dtype_size(int dtype)
{
	switch (dtype) {
	case IANE_GB_U8: return 1;
	case IANE_GB_U16: return 2;
	case IANE_GB_I16: return 2;
	case IANE_GB_I32: return 4;
	case IANE_GB_F32: return 4;
	case IANE_GB_F64: return 8;
	case IANE_GB_BF16: return 2;
	case IANE_GB_I8: return 1;
	case IANE_GB_U32: return 4;
	case IANE_GB_RGB8: return 3;
	default: return 0;
	}
}

const char* dtype_name(int dtype)
{
	switch (dtype) {
	case IANE_GB_U8: return "u8";
	case IANE_GB_U16: return "u16";
	case IANE_GB_I16: return "i16";
	case IANE_GB_I32: return "i32";
	case IANE_GB_F32: return "f32";
	case IANE_GB_F64: return "f64";
	case IANE_GB_BF16: return "bf16";
	case IANE_GB_I8: return "i8";
	case IANE_GB_U32: return "u32";
	case IANE_GB_RGB8: return "rgb8";
	default: return "?";
	}
}

int normalise_view(const iane_gb_view* view, const char* name, DevView* out)
{
	if (!view) {
		return fail(IANE_GB_INVALID_ARGUMENT, std::string(name) + ": null view");
	}
	if (view->rank < 1 || view->rank > IANE_GB_MAX_RANK) {
		return fail(IANE_GB_UNSUPPORTED, std::string(name) + ": rank must be 1..3");
	}
	if (dtype_size(view->dtype) == 0) {
		return fail(IANE_GB_UNSUPPORTED, std::string(name) + ": unknown element type");
	}
	DevView v{};
	v.ptr = static_cast<char*>(view->ptr);
	v.dtype = view->dtype;
	v.rank = view->rank;
	long long count = 1;
	for (int i = 0; i < 3; ++i) {
		if (i < view->rank) {
			if (view->extent[i] < 0) {
				return fail(IANE_GB_INVALID_ARGUMENT, std::string(name) + ": negative extent");
			}
			v.ext[i] = view->extent[i];
			v.stride[i] = view->stride[i];
		} else {
			v.ext[i] = 1;
			v.stride[i] = 0;
		}
		count *= v.ext[i];
	}
	if (count > 0 && !v.ptr) {
		return fail(IANE_GB_INVALID_ARGUMENT, std::string(name) + ": null pointer for a nonempty view");
	}
	const int size = v.dtype == IANE_GB_RGB8 ? 1 : dtype_size(v.dtype); // alignment: a packed pixel has 1
	if (count > 0 && (reinterpret_cast<uintptr_t>(v.ptr) % size) != 0) {
		return fail(IANE_GB_INVALID_ARGUMENT, std::string(name) + ": pointer not aligned to its element");
	}
	for (int i = 0; i < view->rank; ++i) {
		if (v.ext[i] > 1 && v.stride[i] % size != 0) {
			return fail(IANE_GB_INVALID_ARGUMENT, std::string(name) + ": stride not a multiple of the element size");
		}
	}
	*out = v;
	return IANE_GB_OK;
}

bool rows_aligned16(const DevView& v)
{
	if (v.stride[0] != dtype_size(v.dtype) || reinterpret_cast<uintptr_t>(v.ptr) % 16 != 0) {
		return false;
	}
	if (v.ext[1] > 1 && v.stride[1] % 16 != 0) return false;
	if (v.ext[2] > 1 && v.stride[2] % 16 != 0) return false;
	return true;
}

int encode_tensor_map_f32(CUtensorMap* map, const void* base, int nx, int ny, int nz, long long row_pitch,
	long long plane_pitch, int bx, int by)
{
	return encode_tensor_map(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, base, nx, ny, nz, row_pitch, plane_pitch, bx, by);
}

int encode_tensor_map(CUtensorMap* map, int data_type, const void* base, int nx, int ny, int nz, long long row_pitch,
	long long plane_pitch, int bx, int by)
{
	const long long dims[3] = {nx, ny, nz};
	const long long strides[2] = {row_pitch, plane_pitch};
	const int box[3] = {bx, by, 1};
	return encode_tensor_map_nd(map, data_type, 3, base, dims, strides, box);
}

int encode_tensor_map_nd(CUtensorMap* map, int data_type, int rank, const void* base, const long long* dims_in,
	const long long* byte_strides, const int* box_in)
{
	using encode_fn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
		const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
		CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
	static encode_fn encode = nullptr;
	static std::once_flag once;
	static cudaError_t lookup = cudaSuccess;
	std::call_once(once, [] {
		void* fn = nullptr;
		cudaDriverEntryPointQueryResult query{};
		lookup = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &query);
		if (lookup == cudaSuccess && query == cudaDriverEntryPointSuccess) {
			encode = reinterpret_cast<encode_fn>(fn);
		}
	});
	if (!encode) {
		return fail(IANE_GB_CUDA_ERROR, "cuTensorMapEncodeTiled is not available from the driver");
	}
	if (rank < 1 || rank > 5) return fail(IANE_GB_INVALID_ARGUMENT, "tensor map rank must be 1..5");
	cuuint64_t dims[5], strides[4];
	cuuint32_t box[5], estride[5];
	for (int i = 0; i < rank; ++i) {
		dims[i] = static_cast<cuuint64_t>(dims_in[i]);
		box[i] = static_cast<cuuint32_t>(box_in[i]);
		estride[i] = 1;
		if (i > 0) strides[i - 1] = static_cast<cuuint64_t>(byte_strides[i - 1]);
	}
	const CUresult r = encode(map, static_cast<CUtensorMapDataType>(data_type), static_cast<cuuint32_t>(rank),
		const_cast<void*>(base), dims, strides, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
		CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	if (r != CUDA_SUCCESS) {
		return fail(IANE_GB_CUDA_ERROR, "cuTensorMapEncodeTiled failed with code " + std::to_string(static_cast<int>(r)));
	}
	return IANE_GB_OK;
}

int device_sm_count()
{
	int device = 0;
	int count = 0;
	if (cudaGetDevice(&device) != cudaSuccess ||
	    cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || count <= 0) {
		return 148;
	}
	return count;
}

// One status word per device that loads the library; bounded device waits that give up
// write a nonzero code here.
__device__ int g_device_status;

int* device_status_ptr()
{
	static std::mutex lock;
	static int* cached[64] = {};
	int device = 0;
	if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 64) {
		set_error("device status: no current CUDA device");
		return nullptr;
	}
	std::lock_guard<std::mutex> guard(lock);
	if (!cached[device]) {
		void* p = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&p, g_device_status);
		if (e != cudaSuccess) {
			cuda_fail(e, "device status: symbol address");
			return nullptr;
		}
		cached[device] = static_cast<int*>(p);
	}
	return cached[device];
}

}  // namespace iane_gb

using namespace iane_gb;

extern "C" {

int iane_gb_abi_version(void) { return IANE_GB_ABI_VERSION; }

size_t iane_gb_last_error(char* buf, size_t size)
{
	const std::string& m = t_last_error;
	if (buf && size > 0) {
		const size_t n = m.size() < size - 1 ? m.size() : size - 1;
		std::memcpy(buf, m.data(), n);
		buf[n] = '\0';
	}
	return m.size();
}

// Read and clear the current device's status word (waits for the stream first).
int iane_gb_device_status(void* stream)
{
	int* p = device_status_ptr();
	if (!p) {
		return IANE_GB_CUDA_ERROR;
	}
	int value = 0;
	const cudaStream_t s = static_cast<cudaStream_t>(stream);
	IANE_GB_CUDA(cudaMemcpyAsync(&value, p, sizeof value, cudaMemcpyDeviceToHost, s), "device status: read");
	IANE_GB_CUDA(cudaMemsetAsync(p, 0, sizeof value, s), "device status: clear");
	IANE_GB_CUDA(cudaStreamSynchronize(s), "device status: wait");
	if (value != 0) {
		return fail(value, "a bounded device wait gave up (status " + std::to_string(value) + ")");
	}
	return IANE_GB_OK;
}

}  // extern "C"

namespace iane_gb {

// A kernel whose one wait never completes: an mbarrier that expects one arrival that nobody
// makes, waited on with a limit of `limit_ns`; the timeout lands in the status word.
__global__ void wait_probe_kernel(int* status, unsigned long long limit_ns)
{
	__shared__ __align__(8) uint64_t bar;
	if (threadIdx.x == 0) {
		mbar_init(&bar, 1);
		fence_barrier_init();
	}
	__syncthreads();
	if (threadIdx.x == 0 && !mbar_wait_bounded(&bar, 0, limit_ns)) {
		report_device_status(status, IANE_GB_DEVICE_TIMEOUT);
	}
}

// The persistent queues' dependency wait: thread 0 waits for a completion counter in global
// memory (as the queues' counters are; the probe's own pair of device words, so probes must not
// overlap) that nothing raises. Kind 1: the bound runs out, the wait records
// IANE_GB_DEVICE_TIMEOUT and raises the abort flag. Kind 2: warp 1 raises the abort flag after
// 1 ms of global time, and the wait must return then without recording anything.
__device__ unsigned int g_probe_counter;
__device__ int g_probe_abort;

__global__ void counter_probe_kernel(int* status, unsigned long long limit_ns, int kind)
{
	if (threadIdx.x == 0) {
		g_probe_counter = 0u;
		g_probe_abort = 0;
		__threadfence();
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		wait_counter(&g_probe_counter, 1u, &g_probe_abort, status, limit_ns);
	} else if (kind == 2 && threadIdx.x == 32) {
		const uint64_t t0 = global_ns();
		while (global_ns() - t0 < 1000000ull) __nanosleep(1000);
		atomicExch(&g_probe_abort, 1);
	}
}

int convolve_checked(const DevView& s, const DevView& k, const DevView& d, int border, unsigned flags, void* stream,
	const TexSource* tex)
{
	if (s.rank != k.rank || s.rank != d.rank) {
		return fail(IANE_GB_INVALID_ARGUMENT, "convolve: source, kernel and destination need the same rank");
	}
	if (border < IANE_GB_BORDER_CLAMP || border > IANE_GB_BORDER_MIRROR) {
		return fail(IANE_GB_INVALID_ARGUMENT, "convolve: unknown border mode");
	}
	if (flags & ~(IANE_GB_ACC_EXACT | IANE_GB_CONV_FFT | IANE_GB_CONV_AUTO)) {
		return fail(IANE_GB_INVALID_ARGUMENT, "convolve: unknown flags");
	}
	if ((flags & IANE_GB_ACC_EXACT) && (flags & (IANE_GB_CONV_FFT | IANE_GB_CONV_AUTO))) {
		return fail(IANE_GB_INVALID_ARGUMENT, "convolve: the exact mode has no spectral variant");
	}
	// convolution.hpp:107-113: positive odd kernel extents.
	for (int i = 0; i < s.rank; ++i) {
		if (k.ext[i] <= 0 || k.ext[i] % 2 == 0) {
			return fail(IANE_GB_INVALID_ARGUMENT, "Convolution requires positive odd kernel dimensions");
		}
	}
	// transform.hpp:51-63: matching nonnegative dimensions.
	for (int i = 0; i < 3; ++i) {
		if (s.ext[i] != d.ext[i]) {
			return fail(IANE_GB_INVALID_ARGUMENT, "Source and destination require matching nonnegative dimensions");
		}
	}
	if (k.dtype != IANE_GB_F32 && k.dtype != IANE_GB_F64 && k.dtype != IANE_GB_I32) {
		return fail(IANE_GB_UNSUPPORTED, std::string("convolve: kernel element type ") + dtype_name(k.dtype));
	}
	if (d.dtype == IANE_GB_BF16) {
		return fail(IANE_GB_UNSUPPORTED, "convolve: bf16 destinations are not supported");
	}
	const bool rgb = s.dtype == IANE_GB_RGB8 || d.dtype == IANE_GB_RGB8;
	if (rgb && (s.dtype != d.dtype || k.dtype != IANE_GB_F32 || tex)) {
		return fail(IANE_GB_UNSUPPORTED, "convolve: rgb8 takes an rgb8 source and destination and an f32 kernel");
	}
	if (tex && (flags & (IANE_GB_CONV_FFT | IANE_GB_CONV_AUTO))) {
		return fail(IANE_GB_UNSUPPORTED, "convolve: texture sources have no spectral path");
	}
	if (element_count(s) == 0) {
		return IANE_GB_OK;
	}
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	const bool exact = (flags & IANE_GB_ACC_EXACT) != 0;
	if (rgb) {
		if (flags & IANE_GB_CONV_FFT) {
			return fail(IANE_GB_UNSUPPORTED, "convolve: rgb8 has no spectral path");
		}
		// Each channel is a u8 image at byte offset c with the pixel strides. A pixel's sum is
		// per channel: (pixel * k) adds r, g and b independently, and each channel's product
		// of a byte and an f32 tap is exact in FP64, so the reference's sum + product equals
		// the exact mode's fma and the byte conversion is the u8 rule.
		for (int c = 0; c < 3; ++c) {
			DevView sc = s, dc = d;
			sc.dtype = dc.dtype = IANE_GB_U8;
			sc.ptr += c;
			dc.ptr += c;
			int status = IANE_GB_UNSUPPORTED;
			if (!exact) status = launch_conv_f32_tiled(sc, k, dc, border, st);
			if (status == IANE_GB_UNSUPPORTED) status = launch_conv_generic(sc, k, dc, border, exact, st);
			if (status) return status;
		}
		return IANE_GB_OK;
	}
	if (flags & IANE_GB_CONV_FFT) {
		return launch_conv_fft(s, k, d, border, st);
	}
	if ((flags & IANE_GB_CONV_AUTO) && conv_fft_supported(s, k, d)) {
		double direct_s = 0.0, fft_s = 0.0;
		conv_cost_model(s, k, direct_s, fft_s);
		if (fft_s < direct_s) {
			return launch_conv_fft(s, k, d, border, st);
		}
	}
	if (!exact) {
		const int status = launch_conv_f32_tiled(s, k, d, border, st, tex);
		if (status != IANE_GB_UNSUPPORTED) {
			return status;
		}
	}
	return launch_conv_generic(s, k, d, border, exact, st, tex);
}

}  // namespace iane_gb

extern "C" {

int iane_gb_wait_probe(unsigned int limit_us, int kind, void* stream)
{
	if (limit_us == 0 || limit_us > 10000000u) {
		return fail(IANE_GB_INVALID_ARGUMENT, "wait probe: the limit is 1 us .. 10 s");
	}
	if (kind < IANE_GB_PROBE_MBARRIER || kind > IANE_GB_PROBE_COUNTER_ABORT) {
		return fail(IANE_GB_INVALID_ARGUMENT, "wait probe: unknown kind");
	}
	int* status = device_status_ptr();
	if (!status) return IANE_GB_CUDA_ERROR;
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	if (kind == IANE_GB_PROBE_MBARRIER) {
		wait_probe_kernel<<<1, 32, 0, st>>>(status, 1000ull * limit_us);
	} else {
		counter_probe_kernel<<<1, 64, 0, st>>>(status, 1000ull * limit_us, kind);
	}
	IANE_GB_CUDA(cudaGetLastError(), "wait probe: launch");
	return IANE_GB_OK;
}

int iane_gb_convolve(const iane_gb_view* src, const iane_gb_view* kernel, const iane_gb_view* dst, int border,
	unsigned flags, void* stream)
{
	DevView s{}, k{}, d{};
	int status = normalise_view(src, "convolve source", &s);
	if (status) return status;
	status = normalise_view(kernel, "convolve kernel", &k);
	if (status) return status;
	status = normalise_view(dst, "convolve destination", &d);
	if (status) return status;
	return convolve_checked(s, k, d, border, flags, stream, nullptr);
}

int iane_gb_convolve_separable(const iane_gb_view* src, const iane_gb_view* const* taps, const iane_gb_view* dst,
	int border, void* stream)
{
	DevView s{}, d{};
	int status = normalise_view(src, "separable source", &s);
	if (status) return status;
	status = normalise_view(dst, "separable destination", &d);
	if (status) return status;
	if (s.rank != d.rank) {
		return fail(IANE_GB_INVALID_ARGUMENT, "separable: source and destination need the same rank");
	}
	if (s.dtype != IANE_GB_F32 || d.dtype != IANE_GB_F32) {
		return fail(IANE_GB_UNSUPPORTED, "separable: source and destination must be f32");
	}
	if (border < IANE_GB_BORDER_CLAMP || border > IANE_GB_BORDER_MIRROR) {
		return fail(IANE_GB_INVALID_ARGUMENT, "separable: unknown border mode");
	}
	if (!taps) {
		return fail(IANE_GB_INVALID_ARGUMENT, "separable: null tap list");
	}
	DevView t[3]{};
	for (int i = 0; i < 3; ++i) {
		if (i < s.rank) {
			status = normalise_view(taps[i], "separable taps", &t[i]);
			if (status) return status;
			if (t[i].rank != 1 || t[i].dtype != IANE_GB_F32) {
				return fail(IANE_GB_INVALID_ARGUMENT, "separable: taps must be 1-D f32 views");
			}
			if (t[i].ext[0] <= 0 || t[i].ext[0] % 2 == 0) {
				return fail(IANE_GB_INVALID_ARGUMENT, "Convolution requires positive odd kernel dimensions");
			}
		} else {
			t[i] = DevView{};
			t[i].ext[0] = t[i].ext[1] = t[i].ext[2] = 1;
		}
	}
	for (int i = 0; i < 3; ++i) {
		if (s.ext[i] != d.ext[i]) {
			return fail(IANE_GB_INVALID_ARGUMENT, "Source and destination require matching nonnegative dimensions");
		}
	}
	if (element_count(s) == 0) {
		return IANE_GB_OK;
	}
	status = launch_conv_separable_fast(s, t, d, border, static_cast<cudaStream_t>(stream));
	if (status != IANE_GB_UNSUPPORTED) {
		return status;
	}
	return launch_conv_separable(s, t, d, border, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
