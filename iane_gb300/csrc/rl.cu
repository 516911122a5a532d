// Richardson-Lucy as a prepared algorithm: plan (prepare), scratch sizing and run.
//
// Reference: examples/rl_deconvolution/main.cu:51-81 (prepare_rl and the iteration),
// include/iane/execution/prepared.hpp:120-146 (prepare -> scratch_bytes, run with scratch),
// include/iane/execution/run_on.hpp:86-178 (host staging for the end-to-end entry point).
//
// HBM layout of the scratch (each part 256-byte aligned):
//   ratio  : f32 work image, rows padded to a multiple of 4 floats (TMA-addressable)
//   est    : f32 work estimate, same layout (unused when the caller's estimate view already
//            has that layout -- then the passes update it in place)
//   parts  : 3 doubles per block of pass B (statistics partials)
//   misc   : block-completion counter and the flat-start value
//   sync   : queue counter, abort flag and per-plane completion counters of the persistent
//            run (rl_persist.cuh)
#include "kernels.h"
#include "rl.cuh"
#include "rl_tcz.cuh"
#include "rl_batch.cuh"
#include "rl_persist.cuh"

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

struct iane_gb_rl_plan {
	int rank;
	int ext[3];
	int k[3];
	int device;
	float* d_psf;  // packed PSF
	float* d_adj;  // packed adjoint (every axis reversed)
	int* d_cls;    // sensitivity class per coordinate: x then y then z
	float* d_sens; // sensitivity per class triple
	int ccount[3];
	int ilo[3], ihi[3];
	float s_interior;
	long long pitch;       // floats per work-image row
	size_t image_bytes;    // one work image, rounded to 256
	size_t parts_bytes;
	size_t sync_bytes;     // persistent-run words (FP32 path)
	size_t scratch_bytes;
	bool small_tiles;
	bool per_pass;         // IANE_GB_RL_PER_PASS: one launch per pass instead of one per run
	long long pass_blocks;
	// BF16 tensor-core precision path (IANE_GB_RL_BF16_TENSOR)
	bool bf16;
	__nv_bfloat16* d_tmat_psf; // banded T matrices per kernel row, psf and adjoint
	__nv_bfloat16* d_tmat_adj;
	long long pitch16;         // bf16 elements per work-image row (multiple of 8)
	size_t image16_bytes;
	bool tcz;                  // z planes along N (rl_tcz.cuh); T matrices in its layout
};

namespace iane_gb {

int launch_rl_pass_a_lo(int, bool, const CUtensorMap&, const TileArgs&, const EpiRatio&, cudaStream_t);
int launch_rl_pass_a_hi(int, bool, const CUtensorMap&, const TileArgs&, const EpiRatio&, cudaStream_t);
int launch_rl_pass_b_lo(int, bool, const CUtensorMap&, const TileArgs&, const EpiUpdate&, cudaStream_t);
int launch_rl_pass_b_hi(int, bool, const CUtensorMap&, const TileArgs&, const EpiUpdate&, cudaStream_t);

int launch_rl_pass_a(int kx, bool small, const CUtensorMap& map, const TileArgs& a, const EpiRatio& e,
	cudaStream_t stream)
{
	return kx <= 15 ? launch_rl_pass_a_lo(kx, small, map, a, e, stream) : launch_rl_pass_a_hi(kx, small, map, a, e, stream);
}

int launch_rl_pass_b(int kx, bool small, const CUtensorMap& map, const TileArgs& a, const EpiUpdate& e,
	cudaStream_t stream)
{
	return kx <= 15 ? launch_rl_pass_b_lo(kx, small, map, a, e, stream) : launch_rl_pass_b_hi(kx, small, map, a, e, stream);
}

int launch_rl_persist(int kx, const RlPersistArgs& p, cudaStream_t stream)
{
	return kx <= 15 ? launch_rl_persist_lo(kx, p, stream) : launch_rl_persist_hi(kx, p, stream);
}

namespace {

constexpr size_t kAlign = 256;
inline size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

__global__ void gather_f32_kernel(DevView src, float* dst)
{
	const long long n = element_count(src);
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int x = static_cast<int>(i % src.ext[0]);
		const int y = static_cast<int>((i / src.ext[0]) % src.ext[1]);
		const int z = static_cast<int>(i / (static_cast<long long>(src.ext[0]) * src.ext[1]));
		dst[i] = *element_ptr<float>(src, x, y, z);
	}
}

// Observed-based start (main.cu:12-19) or flat start, into the work estimate.
__global__ void rl_init_kernel(DevView obs, float* est, long long pitch, long long plane, float eps, int mode,
	const float* start)
{
	const int nx = obs.ext[0], ny = obs.ext[1], nz = obs.ext[2];
	const long long n = static_cast<long long>(nx) * ny * nz;
	const float flat = mode == IANE_GB_RL_INIT_MEAN ? *start : 0.0f;
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int x = static_cast<int>(i % nx);
		const int y = static_cast<int>((i / nx) % ny);
		const int z = static_cast<int>(i / (static_cast<long long>(nx) * ny));
		float v = flat;
		if (mode == IANE_GB_RL_INIT_OBSERVED) {
			const char* p = obs.ptr + x * obs.stride[0] + y * obs.stride[1] + z * obs.stride[2];
			const float o = obs.dtype == IANE_GB_U8 ? static_cast<float>(*reinterpret_cast<const uint8_t*>(p))
				: *reinterpret_cast<const float*>(p);
			v = o > eps ? o : eps;
		}
		est[z * plane + y * pitch + x] = v;
	}
}

// Sum of the observed image in FP64; the last block writes max(mean, eps) to *start.
__global__ void rl_mean_kernel(DevView obs, double* partials, unsigned int* counter, float* start, float eps)
{
	const int nx = obs.ext[0], ny = obs.ext[1], nz = obs.ext[2];
	const long long n = static_cast<long long>(nx) * ny * nz;
	// every warp takes whole rows (one index division per row, none per voxel), lanes stride x
	const int lane = threadIdx.x & 31;
	const long long warps = static_cast<long long>(gridDim.x) * (blockDim.x >> 5);
	const bool u8 = obs.dtype == IANE_GB_U8;
	double s = 0.0;
	for (long long r = blockIdx.x * static_cast<long long>(blockDim.x >> 5) + (threadIdx.x >> 5);
	     r < static_cast<long long>(ny) * nz; r += warps) {
		const int y = static_cast<int>(r % ny), z = static_cast<int>(r / ny);
		const char* row = obs.ptr + y * obs.stride[1] + z * obs.stride[2];
		for (int x = lane; x < nx; x += 32) {
			const char* p = row + x * obs.stride[0];
			s += u8 ? static_cast<double>(*reinterpret_cast<const uint8_t*>(p)) : static_cast<double>(*reinterpret_cast<const float*>(p));
		}
	}
	__shared__ double red[32];
	__shared__ int last;
	for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
	__syncthreads();
	if (threadIdx.x == 0) {
		double t = 0.0;
		for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += red[w];
		partials[blockIdx.x] = t;
		__threadfence();
		last = atomicAdd(counter, 1u) == gridDim.x - 1;
	}
	__syncthreads();
	if (!last) {
		return;
	}
	// the last block combines the block partials: each thread a strided share, then the warps
	// and the block (a fixed order, so the start value is deterministic)
	__threadfence();
	double t = 0.0;
	for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x) t += __ldcg(&partials[b]);
	for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
	__syncthreads();
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
	__syncthreads();
	if (threadIdx.x == 0) {
		double total = 0.0;
		for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) total += red[w];
		const float mean = static_cast<float>(total / static_cast<double>(n));
		*start = mean > eps ? mean : eps;
		*counter = 0u;
	}
}

// Copy between the work estimate and a caller view (f32 or u8 via to_gray8).
__global__ void rl_copy_kernel(float* est, long long pitch, long long plane, DevView view, int to_view)
{
	const int nx = view.ext[0], ny = view.ext[1], nz = view.ext[2];
	const long long n = static_cast<long long>(nx) * ny * nz;
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int x = static_cast<int>(i % nx);
		const int y = static_cast<int>((i / nx) % ny);
		const int z = static_cast<int>(i / (static_cast<long long>(nx) * ny));
		char* p = view.ptr + x * view.stride[0] + y * view.stride[1] + z * view.stride[2];
		float& e = est[z * plane + y * pitch + x];
		if (to_view) {
			if (view.dtype == IANE_GB_U8) {
				*reinterpret_cast<uint8_t*>(p) = to_gray8(e);
			} else {
				*reinterpret_cast<float*>(p) = e;
			}
		} else {
			e = *reinterpret_cast<const float*>(p);
		}
	}
}

int grid_for(long long n)
{
	const long long blocks = (n + 255) / 256;
	const long long cap = 8LL * device_sm_count();
	return static_cast<int>(blocks < 1 ? 1 : (blocks > cap ? cap : blocks));
}

// Per-axis sensitivity classes: voxel p sees kernel taps [max(0, p+c-n+1), min(k-1, p+c)].
void axis_classes(int n, int k, std::vector<int>& cls, std::vector<std::pair<int, int>>& ranges, int& lo, int& hi)
{
	const int c = k / 2;
	cls.assign(n, 0);
	ranges.clear();
	lo = c;
	hi = n - 1 - c;
	for (int p = 0; p < n; ++p) {
		const int qlo = p + c - n + 1 > 0 ? p + c - n + 1 : 0;
		const int qhi = p + c < k - 1 ? p + c : k - 1;
		int id = -1;
		for (size_t i = 0; i < ranges.size(); ++i) {
			if (ranges[i].first == qlo && ranges[i].second == qhi) {
				id = static_cast<int>(i);
				break;
			}
		}
		if (id < 0) {
			id = static_cast<int>(ranges.size());
			ranges.emplace_back(qlo, qhi);
		}
		cls[p] = id;
	}
}

bool is_work_layout(const DevView& v, long long pitch)
{
	// The caller's estimate can be updated in place when it is f32, packed with our row
	// pitch and 16-byte aligned.
	if (v.dtype != IANE_GB_F32 || v.stride[0] != 4 || reinterpret_cast<uintptr_t>(v.ptr) % 16 != 0) return false;
	if (v.ext[1] > 1 && v.stride[1] != pitch * 4) return false;
	if (v.ext[2] > 1 && v.stride[2] != pitch * 4 * v.ext[1]) return false;
	return true;
}

}  // namespace
}  // namespace iane_gb

namespace iane_gb {

void rl_plan_fill_passes(const iane_gb_rl_plan* plan, TileArgs* pa, TileArgs* pb, EpiRatio* ea, EpiUpdate* eb,
	int* status)
{
	TileArgs t{};
	t.nx = plan->ext[0];
	t.ny = plan->ext[1];
	t.nz = plan->ext[2];
	t.ky = plan->k[1];
	t.kz = plan->k[2];
	t.k_stride[0] = 4;
	t.k_stride[1] = 4LL * plan->k[0];
	t.k_stride[2] = 4LL * plan->k[0] * plan->k[1];
	t.border = IANE_GB_BORDER_ZERO;
	t.status = status;
	*pa = t;
	*pb = t;
	pa->kernel = reinterpret_cast<const char*>(plan->d_psf);
	pb->kernel = reinterpret_cast<const char*>(plan->d_adj);
	const long long plane = plan->pitch * plan->ext[1];
	*ea = EpiRatio{};
	ea->pitch = plan->pitch;
	ea->plane = plane;
	ea->nx = plan->ext[0];
	ea->ny = plan->ext[1];
	*eb = EpiUpdate{};
	eb->pitch = plan->pitch;
	eb->plane = plane;
	eb->nx = plan->ext[0];
	eb->ny = plan->ext[1];
	eb->nz = plan->ext[2];
	eb->cls = plan->d_cls;
	eb->sens = plan->d_sens;
	eb->cx_count = plan->ccount[0];
	eb->cy_count = plan->ccount[1];
	for (int i = 0; i < 3; ++i) {
		eb->ilo[i] = plan->ilo[i];
		eb->ihi[i] = plan->ihi[i];
	}
	eb->s_interior = plan->s_interior;
}

}  // namespace iane_gb

// ------------------------------------------------------------------------------------
// BF16 tensor-core precision path (plans prepared with IANE_GB_RL_BF16_TENSOR).

namespace iane_gb {
namespace {

__global__ void rl_to_bf16_kernel(const float* e, long long pitch, long long plane, __nv_bfloat16* d, long long pitch16,
	long long plane16, int nx, int ny, int nz)
{
	const long long n = static_cast<long long>(nx) * ny * nz;
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int x = static_cast<int>(i % nx);
		const int y = static_cast<int>((i / nx) % ny);
		const int z = static_cast<int>(i / (static_cast<long long>(nx) * ny));
		d[z * plane16 + y * pitch16 + x] = __float2bfloat16_rn(e[z * plane + y * pitch + x]);
	}
}

int rl_run_bf16(iane_gb_rl_plan* plan, const DevView& obs, const DevView& est, int iterations, float epsilon, int init,
	char* base, double* stats, cudaStream_t st)
{
	const int nx = plan->ext[0], ny = plan->ext[1], nz = plan->ext[2];
	const long long pitch = plan->pitch, plane = pitch * ny;
	const long long p16 = plan->pitch16, plane16 = p16 * ny;
	float* work = reinterpret_cast<float*>(base);
	__nv_bfloat16* est16 = reinterpret_cast<__nv_bfloat16*>(base + plan->image_bytes);
	__nv_bfloat16* ratio16 = reinterpret_cast<__nv_bfloat16*>(base + plan->image_bytes + plan->image16_bytes);
	double* parts = reinterpret_cast<double*>(base + plan->image_bytes + 2 * plan->image16_bytes);
	unsigned int* counter = reinterpret_cast<unsigned int*>(reinterpret_cast<char*>(parts) + plan->parts_bytes);
	float* start = reinterpret_cast<float*>(counter + 1);
	const bool in_place = is_work_layout(est, pitch);
	float* e_work = in_place ? reinterpret_cast<float*>(est.ptr) : work;
	const long long n = static_cast<long long>(nx) * ny * nz;

	IANE_GB_CUDA(cudaMemsetAsync(counter, 0, 2 * sizeof(unsigned int), st), "rl_run: clear counter");
	if (init == IANE_GB_RL_INIT_GIVEN) {
		if (!in_place) {
			rl_copy_kernel<<<grid_for(n), 256, 0, st>>>(e_work, pitch, plane, est, 0);
		}
	} else {
		if (init == IANE_GB_RL_INIT_MEAN) {
			rl_mean_kernel<<<grid_for(n), 256, 0, st>>>(obs, parts, counter, start, epsilon);
		}
		rl_init_kernel<<<grid_for(n), 256, 0, st>>>(obs, e_work, pitch, plane, epsilon, init, start);
	}
	rl_to_bf16_kernel<<<grid_for(n), 256, 0, st>>>(e_work, pitch, plane, est16, p16, plane16, nx, ny, nz);
	IANE_GB_CUDA(cudaGetLastError(), "rl_run: launch init");

	int* dstatus = device_status_ptr();
	if (!dstatus) return IANE_GB_CUDA_ERROR;
	const int ky = plan->k[1];
	CUtensorMap map_est{}, map_ratio{};
	int status = encode_tensor_map(&map_est, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, est16, nx, ny, nz, p16 * 2, plane16 * 2,
		8, tc_rows(ky));
	if (status) return status;
	status = encode_tensor_map(&map_ratio, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, ratio16, nx, ny, nz, p16 * 2, plane16 * 2,
		8, tc_rows(ky));
	if (status) return status;

	TcArgs ta{};
	ta.nx = nx;
	ta.ny = ny;
	ta.nz = nz;
	ta.ky = ky;
	ta.kz = plan->k[2];
	ta.status = dstatus;
	ta.smem_bytes = static_cast<int>(plan->tcz ? tcz_smem_bytes(ky, plan->k[2]) : tc_smem_bytes(ky));
	ta.tmem_cols = kTcTmemCols;
	TcArgs tb = ta;
	ta.tmat = plan->d_tmat_psf;
	tb.tmat = plan->d_tmat_adj;

	EpiRatioTc ea{};
	ea.ratio = ratio16;
	ea.pitch = p16;
	ea.plane = plane16;
	ea.obs = obs.ptr;
	for (int i = 0; i < 3; ++i) ea.os[i] = obs.stride[i];
	ea.obs_u8 = obs.dtype == IANE_GB_U8;
	ea.eps = epsilon;
	ea.nx = nx;
	ea.ny = ny;

	EpiUpdateTc eb{};
	eb.est = e_work;
	eb.pitch = pitch;
	eb.plane = plane;
	eb.est16 = est16;
	eb.pitch16 = p16;
	eb.plane16 = plane16;
	eb.eps = epsilon;
	eb.nx = nx;
	eb.ny = ny;
	eb.nz = nz;
	eb.cls = plan->d_cls;
	eb.sens = plan->d_sens;
	eb.cx_count = plan->ccount[0];
	eb.cy_count = plan->ccount[1];
	for (int i = 0; i < 3; ++i) {
		eb.ilo[i] = plan->ilo[i];
		eb.ihi[i] = plan->ihi[i];
		eb.outs[i] = est.stride[i];
	}
	eb.s_interior = plan->s_interior;
	eb.partials = parts;
	eb.counter = counter;
	eb.out = est.ptr;
	eb.out_u8 = est.dtype == IANE_GB_U8;
	for (int it = 0; it < iterations; ++it) {
		status = plan->tcz ? launch_tcz_pass_a(map_est, ta, ea, st) : launch_tc_pass_a(map_est, ta, ea, st);
		if (status) return status;
		eb.want_stats = stats != nullptr;
		eb.stats = stats ? stats + 2 * it : nullptr;
		eb.write_out = (!in_place && it == iterations - 1) ? 1 : 0;
		status = plan->tcz ? launch_tcz_pass_b(map_ratio, tb, eb, st) : launch_tc_pass_b(map_ratio, tb, eb, st);
		if (status) return status;
	}
	if (iterations == 0 && !in_place) {
		rl_copy_kernel<<<grid_for(n), 256, 0, st>>>(e_work, pitch, plane, est, 1);
		IANE_GB_CUDA(cudaGetLastError(), "rl_run: launch copy-out");
	}
	return IANE_GB_OK;
}

}  // namespace
}  // namespace iane_gb

// ------------------------------------------------------------------------------------
// Allocation-free variant (iane_gb_rl_run_noalloc).
//
// Some callers cannot call cudaMalloc: plugins loaded into a host application that owns the
// device allocator (a pooled allocator, or a memory budget the plugin must not bypass), and
// real-time loops that must not block in the driver's allocator, whose cudaMalloc and
// cudaFree may synchronise the device. For them the variant
// keeps every byte of RL's scratch -- ratio image, work estimate, sensitivity classes and
// table, mean partials -- in the file-scope array below, sized for images of at most
// kNoAllocMaxVoxels padded voxels. Every GPU that loads this library holds the array
// (about 32.4 MiB) until the process exits.

namespace iane_gb {
namespace {

constexpr long long kNoAllocMaxVoxels = 1LL << 22;  // round_up(nx, 4) * ny * nz
constexpr int kNoAllocMaxAxisSum = 1 << 16;          // nx + ny + nz
constexpr long long kNoAllocMaxTaps = 1LL << 15;     // PSF taps (also bounds the class table)
constexpr int kNoAllocMaxExtent = 63;                // PSF extent per axis
constexpr int kNoAllocMaxPartials = 4096;            // blocks of the mean reduction
constexpr size_t kNoAllocImageBytes = static_cast<size_t>(kNoAllocMaxVoxels) * sizeof(float);
constexpr size_t kNoAllocClsOffset = 2 * kNoAllocImageBytes;
constexpr size_t kNoAllocTableOffset = kNoAllocClsOffset + kNoAllocMaxAxisSum * sizeof(int);
constexpr size_t kNoAllocRangeOffset = kNoAllocTableOffset + kNoAllocMaxTaps * sizeof(float);
constexpr size_t kNoAllocPartsOffset = kNoAllocRangeOffset + 256 * 3 * 2 * sizeof(int);
constexpr size_t kNoAllocCounterOffset = kNoAllocPartsOffset + kNoAllocMaxPartials * sizeof(double);
constexpr size_t kNoAllocBytes = kNoAllocCounterOffset + 256;

}  // namespace
}  // namespace iane_gb

// The shared scratch of iane_gb_rl_run_noalloc. In host code this name is only a host-side
// stand-in: the device address comes from cudaGetSymbolAddress (noalloc_scratch()).
static __device__ __align__(256) unsigned char iane_gb_rl_noalloc_scratch[iane_gb::kNoAllocBytes];

namespace iane_gb {
namespace {

// Device address of the array on the current device, looked up once per device with that
// device current. Null on failure, with the error recorded.
char* noalloc_scratch()
{
	static std::mutex lock;
	static char* cached[64] = {};
	int device = 0;
	if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 64) {
		set_error("rl_run_noalloc: no current CUDA device");
		return nullptr;
	}
	std::lock_guard<std::mutex> guard(lock);
	if (!cached[device]) {
		void* p = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&p, iane_gb_rl_noalloc_scratch);
		if (e != cudaSuccess || !p) {
			cuda_fail(e, "rl_run_noalloc: address of the static scratch");
			return nullptr;
		}
		cached[device] = static_cast<char*>(p);
	}
	return cached[device];
}

// Number of sensitivity classes along one axis: the (first, last) tap ranges of
// axis_classes() change monotonically with the coordinate, so classes are runs.
int count_classes(int n, int k)
{
	const int c = k / 2;
	int count = 0, last_lo = -1, last_hi = -1;
	for (int p = 0; p < n; ++p) {
		const int qlo = p + c - n + 1 > 0 ? p + c - n + 1 : 0;
		const int qhi = p + c < k - 1 ? p + c : k - 1;
		if (qlo != last_lo || qhi != last_hi) {
			++count;
			last_lo = qlo;
			last_hi = qhi;
		}
	}
	return count;
}

// Class index per coordinate (x at 0, y at nx, z at nx + ny) and each class's tap range,
// numbered in order of appearance exactly as axis_classes() does on the host.
__global__ void noalloc_classes_kernel(int nx, int ny, int nz, int kx, int ky, int kz, int* cls, int* ranges)
{
	const int axis = threadIdx.x;
	if (axis >= 3) return;
	const int n = axis == 0 ? nx : (axis == 1 ? ny : nz);
	const int k = axis == 0 ? kx : (axis == 1 ? ky : kz);
	int* out = cls + (axis == 0 ? 0 : (axis == 1 ? nx : nx + ny));
	int* range = ranges + axis * 256 * 2;
	const int c = k / 2;
	int count = 0, last_lo = -1, last_hi = -1;
	for (int p = 0; p < n; ++p) {
		const int qlo = p + c - n + 1 > 0 ? p + c - n + 1 : 0;
		const int qhi = p + c < k - 1 ? p + c : k - 1;
		if (qlo != last_lo || qhi != last_hi) {
			range[2 * count] = qlo;
			range[2 * count + 1] = qhi;
			++count;
			last_lo = qlo;
			last_hi = qhi;
		}
		out[p] = count - 1;
	}
}

// Sensitivity of each class triple: the adjoint's zero-border response to an image of ones,
// every tap in raster order with FP64 fma (1 inside the class's range, 0 outside), as the
// reference's convolution_filter computes it; the adjoint tap q is PSF tap (k - 1 - q).
__global__ void noalloc_table_kernel(DevView psf, const int* ranges, int cx, int cy, int cz, float* table)
{
	const int kx = psf.ext[0], ky = psf.ext[1], kz = psf.ext[2];
	const int total = cx * cy * cz;
	for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < total; id += gridDim.x * blockDim.x) {
		const int ix = id % cx, iy = (id / cx) % cy, iz = id / (cx * cy);
		const int* rx = ranges + 0 * 512 + 2 * ix;
		const int* ry = ranges + 1 * 512 + 2 * iy;
		const int* rz = ranges + 2 * 512 + 2 * iz;
		double sum = 0.0;
		for (int qz = 0; qz < kz; ++qz) {
			for (int qy = 0; qy < ky; ++qy) {
				for (int qx = 0; qx < kx; ++qx) {
					const bool inside = qx >= rx[0] && qx <= rx[1] && qy >= ry[0] && qy <= ry[1] && qz >= rz[0] &&
						qz <= rz[1];
					const float k = *element_ptr<float>(psf, kx - 1 - qx, ky - 1 - qy, kz - 1 - qz);
					sum = fma(inside ? 1.0 : 0.0, static_cast<double>(k), sum);
				}
			}
		}
		table[id] = static_cast<float>(sum);
	}
}

}  // namespace
}  // namespace iane_gb

using namespace iane_gb;

extern "C" {

static int rl_prepare_impl(const iane_gb_view* psf, int rank, const int32_t* extent, unsigned flags, void* stream,
	iane_gb_rl_plan** out)
{
	const bool bf16 = (flags & IANE_GB_RL_BF16_TENSOR) != 0;
	if (flags & ~(IANE_GB_RL_BF16_TENSOR | IANE_GB_RL_PER_PASS)) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_prepare: unknown flags");
	}
	if (!out || !extent) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_prepare: null argument");
	}
	*out = nullptr;
	DevView k{};
	int status = normalise_view(psf, "rl_prepare psf", &k);
	if (status) return status;
	if (rank < 1 || rank > 3 || k.rank != rank) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_prepare: PSF rank must equal the image rank (1..3)");
	}
	if (k.dtype != IANE_GB_F32) {
		return fail(IANE_GB_UNSUPPORTED, "rl_prepare: the PSF must be f32");
	}
	int ext[3] = {1, 1, 1};
	for (int i = 0; i < rank; ++i) {
		if (k.ext[i] <= 0 || k.ext[i] % 2 == 0) {
			return fail(IANE_GB_INVALID_ARGUMENT, "Convolution requires positive odd kernel dimensions");
		}
		if (extent[i] < 0) {
			return fail(IANE_GB_INVALID_ARGUMENT, "rl_prepare: negative image extent");
		}
		ext[i] = extent[i];
	}
	if (k.ext[0] > 31 || k.ext[1] > 63) {
		return fail(IANE_GB_UNSUPPORTED, "rl_prepare: PSF wider than 31 along axis 0 or 63 along axis 1");
	}
	if (bf16 && k.ext[0] > 17) {
		return fail(IANE_GB_UNSUPPORTED, "rl_prepare: the BF16 tensor-core path takes PSFs up to 17 wide");
	}
	// The passes stream the PSF plane by plane through shared memory: kx <= 31 and ky <= 63
	// (checked above) bound it, kz does not.
	const long long taps = static_cast<long long>(k.ext[0]) * k.ext[1] * k.ext[2];
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	auto* plan = new iane_gb_rl_plan{};
	plan->rank = rank;
	plan->bf16 = bf16;
	plan->per_pass = (flags & IANE_GB_RL_PER_PASS) != 0;
	for (int i = 0; i < 3; ++i) {
		plan->ext[i] = ext[i];
		plan->k[i] = k.ext[i];
	}
	cudaGetDevice(&plan->device);
	auto cleanup = [&](int code) {
		iane_gb_rl_destroy(plan);
		return code;
	};
	if (cudaMalloc(&plan->d_psf, taps * sizeof(float)) != cudaSuccess ||
	    cudaMalloc(&plan->d_adj, taps * sizeof(float)) != cudaSuccess) {
		return cleanup(cuda_fail(cudaGetLastError(), "rl_prepare: allocate PSF copies"));
	}
	gather_f32_kernel<<<grid_for(taps), 256, 0, st>>>(k, plan->d_psf);
	std::vector<float> h_psf(taps), h_adj(taps);
	if (cudaMemcpyAsync(h_psf.data(), plan->d_psf, taps * sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
	    cudaStreamSynchronize(st) != cudaSuccess) {
		return cleanup(cuda_fail(cudaGetLastError(), "rl_prepare: read PSF"));
	}
	for (long long i = 0; i < taps; ++i) {
		if (!std::isfinite(h_psf[i])) {
			return cleanup(fail(IANE_GB_INVALID_ARGUMENT, "rl_prepare: PSF coefficients must be finite"));
		}
		if (bf16) {
			// the precision path convolves with the bf16-rounded PSF; everything derived
			// from it (adjoint, sensitivity) uses those same values
			h_psf[i] = __bfloat162float(__float2bfloat16_rn(h_psf[i]));
		}
	}
	for (long long i = 0; i < taps; ++i) {
		h_adj[i] = h_psf[taps - 1 - i]; // reverse_copy of the packed PSF (main.cu:106-107)
	}
	// Sensitivity = zero-border convolution of an all-ones image with the adjoint
	// (main.cu:62-64): for finite taps the out-of-range terms fma(0, k, s) leave s unchanged,
	// so each class sums its in-range taps in raster order with FP64 fma exactly as the
	// reference's convolution_filter does, then rounds to float.
	std::vector<int> cls[3];
	std::vector<std::pair<int, int>> ranges[3];
	for (int a = 0; a < 3; ++a) {
		axis_classes(ext[a], k.ext[a], cls[a], ranges[a], plan->ilo[a], plan->ihi[a]);
		plan->ccount[a] = static_cast<int>(ranges[a].size());
	}
	const long long ncls = static_cast<long long>(plan->ccount[0]) * plan->ccount[1] * plan->ccount[2];
	std::vector<float> table(ncls > 0 ? ncls : 1, 0.0f);
	plan->s_interior = 0.0f;
	for (int cz = 0; cz < plan->ccount[2]; ++cz) {
		for (int cy = 0; cy < plan->ccount[1]; ++cy) {
			for (int cx = 0; cx < plan->ccount[0]; ++cx) {
				double sum = 0.0;
				for (int qz = ranges[2][cz].first; qz <= ranges[2][cz].second; ++qz)
					for (int qy = ranges[1][cy].first; qy <= ranges[1][cy].second; ++qy)
						for (int qx = ranges[0][cx].first; qx <= ranges[0][cx].second; ++qx)
							sum = std::fma(1.0, static_cast<double>(
								h_adj[(static_cast<long long>(qz) * k.ext[1] + qy) * k.ext[0] + qx]), sum);
				const float v = static_cast<float>(sum);
				table[(static_cast<long long>(cz) * plan->ccount[1] + cy) * plan->ccount[0] + cx] = v;
				bool interior = true;
				for (int a = 0; a < 3; ++a) {
					const auto& r = ranges[a][a == 0 ? cx : (a == 1 ? cy : cz)];
					interior = interior && r.first == 0 && r.second == k.ext[a] - 1;
				}
				if (interior) plan->s_interior = v;
			}
		}
	}
	std::vector<int> all_cls;
	for (int a = 0; a < 3; ++a) all_cls.insert(all_cls.end(), cls[a].begin(), cls[a].end());
	if (cudaMalloc(&plan->d_cls, (all_cls.size() + 1) * sizeof(int)) != cudaSuccess ||
	    cudaMalloc(&plan->d_sens, table.size() * sizeof(float)) != cudaSuccess) {
		return cleanup(cuda_fail(cudaGetLastError(), "rl_prepare: allocate sensitivity tables"));
	}
	if (bf16) {
		// T_{b,qz}[k][n] = kernel[qz][b][n + rx + 8 - k], stored [qz][b][k / 8][n][k % 8] for
		// tc_conv_kernel, or [b][k / 8][qz][n][k % 8] (all planes N-contiguous) for
		// tcz_conv_kernel when they fit in its shared memory
		const int kx = k.ext[0], ky = k.ext[1], kz = k.ext[2], rx = kx / 2;
		plan->tcz = tcz_supported(kx, ky, kz);
		const size_t per = static_cast<size_t>(kTcTmatBytes / 2);
		std::vector<__nv_bfloat16> tp(static_cast<size_t>(kz) * ky * per), ta(tp.size());
		for (int qz = 0; qz < kz; ++qz)
			for (int b = 0; b < ky; ++b)
				for (int kk = 0; kk < 32; ++kk)
					for (int n = 0; n < 16; ++n) {
						const int tap = n + rx + kTcXA - kk;
						const size_t at = plan->tcz
							? ((static_cast<size_t>(b) * 4 + kk / 8) * kz + qz) * 128 + n * 8 + kk % 8
							: (static_cast<size_t>(qz) * ky + b) * per + (kk / 8) * 128 + n * 8 + kk % 8;
						const size_t src = (static_cast<size_t>(qz) * ky + b) * kx + tap;
						tp[at] = __float2bfloat16_rn(tap >= 0 && tap < kx ? h_psf[src] : 0.0f);
						ta[at] = __float2bfloat16_rn(tap >= 0 && tap < kx ? h_adj[src] : 0.0f);
					}
		if (cudaMalloc(&plan->d_tmat_psf, tp.size() * sizeof(__nv_bfloat16)) != cudaSuccess ||
		    cudaMalloc(&plan->d_tmat_adj, ta.size() * sizeof(__nv_bfloat16)) != cudaSuccess ||
		    cudaMemcpyAsync(plan->d_tmat_psf, tp.data(), tp.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, st) !=
		        cudaSuccess ||
		    cudaMemcpyAsync(plan->d_tmat_adj, ta.data(), ta.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, st) !=
		        cudaSuccess ||
		    cudaStreamSynchronize(st) != cudaSuccess) {
			return cleanup(cuda_fail(cudaGetLastError(), "rl_prepare: upload tensor-core matrices"));
		}
	}
	if (cudaMemcpyAsync(plan->d_adj, h_adj.data(), taps * sizeof(float), cudaMemcpyHostToDevice, st) != cudaSuccess ||
	    (!all_cls.empty() && cudaMemcpyAsync(plan->d_cls, all_cls.data(), all_cls.size() * sizeof(int),
	                         cudaMemcpyHostToDevice, st) != cudaSuccess) ||
	    cudaMemcpyAsync(plan->d_sens, table.data(), table.size() * sizeof(float), cudaMemcpyHostToDevice, st) !=
	        cudaSuccess ||
	    cudaStreamSynchronize(st) != cudaSuccess) {
		return cleanup(cuda_fail(cudaGetLastError(), "rl_prepare: upload tables"));
	}
	// Work-image layout and scratch size.
	plan->pitch = (static_cast<long long>(ext[0]) + 3) & ~3LL;
	plan->image_bytes = round_up(static_cast<size_t>(plan->pitch) * ext[1] * ext[2] * sizeof(float), kAlign);
	const long long big_tiles = static_cast<long long>((ext[0] + 63) / 64) * ((ext[1] + 63) / 64) * ext[2];
	plan->small_tiles = big_tiles < 2LL * device_sm_count();
	const int t = plan->small_tiles ? 32 : 64;
	plan->pass_blocks = static_cast<long long>((ext[0] + t - 1) / t) * ((ext[1] + t - 1) / t) * ext[2];
	const long long mean_blocks = 8LL * device_sm_count();
	// partials: the mean's blocks, or 3 doubles per pass B block -- two such buffers (one per
	// iteration parity) for the persistent run's statistics
	const long long stat_parts = plan->pass_blocks * 3 * (plan->small_tiles ? 1 : 2);
	plan->parts_bytes = round_up(static_cast<size_t>(
		(stat_parts > mean_blocks ? stat_parts : mean_blocks) * sizeof(double)), kAlign);
	plan->sync_bytes = round_up(rl_persist_sync_bytes(ext[2]), kAlign);
	plan->scratch_bytes = 2 * plan->image_bytes + plan->parts_bytes + 2 * kAlign + plan->sync_bytes;
	if (bf16) {
		// scratch: f32 work estimate, bf16 estimate shadow, bf16 ratio, partials, counter
		plan->pitch16 = (static_cast<long long>(ext[0]) + 7) & ~7LL;
		plan->image16_bytes = round_up(static_cast<size_t>(plan->pitch16) * ext[1] * ext[2] * 2, kAlign);
		plan->pass_blocks = plan->tcz
			? static_cast<long long>((ext[0] + 15) / 16) * ((ext[1] + kTcM - 1) / kTcM) * ((ext[2] + kTczZ - 1) / kTczZ)
			: static_cast<long long>((ext[0] + kTcN - 1) / kTcN) * ((ext[1] + kTcM - 1) / kTcM) * ext[2];
		plan->parts_bytes = round_up(static_cast<size_t>(
			(plan->pass_blocks * 3 > mean_blocks ? plan->pass_blocks * 3 : mean_blocks) * sizeof(double)), kAlign);
		plan->scratch_bytes = plan->image_bytes + 2 * plan->image16_bytes + plan->parts_bytes + 2 * kAlign;
	}
	*out = plan;
	return IANE_GB_OK;
}

int iane_gb_rl_prepare(const iane_gb_view* psf, int rank, const int32_t* extent, void* stream, iane_gb_rl_plan** out)
{
	return rl_prepare_impl(psf, rank, extent, 0u, stream, out);
}

int iane_gb_rl_prepare_ex(const iane_gb_view* psf, int rank, const int32_t* extent, unsigned flags, void* stream,
	iane_gb_rl_plan** out)
{
	return rl_prepare_impl(psf, rank, extent, flags, stream, out);
}

size_t iane_gb_rl_scratch_bytes(const iane_gb_rl_plan* plan)
{
	return plan ? plan->scratch_bytes : 0;
}

int iane_gb_rl_destroy(iane_gb_rl_plan* plan)
{
	if (!plan) {
		return IANE_GB_OK;
	}
	cudaFree(plan->d_psf);
	cudaFree(plan->d_adj);
	cudaFree(plan->d_cls);
	cudaFree(plan->d_sens);
	cudaFree(plan->d_tmat_psf);
	cudaFree(plan->d_tmat_adj);
	delete plan;
	return IANE_GB_OK;
}

int iane_gb_rl_run(iane_gb_rl_plan* plan, const iane_gb_view* observed, const iane_gb_view* estimate,
	int iterations, float epsilon, int init, void* scratch, size_t scratch_bytes, double* stats, void* stream)
{
	if (!plan) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_run: null plan");
	}
	DevView obs{}, est{};
	int status = normalise_view(observed, "rl_run observed", &obs);
	if (status) return status;
	status = normalise_view(estimate, "rl_run estimate", &est);
	if (status) return status;
	if (obs.rank != plan->rank || est.rank != plan->rank) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_run: views must have the prepared rank");
	}
	for (int i = 0; i < 3; ++i) {
		if (obs.ext[i] != plan->ext[i] || est.ext[i] != plan->ext[i]) {
			return fail(IANE_GB_INVALID_ARGUMENT, "rl_run: views must have the prepared extents");
		}
	}
	if (obs.dtype != IANE_GB_F32 && obs.dtype != IANE_GB_U8) {
		return fail(IANE_GB_UNSUPPORTED, "rl_run: observed image must be f32 or u8");
	}
	if (est.dtype != IANE_GB_F32 && est.dtype != IANE_GB_U8) {
		return fail(IANE_GB_UNSUPPORTED, "rl_run: estimate must be f32 or u8");
	}
	if (iterations < 0 || !(epsilon > 0.0f) || !std::isfinite(epsilon)) {
		return fail(IANE_GB_INVALID_ARGUMENT, "Iterations and finite epsilon must be positive");
	}
	if (init < IANE_GB_RL_INIT_OBSERVED || init > IANE_GB_RL_INIT_GIVEN) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_run: unknown init mode");
	}
	if (init == IANE_GB_RL_INIT_GIVEN && est.dtype != IANE_GB_F32) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_run: a given start needs an f32 estimate");
	}
	if (!scratch || scratch_bytes < plan->scratch_bytes) {
		return fail(IANE_GB_LENGTH_ERROR, "Prepared operation exceeded its scratch reservation");
	}
	if (element_count(obs) == 0) {
		return IANE_GB_OK;
	}
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	char* base = reinterpret_cast<char*>(round_up(reinterpret_cast<uintptr_t>(scratch), kAlign));
	if (base + (plan->scratch_bytes - kAlign) > static_cast<char*>(scratch) + scratch_bytes) {
		return fail(IANE_GB_LENGTH_ERROR, "Prepared operation exceeded its scratch reservation");
	}
	if (plan->bf16) {
		return rl_run_bf16(plan, obs, est, iterations, epsilon, init, base, stats, static_cast<cudaStream_t>(stream));
	}
	float* ratio = reinterpret_cast<float*>(base);
	float* work = reinterpret_cast<float*>(base + plan->image_bytes);
	double* parts = reinterpret_cast<double*>(base + 2 * plan->image_bytes);
	unsigned int* counter = reinterpret_cast<unsigned int*>(base + 2 * plan->image_bytes + plan->parts_bytes);
	float* start = reinterpret_cast<float*>(counter + 1);
	const int nx = plan->ext[0], ny = plan->ext[1], nz = plan->ext[2];
	const long long pitch = plan->pitch, plane = pitch * ny;
	const bool in_place = is_work_layout(est, pitch);
	float* e_work = in_place ? reinterpret_cast<float*>(est.ptr) : work;
	const long long n = static_cast<long long>(nx) * ny * nz;

	IANE_GB_CUDA(cudaMemsetAsync(counter, 0, 2 * sizeof(unsigned int), st), "rl_run: clear counter");
	if (init == IANE_GB_RL_INIT_GIVEN) {
		if (!in_place) {
			rl_copy_kernel<<<grid_for(n), 256, 0, st>>>(e_work, pitch, plane, est, 0);
		}
	} else {
		if (init == IANE_GB_RL_INIT_MEAN) {
			rl_mean_kernel<<<grid_for(n), 256, 0, st>>>(obs, parts, counter, start, epsilon);
		}
		rl_init_kernel<<<grid_for(n), 256, 0, st>>>(obs, e_work, pitch, plane, epsilon, init, start);
	}
	IANE_GB_CUDA(cudaGetLastError(), "rl_run: launch init");

	int* dstatus = device_status_ptr();
	if (!dstatus) return IANE_GB_CUDA_ERROR;
	const int kx = plan->k[0];
	// Tile shape of the launches below: (1, 1) warps for small images, else (2, 2).
	const int wx = plan->small_tiles ? 1 : 2;
	const int wy = wx;
	const int box_w = tile_pitch(kx, wx);
	const int box_h = 32 * wy + 2 * (plan->k[1] / 2);
	CUtensorMap map_est{}, map_ratio{};
	status = encode_tensor_map_f32(&map_est, e_work, nx, ny, nz, pitch * 4, plane * 4, box_w, box_h);
	if (status) return status;
	status = encode_tensor_map_f32(&map_ratio, ratio, nx, ny, nz, pitch * 4, plane * 4, box_w, box_h);
	if (status) return status;

	TileArgs ta{};
	ta.nx = nx;
	ta.ny = ny;
	ta.nz = nz;
	ta.ky = plan->k[1];
	ta.kz = plan->k[2];
	ta.k_stride[0] = 4;
	ta.k_stride[1] = 4LL * plan->k[0];
	ta.k_stride[2] = 4LL * plan->k[0] * plan->k[1];
	ta.border = IANE_GB_BORDER_ZERO;
	ta.status = dstatus;
	TileArgs tb = ta;
	ta.kernel = reinterpret_cast<const char*>(plan->d_psf);
	tb.kernel = reinterpret_cast<const char*>(plan->d_adj);

	EpiRatio ea{};
	ea.ratio = ratio;
	ea.pitch = pitch;
	ea.plane = plane;
	ea.obs = obs.ptr;
	for (int i = 0; i < 3; ++i) ea.os[i] = obs.stride[i];
	ea.obs_u8 = obs.dtype == IANE_GB_U8;
	ea.eps = epsilon;
	ea.nx = nx;
	ea.ny = ny;

	EpiUpdate eb{};
	eb.est = e_work;
	eb.pitch = pitch;
	eb.plane = plane;
	eb.eps = epsilon;
	eb.nx = nx;
	eb.ny = ny;
	eb.nz = nz;
	eb.cls = plan->d_cls;
	eb.sens = plan->d_sens;
	eb.cx_count = plan->ccount[0];
	eb.cy_count = plan->ccount[1];
	for (int i = 0; i < 3; ++i) {
		eb.ilo[i] = plan->ilo[i];
		eb.ihi[i] = plan->ihi[i];
		eb.outs[i] = est.stride[i];
	}
	eb.s_interior = plan->s_interior;
	eb.partials = parts;
	eb.counter = counter;
	eb.out = est.ptr;
	eb.out_u8 = est.dtype == IANE_GB_U8;

	// One persistent launch for the whole run (rl_persist.cuh) unless the image is small enough for
	// 32 x 32 tiles or the plan asks for one launch per pass.
	const long long tiles_x = (nx + 63) / 64, tiles_y = (ny + 63) / 64;
	const bool persistent = !plan->per_pass && !plan->small_tiles && iterations > 0 &&
		tiles_x * tiles_y * nz * 2LL * iterations < (1LL << 31);
	if (persistent) {
		unsigned int* sync = reinterpret_cast<unsigned int*>(base + 2 * plan->image_bytes + plan->parts_bytes + kAlign);
		RlPersistArgs pa{};
		pa.map_est = map_est;
		pa.map_ratio = map_ratio;
		pa.pass_a = ta;
		pa.pass_b = tb;
		pa.epi_a = ea;
		eb.want_stats = 0;
		eb.stats = nullptr;
		eb.write_out = in_place ? 0 : 1;
		pa.epi_b = eb;
		pa.tiles_x = static_cast<int>(tiles_x);
		pa.tiles_y = static_cast<int>(tiles_y);
		pa.nz = nz;
		pa.phases = 2 * iterations;
		pa.queue = sync;
		pa.abort = reinterpret_cast<int*>(sync + 1);
		pa.done = sync + 2;
		pa.parts = parts;
		pa.stats = stats;
		pa.stat_count = sync + 2 + nz;
		pa.stat_done = sync + 4 + nz;
		IANE_GB_CUDA(cudaMemsetAsync(sync, 0, rl_persist_sync_bytes(nz), st), "rl_run: clear queue");
		return launch_rl_persist(kx, pa, st);
	}
	for (int it = 0; it < iterations; ++it) {
		status = launch_rl_pass_a(kx, plan->small_tiles, map_est, ta, ea, st);
		if (status) return status;
		eb.want_stats = stats != nullptr;
		eb.stats = stats ? stats + 2 * it : nullptr;
		eb.write_out = (!in_place && it == iterations - 1) ? 1 : 0;
		status = launch_rl_pass_b(kx, plan->small_tiles, map_ratio, tb, eb, st);
		if (status) return status;
	}
	if (iterations == 0 && !in_place) {
		rl_copy_kernel<<<grid_for(n), 256, 0, st>>>(e_work, pitch, plane, est, 1);
		IANE_GB_CUDA(cudaGetLastError(), "rl_run: launch copy-out");
	}
	return IANE_GB_OK;
}

size_t iane_gb_rl_host_scratch_bytes(const iane_gb_rl_plan* plan, int observed_dtype)
{
	if (!plan) return 0;
	const size_t n = static_cast<size_t>(plan->ext[0]) * plan->ext[1] * plan->ext[2];
	const size_t obs = round_up(n * (observed_dtype == IANE_GB_U8 ? 1 : 4), kAlign);
	const size_t est = round_up(static_cast<size_t>(plan->pitch) * plan->ext[1] * plan->ext[2] * 4, kAlign);
	return plan->scratch_bytes + obs + est + kAlign;
}

int iane_gb_rl_run_host(iane_gb_rl_plan* plan, const void* host_observed, int observed_dtype, float* host_estimate,
	int iterations, float epsilon, int init, void* scratch, size_t scratch_bytes, void* stream)
{
	if (!plan || !host_observed || !host_estimate) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_run_host: null argument");
	}
	if (observed_dtype != IANE_GB_U8 && observed_dtype != IANE_GB_F32) {
		return fail(IANE_GB_UNSUPPORTED, "rl_run_host: observed image must be f32 or u8");
	}
	if (!scratch || scratch_bytes < iane_gb_rl_host_scratch_bytes(plan, observed_dtype)) {
		return fail(IANE_GB_LENGTH_ERROR, "Prepared operation exceeded its scratch reservation");
	}
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	const int nx = plan->ext[0], ny = plan->ext[1], nz = plan->ext[2];
	const size_t n = static_cast<size_t>(nx) * ny * nz;
	const int esize = observed_dtype == IANE_GB_U8 ? 1 : 4;
	char* base = reinterpret_cast<char*>(round_up(reinterpret_cast<uintptr_t>(scratch), kAlign));
	char* d_obs = base + plan->scratch_bytes;
	float* d_est = reinterpret_cast<float*>(d_obs + round_up(n * esize, kAlign));
	const long long pitch = plan->pitch;
	iane_gb_view ov{}, ev{};
	ov.ptr = d_obs;
	ov.dtype = observed_dtype;
	ov.rank = plan->rank;
	ev.ptr = d_est;
	ev.dtype = IANE_GB_F32;
	ev.rank = plan->rank;
	long long s = esize;
	for (int i = 0; i < plan->rank; ++i) {
		ov.extent[i] = ev.extent[i] = plan->ext[i];
		ov.stride[i] = s;
		s *= plan->ext[i];
	}
	ev.stride[0] = 4;
	ev.stride[1] = pitch * 4;
	ev.stride[2] = pitch * 4 * ny;
	IANE_GB_CUDA(cudaMemcpyAsync(d_obs, host_observed, n * esize, cudaMemcpyHostToDevice, st), "rl_run_host: upload");
	if (init == IANE_GB_RL_INIT_GIVEN) {
		IANE_GB_CUDA(cudaMemcpy2DAsync(d_est, pitch * 4, host_estimate, nx * 4, nx * 4, static_cast<size_t>(ny) * nz,
			cudaMemcpyHostToDevice, st), "rl_run_host: upload start");
	}
	const int status = iane_gb_rl_run(plan, &ov, &ev, iterations, epsilon, init, base, plan->scratch_bytes, nullptr,
		stream);
	if (status) return status;
	IANE_GB_CUDA(cudaMemcpy2DAsync(host_estimate, nx * 4, d_est, pitch * 4, nx * 4, static_cast<size_t>(ny) * nz,
		cudaMemcpyDeviceToHost, st), "rl_run_host: download");
	IANE_GB_CUDA(cudaStreamSynchronize(st), "rl_run_host: wait");
	return IANE_GB_OK;
}


int iane_gb_rl_run_noalloc(const iane_gb_view* psf, const iane_gb_view* observed, const iane_gb_view* estimate,
	int iterations, float epsilon, int init, void* stream)
{
	DevView k{}, obs{}, est{};
	int status = normalise_view(psf, "rl_run_noalloc psf", &k);
	if (status) return status;
	status = normalise_view(observed, "rl_run_noalloc observed", &obs);
	if (status) return status;
	status = normalise_view(estimate, "rl_run_noalloc estimate", &est);
	if (status) return status;
	if (k.rank != obs.rank || est.rank != obs.rank) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_run_noalloc: PSF, observed and estimate need the same rank");
	}
	for (int i = 0; i < 3; ++i) {
		if (est.ext[i] != obs.ext[i]) {
			return fail(IANE_GB_INVALID_ARGUMENT, "Source and destination require matching nonnegative dimensions");
		}
		if (i < k.rank && (k.ext[i] <= 0 || k.ext[i] % 2 == 0)) {
			return fail(IANE_GB_INVALID_ARGUMENT, "Convolution requires positive odd kernel dimensions");
		}
	}
	if (k.dtype != IANE_GB_F32) {
		return fail(IANE_GB_UNSUPPORTED, "rl_run_noalloc: the PSF must be f32");
	}
	if (obs.dtype != IANE_GB_F32 && obs.dtype != IANE_GB_U8) {
		return fail(IANE_GB_UNSUPPORTED, "rl_run_noalloc: observed image must be f32 or u8");
	}
	if (est.dtype != IANE_GB_F32 && est.dtype != IANE_GB_U8) {
		return fail(IANE_GB_UNSUPPORTED, "rl_run_noalloc: estimate must be f32 or u8");
	}
	if (iterations < 0 || !(epsilon > 0.0f) || !std::isfinite(epsilon)) {
		return fail(IANE_GB_INVALID_ARGUMENT, "Iterations and finite epsilon must be positive");
	}
	if (init < IANE_GB_RL_INIT_OBSERVED || init > IANE_GB_RL_INIT_GIVEN ||
	    (init == IANE_GB_RL_INIT_GIVEN && est.dtype != IANE_GB_F32)) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_run_noalloc: unknown init mode or a given start without f32");
	}
	const int nx = obs.ext[0], ny = obs.ext[1], nz = obs.ext[2];
	const long long pitch = (static_cast<long long>(nx) + 3) & ~3LL, plane = pitch * ny;
	const long long taps = static_cast<long long>(k.ext[0]) * k.ext[1] * k.ext[2];
	if (pitch * ny * nz > kNoAllocMaxVoxels || static_cast<long long>(nx) + ny + nz > kNoAllocMaxAxisSum) {
		return fail(IANE_GB_LENGTH_ERROR, "rl_run_noalloc: image larger than the static scratch (at most 4194304 "
			"voxels with rows padded to a multiple of 4, and nx + ny + nz <= 65536)");
	}
	if (k.ext[0] > 31 || k.ext[1] > kNoAllocMaxExtent || k.ext[2] > kNoAllocMaxExtent || taps > kNoAllocMaxTaps) {
		return fail(IANE_GB_LENGTH_ERROR, "rl_run_noalloc: PSF larger than the static scratch allows (width <= 31, "
			"height and depth <= 63, at most 32768 taps)");
	}
	if (element_count(obs) == 0) {
		return IANE_GB_OK;
	}
	char* base = noalloc_scratch();
	if (!base) return IANE_GB_CUDA_ERROR;
	int* dstatus = device_status_ptr();
	if (!dstatus) return IANE_GB_CUDA_ERROR;
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	float* ratio = reinterpret_cast<float*>(base);
	float* work = reinterpret_cast<float*>(base + kNoAllocImageBytes);
	int* cls = reinterpret_cast<int*>(base + kNoAllocClsOffset);
	float* table = reinterpret_cast<float*>(base + kNoAllocTableOffset);
	int* ranges = reinterpret_cast<int*>(base + kNoAllocRangeOffset);
	double* parts = reinterpret_cast<double*>(base + kNoAllocPartsOffset);
	unsigned int* counter = reinterpret_cast<unsigned int*>(base + kNoAllocCounterOffset);
	float* start = reinterpret_cast<float*>(counter + 1);
	const bool in_place = is_work_layout(est, pitch);
	float* e_work = in_place ? reinterpret_cast<float*>(est.ptr) : work;
	const long long n = static_cast<long long>(nx) * ny * nz;
	const int ccount[3] = {count_classes(nx, k.ext[0]), count_classes(ny, k.ext[1]), count_classes(nz, k.ext[2])};

	// The array keeps the previous call's contents: reset the completion counter.
	IANE_GB_CUDA(cudaMemsetAsync(counter, 0, 2 * sizeof(unsigned int), st), "rl_run_noalloc: clear counter");
	noalloc_classes_kernel<<<1, 32, 0, st>>>(nx, ny, nz, k.ext[0], k.ext[1], k.ext[2], cls, ranges);
	const int classes = ccount[0] * ccount[1] * ccount[2];
	noalloc_table_kernel<<<(classes + 127) / 128, 128, 0, st>>>(k, ranges, ccount[0], ccount[1], ccount[2], table);
	IANE_GB_CUDA(cudaGetLastError(), "rl_run_noalloc: launch table kernels");
	if (init == IANE_GB_RL_INIT_GIVEN) {
		if (!in_place) {
			rl_copy_kernel<<<grid_for(n), 256, 0, st>>>(e_work, pitch, plane, est, 0);
		}
	} else {
		if (init == IANE_GB_RL_INIT_MEAN) {
			// one partial per block in a region of kNoAllocMaxPartials doubles; the kernel's
			// grid-stride loop covers the image with any grid
			const int mean_grid = grid_for(n) < kNoAllocMaxPartials ? grid_for(n) : kNoAllocMaxPartials;
			rl_mean_kernel<<<mean_grid, 256, 0, st>>>(obs, parts, counter, start, epsilon);
		}
		rl_init_kernel<<<grid_for(n), 256, 0, st>>>(obs, e_work, pitch, plane, epsilon, init, start);
	}
	IANE_GB_CUDA(cudaGetLastError(), "rl_run_noalloc: launch init");

	const long long big_tiles = static_cast<long long>((nx + 63) / 64) * ((ny + 63) / 64) * nz;
	const bool small = big_tiles < 2LL * device_sm_count();
	const int kx = k.ext[0];
	const int wx = small ? 1 : 2;
	const int wy = wx;
	CUtensorMap map_est{}, map_ratio{};
	status = encode_tensor_map_f32(&map_est, e_work, nx, ny, nz, pitch * 4, plane * 4, tile_pitch(kx, wx),
		32 * wy + 2 * (k.ext[1] / 2));
	if (status) return status;
	status = encode_tensor_map_f32(&map_ratio, ratio, nx, ny, nz, pitch * 4, plane * 4, tile_pitch(kx, wx),
		32 * wy + 2 * (k.ext[1] / 2));
	if (status) return status;

	TileArgs ta{};
	ta.nx = nx;
	ta.ny = ny;
	ta.nz = nz;
	ta.ky = k.ext[1];
	ta.kz = k.ext[2];
	ta.border = IANE_GB_BORDER_ZERO;
	ta.status = dstatus;
	TileArgs tb = ta;
	// pass A reads the caller's PSF view as given; pass B reads it backwards along every
	// axis, which is the adjoint, without a copy
	ta.kernel = k.ptr;
	tb.kernel = k.ptr + (k.ext[0] - 1) * k.stride[0] + (k.ext[1] - 1) * k.stride[1] + (k.ext[2] - 1) * k.stride[2];
	for (int i = 0; i < 3; ++i) {
		ta.k_stride[i] = k.stride[i];
		tb.k_stride[i] = -k.stride[i];
	}
	EpiRatio ea{};
	ea.ratio = ratio;
	ea.pitch = pitch;
	ea.plane = plane;
	ea.obs = obs.ptr;
	for (int i = 0; i < 3; ++i) ea.os[i] = obs.stride[i];
	ea.obs_u8 = obs.dtype == IANE_GB_U8;
	ea.eps = epsilon;
	ea.nx = nx;
	ea.ny = ny;
	EpiUpdate eb{};
	eb.est = e_work;
	eb.pitch = pitch;
	eb.plane = plane;
	eb.eps = epsilon;
	eb.nx = nx;
	eb.ny = ny;
	eb.nz = nz;
	eb.cls = cls;
	eb.sens = table;
	eb.cx_count = ccount[0];
	eb.cy_count = ccount[1];
	for (int i = 0; i < 3; ++i) {
		eb.ilo[i] = 1; // no interior shortcut: every voxel reads its class's table entry
		eb.ihi[i] = 0;
		eb.outs[i] = est.stride[i];
	}
	eb.out = est.ptr;
	eb.out_u8 = est.dtype == IANE_GB_U8;
	for (int it = 0; it < iterations; ++it) {
		status = launch_rl_pass_a(kx, small, map_est, ta, ea, st);
		if (status) return status;
		eb.write_out = (!in_place && it == iterations - 1) ? 1 : 0;
		status = launch_rl_pass_b(kx, small, map_ratio, tb, eb, st);
		if (status) return status;
	}
	if (iterations == 0 && !in_place) {
		rl_copy_kernel<<<grid_for(n), 256, 0, st>>>(e_work, pitch, plane, est, 1);
		IANE_GB_CUDA(cudaGetLastError(), "rl_run_noalloc: launch copy-out");
	}
	return IANE_GB_OK;
}

}  // extern "C"
