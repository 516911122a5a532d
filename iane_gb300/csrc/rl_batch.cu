// Batched Richardson-Lucy: plans, autotuned tile shapes, the CUDA-graph schedule and the
// C-ABI entry points iane_gb_rl_batch_*. See rl_batch.cuh for the execution design.
#include "kernels.h"
#include "rl_batch.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

namespace iane_gb {
namespace {

constexpr size_t kAlignB = 256;
constexpr int kMaxBatchIterations = 4096;
inline size_t align_up(size_t v) { return (v + kAlignB - 1) / kAlignB * kAlignB; }

// Per-image description for the batched start-value kernels.
struct InitDesc {
	DevView obs;
	DevView est;
	float* work;
	long long pitch;
	int in_place;
};

__global__ void batch_mean_kernel(const InitDesc* d, float* starts, float eps)
{
	const InitDesc& im = d[blockIdx.x];
	const int nx = im.obs.ext[0], ny = im.obs.ext[1];
	const long long n = static_cast<long long>(nx) * ny;
	double s = 0.0;
	for (long long i = threadIdx.x; i < n; i += blockDim.x) {
		const int x = static_cast<int>(i % nx), y = static_cast<int>(i / nx);
		const char* p = im.obs.ptr + x * im.obs.stride[0] + y * im.obs.stride[1];
		s += im.obs.dtype == IANE_GB_U8 ? static_cast<double>(*reinterpret_cast<const uint8_t*>(p))
			: static_cast<double>(*reinterpret_cast<const float*>(p));
	}
	__shared__ double red[32];
	for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
	__syncthreads();
	if (threadIdx.x == 0) {
		double t = 0.0;
		for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += red[w];
		const float mean = static_cast<float>(t / static_cast<double>(n > 0 ? n : 1));
		starts[blockIdx.x] = mean > eps ? mean : eps;
	}
}

// mode: RL start mode, or -1 = copy the work estimate out to the caller's view.
__global__ void batch_init_kernel(const InitDesc* d, const float* starts, float eps, int mode)
{
	const InitDesc& im = d[blockIdx.x];
	const int nx = im.obs.ext[0], ny = im.obs.ext[1];
	const long long n = static_cast<long long>(nx) * ny;
	for (long long i = blockIdx.y * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
	     i += static_cast<long long>(gridDim.y) * blockDim.x) {
		const int x = static_cast<int>(i % nx), y = static_cast<int>(i / nx);
		float& w = im.work[y * im.pitch + x];
		char* e = im.est.ptr + x * im.est.stride[0] + y * im.est.stride[1];
		if (mode < 0) {
			if (!im.in_place) {
				if (im.est.dtype == IANE_GB_U8) {
					*reinterpret_cast<uint8_t*>(e) = to_gray8(w);
				} else {
					*reinterpret_cast<float*>(e) = w;
				}
			}
		} else if (mode == IANE_GB_RL_INIT_GIVEN) {
			if (!im.in_place) w = *reinterpret_cast<const float*>(e);
		} else if (mode == IANE_GB_RL_INIT_MEAN) {
			w = starts[blockIdx.x];
		} else {
			const char* p = im.obs.ptr + x * im.obs.stride[0] + y * im.obs.stride[1];
			const float o = im.obs.dtype == IANE_GB_U8 ? static_cast<float>(*reinterpret_cast<const uint8_t*>(p))
				: *reinterpret_cast<const float*>(p);
			w = o > eps ? o : eps;
		}
	}
}

int occupancy_grid(int wx, bool wide, size_t smem, size_t items);

bool work_layout(const DevView& v, long long pitch)
{
	if (v.dtype != IANE_GB_F32 || v.stride[0] != 4 || reinterpret_cast<uintptr_t>(v.ptr) % 16 != 0) return false;
	if (v.ext[1] > 1 && v.stride[1] != pitch * 4) return false;
	return true;
}

// ---------------------------------------------------------------------------------------
// autotuner: tile shape per (shape, PSF size, dtype, SM count), cached in a text file

struct TuneCache {
	std::mutex lock;
	bool loaded = false;
	std::map<std::string, int> choice;
	std::string path;
};

TuneCache& tune_cache()
{
	static TuneCache c;
	return c;
}

std::string cache_path()
{
	if (const char* p = std::getenv("IANE_GB_TUNE_CACHE")) return p;
	if (const char* h = std::getenv("HOME")) return std::string(h) + "/.cache/iane_gb300_tune.txt";
	return "iane_gb300_tune.txt";
}

std::string tune_key(int nx, int ny, int kx, int ky)
{
	std::ostringstream k;
	k << "rl2d-classes f32 " << nx << "x" << ny << " psf " << kx << "x" << ky << " sms " << device_sm_count();
	return k.str();
}

void load_cache(TuneCache& c)
{
	if (c.loaded) return;
	c.loaded = true;
	c.path = cache_path();
	std::ifstream in(c.path);
	std::string line;
	while (std::getline(in, line)) {
		// "<key> | <ms 32x32> <ms 64x64> |<choice>"
		const auto first = line.find(" | ");
		const auto last = line.rfind('|');
		if (first == std::string::npos || last == std::string::npos || last <= first + 1) continue;
		const int wx = std::atoi(line.c_str() + last + 1);
		if (wx == 1 || wx == 2) c.choice[line.substr(0, first)] = wx;
	}
}

}  // namespace

int batch_autotune(const std::vector<int>& nx, const std::vector<int>& ny, const std::vector<int>& kx,
	const std::vector<int>& ky, const std::vector<iane_gb_rl_plan*>& plans, std::vector<int>& wx, cudaStream_t stream)
{
	TuneCache& cache = tune_cache();
	std::lock_guard<std::mutex> guard(cache.lock);
	load_cache(cache);
	int* status = device_status_ptr();
	if (!status) return IANE_GB_CUDA_ERROR;
	const int n = static_cast<int>(nx.size());
	std::vector<int> todo;
	for (int i = 0; i < n; ++i) {
		const auto it = cache.choice.find(tune_key(nx[i], ny[i], kx[i], ky[i]));
		if (it != cache.choice.end()) {
			wx[i] = it->second;
		} else {
			todo.push_back(i);
		}
	}
	if (todo.empty()) return IANE_GB_OK;
	const int sms = device_sm_count();
	size_t max_bytes = 0;
	for (int i : todo) {
		max_bytes = std::max(max_bytes, align_up(static_cast<size_t>((nx[i] + 3) & ~3) * ny[i] * 4));
	}
	const int max_copies = 256;
	char* buf = nullptr;
	BatchImage* d_images = nullptr;
	BatchItem* d_items = nullptr;
	unsigned int* counter = nullptr;
	const size_t max_items = 1 << 16;
	cudaEvent_t t0 = nullptr, t1 = nullptr;
	auto release = [&](int code) {
		cudaFree(buf);
		cudaFree(d_images);
		cudaFree(d_items);
		cudaFree(counter);
		if (t0) cudaEventDestroy(t0);
		if (t1) cudaEventDestroy(t1);
		return code;
	};
	if (cudaMalloc(&buf, 3 * max_bytes) != cudaSuccess || cudaMemsetAsync(buf, 0, 3 * max_bytes, stream) != cudaSuccess ||
	    cudaMalloc(&d_images, max_copies * sizeof(BatchImage)) != cudaSuccess ||
	    cudaMalloc(&d_items, max_items * sizeof(BatchItem)) != cudaSuccess ||
	    cudaMalloc(&counter, 8 * sizeof(unsigned int)) != cudaSuccess || cudaEventCreate(&t0) != cudaSuccess ||
	    cudaEventCreate(&t1) != cudaSuccess) {
		return release(cuda_fail(cudaGetLastError(), "autotune: allocate"));
	}
	std::ofstream log(cache.path, std::ios::app);
	for (int i : todo) {
		const std::string key = tune_key(nx[i], ny[i], kx[i], ky[i]);
		if (cache.choice.count(key)) {
			wx[i] = cache.choice[key];
			continue;
		}
		const long long pitch = (static_cast<long long>(nx[i]) + 3) & ~3LL, plane = pitch * ny[i];
		float ms[2] = {0.0f, 0.0f};
		for (int w = 1; w <= 2; ++w) {
			const int t = 32 * w;
			const int tiles = ((nx[i] + t - 1) / t) * ((ny[i] + t - 1) / t);
			// enough copies of this image's tiles to occupy every SM several times over
			const int copies = std::min(max_copies, std::max(1, (8 * sms + tiles - 1) / tiles));
			std::vector<BatchImage> host(copies);
			BatchImage im{};
			int st = encode_tensor_map_f32(&im.map_est, buf, nx[i], ny[i], 1, pitch * 4, plane * 4, tile_pitch(kx[i], w),
				t + 2 * (ky[i] / 2));
			if (st) return release(st);
			im.map_ratio = im.map_est;
			rl_plan_fill_passes(plans[i], &im.pass_a, &im.pass_b, &im.epi_a, &im.epi_b, status);
			im.epi_a.ratio = reinterpret_cast<float*>(buf + max_bytes);
			im.epi_a.obs = buf + 2 * max_bytes;
			im.epi_a.os[0] = 4;
			im.epi_a.os[1] = pitch * 4;
			im.epi_a.eps = 1e-6f;
			im.kx = kx[i];
			im.tiles_x = (nx[i] + t - 1) / t;
			for (auto& h : host) h = im;
			std::vector<BatchItem> items;
			for (int c = 0; c < copies && static_cast<size_t>(items.size()) + tiles <= max_items; ++c)
				for (int k = 0; k < tiles; ++k) items.push_back(BatchItem{c, k});
			if (cudaMemcpy(d_images, host.data(), copies * sizeof(BatchImage), cudaMemcpyHostToDevice) != cudaSuccess ||
			    cudaMemcpy(d_items, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice) != cudaSuccess) {
				return release(cuda_fail(cudaGetLastError(), "autotune: upload"));
			}
			const size_t smem = batch_tile_smem(w, kx[i], ky[i]);
			const int grid = occupancy_grid(w, batch_wide(kx[i]), smem, items.size());
			for (int rep = 0; rep < 4; ++rep) {
				if (rep == 1) cudaEventRecord(t0, stream);
				cudaMemsetAsync(counter, 0, sizeof(unsigned int), stream);
				st = launch_batch_pass(w, batch_wide(kx[i]), false, d_images, d_items, static_cast<int>(items.size()), counter, 0, grid, smem,
					stream);
				if (st) return release(st);
			}
			cudaEventRecord(t1, stream);
			IANE_GB_CUDA(cudaEventSynchronize(t1), "autotune: time");
			float elapsed = 0.0f;
			cudaEventElapsedTime(&elapsed, t0, t1);
			ms[w - 1] = elapsed / (3.0f * static_cast<float>(items.size() / tiles));
		}
		wx[i] = ms[0] < ms[1] ? 1 : 2;
		cache.choice[key] = wx[i];
		if (log) log << key << " | " << ms[0] << " " << ms[1] << " |" << wx[i] << "\n";
	}
	return release(IANE_GB_OK);
}

}  // namespace iane_gb

struct iane_gb_rl_batch {
	int count = 0;
	std::vector<iane_gb_rl_plan*> plans;
	std::vector<int> nx, ny, kx, ky, wx;
	std::vector<long long> pitch;
	std::vector<size_t> off;               // per image: ratio at off, work at off + image bytes
	std::vector<size_t> img_bytes;
	// per group (batch_group: 32x32 / 64x64 tiles x narrow / wide PSFs)
	std::vector<iane_gb::BatchItem> items[iane_gb::kBatchGroups];
	iane_gb::BatchItem* d_items[iane_gb::kBatchGroups] = {};
	size_t smem[iane_gb::kBatchGroups] = {};
	int grid[iane_gb::kBatchGroups] = {};
	iane_gb::BatchImage* d_images = nullptr;
	iane_gb::InitDesc* d_init = nullptr;
	size_t parts_off = 0, counter_off = 0, scratch_bytes = 0;
	cudaStream_t side[iane_gb::kBatchGroups] = {};  // side[0] carries the capture
	cudaEvent_t fork = nullptr;
	cudaEvent_t join[iane_gb::kBatchGroups] = {};
	cudaGraphExec_t exec = nullptr;
	std::string key;
};

namespace iane_gb {
namespace {

// Build descriptors for one run and the graph that performs it.
int build_graph(iane_gb_rl_batch* b, const DevView* obs, const DevView* est, int iterations, float eps, int init,
	char* base)
{
	const int n = b->count;
	std::vector<BatchImage> host(n);
	std::vector<InitDesc> idesc(n);
	int* status = device_status_ptr();
	if (!status) return IANE_GB_CUDA_ERROR;
	for (int i = 0; i < n; ++i) {
		const iane_gb_rl_plan* p = b->plans[i];
		(void)p;
		const int nx = b->nx[i], ny = b->ny[i], kxi = b->kx[i], kyi = b->ky[i], w = b->wx[i];
		const long long pitch = b->pitch[i], plane = pitch * ny;
		float* ratio = reinterpret_cast<float*>(base + b->off[i]);
		float* work = reinterpret_cast<float*>(base + b->off[i] + b->img_bytes[i]);
		const bool in_place = work_layout(est[i], pitch);
		float* e_work = in_place ? reinterpret_cast<float*>(est[i].ptr) : work;
		BatchImage& im = host[i];
		std::memset(&im, 0, sizeof im);
		int st = encode_tensor_map_f32(&im.map_est, e_work, nx, ny, 1, pitch * 4, plane * 4, tile_pitch(kxi, w),
			32 * w + 2 * (kyi / 2));
		if (st) return st;
		st = encode_tensor_map_f32(&im.map_ratio, ratio, nx, ny, 1, pitch * 4, plane * 4, tile_pitch(kxi, w),
			32 * w + 2 * (kyi / 2));
		if (st) return st;
		rl_plan_fill_passes(b->plans[i], &im.pass_a, &im.pass_b, &im.epi_a, &im.epi_b, status);
		im.epi_a.ratio = ratio;
		im.epi_a.obs = obs[i].ptr;
		for (int a = 0; a < 3; ++a) im.epi_a.os[a] = obs[i].stride[a];
		im.epi_a.obs_u8 = obs[i].dtype == IANE_GB_U8;
		im.epi_a.eps = eps;
		im.epi_b.est = e_work;
		im.epi_b.eps = eps;
		im.epi_b.out = est[i].ptr;
		for (int a = 0; a < 3; ++a) im.epi_b.outs[a] = est[i].stride[a];
		im.epi_b.out_u8 = est[i].dtype == IANE_GB_U8;
		im.kx = kxi;
		im.tiles_x = (nx + 32 * w - 1) / (32 * w);
		im.write_out_final = in_place ? 0 : 1;
		idesc[i].obs = obs[i];
		idesc[i].est = est[i];
		idesc[i].work = e_work;
		idesc[i].pitch = pitch;
		idesc[i].in_place = in_place ? 1 : 0;
	}
	IANE_GB_CUDA(cudaMemcpy(b->d_images, host.data(), n * sizeof(BatchImage), cudaMemcpyHostToDevice),
		"batch: upload image descriptors");
	IANE_GB_CUDA(cudaMemcpy(b->d_init, idesc.data(), n * sizeof(InitDesc), cudaMemcpyHostToDevice),
		"batch: upload start descriptors");

	double* parts = reinterpret_cast<double*>(base + b->parts_off);
	float* starts = reinterpret_cast<float*>(parts);
	unsigned int* counters = reinterpret_cast<unsigned int*>(base + b->counter_off);
	cudaStream_t s0 = b->side[0];
	cudaGraph_t graph = nullptr;
	IANE_GB_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal), "batch: begin capture");
	auto abort_capture = [&](int code) {
		cudaGraph_t g = nullptr;
		cudaStreamEndCapture(s0, &g);
		if (g) cudaGraphDestroy(g);
		return code;
	};
	if (cudaMemsetAsync(counters, 0, static_cast<size_t>(2 * kBatchGroups * (iterations + 1)) * sizeof(unsigned int),
	        s0) != cudaSuccess) {
		return abort_capture(cuda_fail(cudaGetLastError(), "batch: clear counters"));
	}
	if (init == IANE_GB_RL_INIT_MEAN) {
		batch_mean_kernel<<<n, 256, 0, s0>>>(b->d_init, starts, eps);
	}
	batch_init_kernel<<<dim3(n, 16), 256, 0, s0>>>(b->d_init, starts, eps, init);
	for (int t = 0; t < iterations; ++t) {
		for (int pass = 0; pass < 2; ++pass) {
			unsigned int* c = counters + 2 * kBatchGroups * t + kBatchGroups * pass;
			if (cudaEventRecord(b->fork, s0) != cudaSuccess) {
				return abort_capture(cuda_fail(cudaGetLastError(), "batch: fork"));
			}
			for (int g = 1; g < kBatchGroups; ++g) {
				if (!b->items[g].empty() && cudaStreamWaitEvent(b->side[g], b->fork, 0) != cudaSuccess) {
					return abort_capture(cuda_fail(cudaGetLastError(), "batch: fork"));
				}
			}
			// the larger groups first on the capture stream; every group on its own branch
			for (int g = 0; g < kBatchGroups; ++g) {
				if (b->items[g].empty()) continue;
				const int st = launch_batch_pass(1 + (g & 1), (g & 2) != 0, pass == 1, b->d_images, b->d_items[g],
					static_cast<int>(b->items[g].size()), c + g, t == iterations - 1, b->grid[g], b->smem[g],
					g == 0 ? s0 : b->side[g]);
				if (st) return abort_capture(st);
			}
			for (int g = 1; g < kBatchGroups; ++g) {
				if (b->items[g].empty()) continue;
				if (cudaEventRecord(b->join[g], b->side[g]) != cudaSuccess ||
				    cudaStreamWaitEvent(s0, b->join[g], 0) != cudaSuccess) {
					return abort_capture(cuda_fail(cudaGetLastError(), "batch: join"));
				}
			}
		}
	}
	if (iterations == 0) {
		batch_init_kernel<<<dim3(n, 16), 256, 0, s0>>>(b->d_init, starts, eps, -1);
	}
	IANE_GB_CUDA(cudaStreamEndCapture(s0, &graph), "batch: end capture");
	if (b->exec) {
		cudaGraphExecDestroy(b->exec);
		b->exec = nullptr;
	}
	const cudaError_t e = cudaGraphInstantiate(&b->exec, graph, 0);
	cudaGraphDestroy(graph);
	IANE_GB_CUDA(e, "batch: instantiate graph");
	return IANE_GB_OK;
}

int occupancy_grid(int wx, bool wide, size_t smem, size_t items)
{
	int per_sm = 1;
	const size_t total = smem + 32;
	const void* kernel = batch_kernel_handle(wx, wide);
	cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(total));
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32 * wx * wx, total);
	const long long g = static_cast<long long>(device_sm_count()) * std::max(1, per_sm);
	return static_cast<int>(std::max<long long>(1, std::min<long long>(g, static_cast<long long>(items))));
}

void fill_items(iane_gb_rl_batch* b)
{
	for (int g = 0; g < kBatchGroups; ++g) b->items[g].clear();
	std::vector<int> order(b->count);
	for (int i = 0; i < b->count; ++i) order[i] = i;
	// group images by PSF width so that consecutive work items run the same kernel code
	std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b->kx[a] < b->kx[c]; });
	for (int i : order) {
		const int w = b->wx[i], t = 32 * w;
		const int tiles = ((b->nx[i] + t - 1) / t) * ((b->ny[i] + t - 1) / t);
		const int g = batch_group(w, b->kx[i]);
		for (int k = 0; k < tiles; ++k) b->items[g].push_back(BatchItem{i, k});
		b->smem[g] = std::max(b->smem[g], batch_tile_smem(w, b->kx[i], b->ky[i]));
	}
}

}  // namespace
}  // namespace iane_gb

using namespace iane_gb;

extern "C" {

int iane_gb_rl_batch_destroy(iane_gb_rl_batch* b)
{
	if (!b) return IANE_GB_OK;
	for (auto* p : b->plans) iane_gb_rl_destroy(p);
	for (int g = 0; g < kBatchGroups; ++g) cudaFree(b->d_items[g]);
	cudaFree(b->d_images);
	cudaFree(b->d_init);
	if (b->exec) cudaGraphExecDestroy(b->exec);
	if (b->fork) cudaEventDestroy(b->fork);
	for (int g = 0; g < kBatchGroups; ++g) {
		if (b->join[g]) cudaEventDestroy(b->join[g]);
		if (b->side[g]) cudaStreamDestroy(b->side[g]);
	}
	delete b;
	return IANE_GB_OK;
}

int iane_gb_rl_batch_prepare(const iane_gb_view* psfs, int count, const int32_t* extents, unsigned flags,
	void* stream, iane_gb_rl_batch** out)
{
	if (!out || !psfs || !extents || count < 1) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_batch_prepare: need at least one image");
	}
	if (flags & ~IANE_GB_BATCH_AUTOTUNE) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_batch_prepare: unknown flags");
	}
	*out = nullptr;
	auto* b = new iane_gb_rl_batch{};
	b->count = count;
	auto cleanup = [&](int code) {
		iane_gb_rl_batch_destroy(b);
		return code;
	};
	for (int i = 0; i < count; ++i) {
		const int32_t ext[3] = {extents[2 * i], extents[2 * i + 1], 1};
		if (psfs[i].rank != 2) {
			return cleanup(fail(IANE_GB_INVALID_ARGUMENT, "rl_batch_prepare: the batch takes 2-D images and PSFs"));
		}
		iane_gb_rl_plan* p = nullptr;
		const int st = iane_gb_rl_prepare(&psfs[i], 2, ext, stream, &p);
		if (st) return cleanup(st);
		b->plans.push_back(p);
		b->nx.push_back(ext[0]);
		b->ny.push_back(ext[1]);
		b->kx.push_back(psfs[i].extent[0]);
		b->ky.push_back(psfs[i].extent[1]);
		b->pitch.push_back((static_cast<long long>(ext[0]) + 3) & ~3LL);
	}
	// tile shape per image: the tuner's cached (or freshly measured) choice, else 64x64 tiles
	// for images at least 48 wide and high
	b->wx.assign(count, 2);
	for (int i = 0; i < count; ++i) {
		if (b->nx[i] < 48 || b->ny[i] < 48) b->wx[i] = 1;
	}
	if (flags & IANE_GB_BATCH_AUTOTUNE) {
		const int st = batch_autotune(b->nx, b->ny, b->kx, b->ky, b->plans, b->wx, static_cast<cudaStream_t>(stream));
		if (st) return cleanup(st);
	}
	size_t off = 0;
	for (int i = 0; i < count; ++i) {
		const size_t bytes = align_up(static_cast<size_t>(b->pitch[i]) * b->ny[i] * 4);
		b->off.push_back(off);
		b->img_bytes.push_back(bytes);
		off += 2 * bytes;
	}
	b->parts_off = off;
	off += align_up(static_cast<size_t>(count) * sizeof(float));
	b->counter_off = off;
	off += align_up(static_cast<size_t>(2 * kBatchGroups * (kMaxBatchIterations + 1)) * sizeof(unsigned int));
	b->scratch_bytes = off + kAlignB;
	fill_items(b);
	for (int g = 0; g < kBatchGroups; ++g) {
		if (b->items[g].empty()) continue;
		b->grid[g] = occupancy_grid(1 + (g & 1), (g & 2) != 0, b->smem[g], b->items[g].size());
		if (cudaMalloc(&b->d_items[g], b->items[g].size() * sizeof(BatchItem)) != cudaSuccess ||
		    cudaMemcpy(b->d_items[g], b->items[g].data(), b->items[g].size() * sizeof(BatchItem),
		        cudaMemcpyHostToDevice) != cudaSuccess) {
			return cleanup(cuda_fail(cudaGetLastError(), "rl_batch_prepare: upload work items"));
		}
	}
	if (cudaMalloc(&b->d_images, count * sizeof(BatchImage)) != cudaSuccess ||
	    cudaMalloc(&b->d_init, count * sizeof(InitDesc)) != cudaSuccess ||
	    cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
		return cleanup(cuda_fail(cudaGetLastError(), "rl_batch_prepare: allocate descriptors"));
	}
	for (int g = 0; g < kBatchGroups; ++g) {
		if (cudaStreamCreateWithFlags(&b->side[g], cudaStreamNonBlocking) != cudaSuccess ||
		    cudaEventCreateWithFlags(&b->join[g], cudaEventDisableTiming) != cudaSuccess) {
			return cleanup(cuda_fail(cudaGetLastError(), "rl_batch_prepare: allocate streams"));
		}
	}
	*out = b;
	return IANE_GB_OK;
}

size_t iane_gb_rl_batch_scratch_bytes(const iane_gb_rl_batch* b)
{
	return b ? b->scratch_bytes : 0;
}

int iane_gb_rl_batch_tiles(const iane_gb_rl_batch* b, int32_t* tile_width)
{
	if (!b || !tile_width) return fail(IANE_GB_INVALID_ARGUMENT, "rl_batch_tiles: null argument");
	for (int i = 0; i < b->count; ++i) tile_width[i] = 32 * b->wx[i];
	return IANE_GB_OK;
}

int iane_gb_rl_batch_run(iane_gb_rl_batch* b, const iane_gb_view* observed, const iane_gb_view* estimates,
	int iterations, float epsilon, int init, void* scratch, size_t scratch_bytes, void* stream)
{
	if (!b || !observed || !estimates) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_batch_run: null argument");
	}
	if (iterations < 0 || iterations > kMaxBatchIterations || !(epsilon > 0.0f) || !std::isfinite(epsilon)) {
		return fail(IANE_GB_INVALID_ARGUMENT, "Iterations and finite epsilon must be positive");
	}
	if (init < IANE_GB_RL_INIT_OBSERVED || init > IANE_GB_RL_INIT_GIVEN) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_batch_run: unknown init mode");
	}
	if (!scratch || scratch_bytes < b->scratch_bytes) {
		return fail(IANE_GB_LENGTH_ERROR, "Prepared operation exceeded its scratch reservation");
	}
	std::vector<DevView> obs(b->count), est(b->count);
	std::ostringstream key;
	key << scratch << ' ' << iterations << ' ' << epsilon << ' ' << init;
	for (int i = 0; i < b->count; ++i) {
		int st = normalise_view(&observed[i], "rl_batch_run observed", &obs[i]);
		if (st) return st;
		st = normalise_view(&estimates[i], "rl_batch_run estimate", &est[i]);
		if (st) return st;
		if (obs[i].rank != 2 || est[i].rank != 2 || obs[i].ext[0] != b->nx[i] || obs[i].ext[1] != b->ny[i] ||
		    est[i].ext[0] != b->nx[i] || est[i].ext[1] != b->ny[i]) {
			return fail(IANE_GB_INVALID_ARGUMENT, "rl_batch_run: views must have the prepared 2-D extents");
		}
		if ((obs[i].dtype != IANE_GB_F32 && obs[i].dtype != IANE_GB_U8) ||
		    (est[i].dtype != IANE_GB_F32 && est[i].dtype != IANE_GB_U8) ||
		    (init == IANE_GB_RL_INIT_GIVEN && est[i].dtype != IANE_GB_F32)) {
			return fail(IANE_GB_UNSUPPORTED, "rl_batch_run: observed f32/u8, estimate f32/u8 (f32 for a given start)");
		}
		key << ' ' << static_cast<const void*>(obs[i].ptr) << ' ' << obs[i].stride[0] << ' ' << obs[i].stride[1] << ' '
			<< obs[i].dtype << ' ' << static_cast<const void*>(est[i].ptr) << ' ' << est[i].stride[0] << ' '
			<< est[i].stride[1] << ' ' << est[i].dtype;
	}
	char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(scratch) + kAlignB - 1) / kAlignB * kAlignB);
	if (!b->exec || key.str() != b->key) {
		// a new configuration: describe the run and capture it (the capture runs nothing)
		IANE_GB_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "rl_batch_run: wait before capture");
		const int st = build_graph(b, obs.data(), est.data(), iterations, epsilon, init, base);
		if (st) {
			b->key.clear();
			return st;
		}
		b->key = key.str();
	}
	IANE_GB_CUDA(cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)), "rl_batch_run: launch graph");
	return IANE_GB_OK;
}

}  // extern "C"
