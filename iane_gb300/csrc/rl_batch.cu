// Batched Richardson-Lucy: plans, the work queue, the autotuned launch configuration, the
// CUDA graph of a run and the C-ABI entry points iane_gb_rl_batch_*. See rl_batch.cuh for the
// execution design.
#include "kernels.h"
#include "rl_batch.cuh"

#include <algorithm>
#include <array>
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

bool work_layout(const DevView& v, long long pitch)
{
	if (v.dtype != IANE_GB_F32 || v.stride[0] != 4 || reinterpret_cast<uintptr_t>(v.ptr) % 16 != 0) return false;
	if (v.ext[1] > 1 && v.stride[1] != pitch * 4) return false;
	return true;
}

int tiles_of(int n) { return (n + kBatchTile - 1) / kBatchTile; }

// Queue orders of one phase's items (the autotuner picks one per batch).
constexpr int kOrderLargestFirst = 0; // images by descending tile count
constexpr int kOrderByWidth = 1;      // images by PSF width, then by descending tile count
constexpr int kOrders = 2;

// Item shapes: tiles per item (along x) by PSF width, one rule per grouping level. Narrow PSFs
// do little arithmetic per tile, so their items carry the per-item queue, dependency and
// completion work over several tiles and load the taps once.
constexpr int kGroups = 4;
int tiles_per_item(int kx, int group)
{
	switch (group) {
	case 1: return kx <= 11 ? 2 : 1;
	case 2: return kx <= 11 ? 4 : 1;
	case 3: return kx <= 7 ? 4 : (kx <= 15 ? 2 : 1);
	default: return 1;
	}
}

std::vector<BatchItem> make_items(const std::vector<int>& nx, const std::vector<int>& ny, const std::vector<int>& kx,
	int order, int group)
{
	const int n = static_cast<int>(nx.size());
	std::vector<int> idx(n);
	for (int i = 0; i < n; ++i) idx[i] = i;
	auto tiles = [&](int i) { return tiles_of(nx[i]) * tiles_of(ny[i]); };
	std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
		if (order == kOrderByWidth && kx[a] != kx[b]) return kx[a] < kx[b];
		return tiles(a) > tiles(b);
	});
	std::vector<BatchItem> items;
	for (int i : idx) {
		const int tx = tiles_of(nx[i]), ty = tiles_of(ny[i]), s = tiles_per_item(kx[i], group);
		for (int r = 0; r < ty; ++r) {
			for (int c = 0; c < tx; c += s) items.push_back(BatchItem{i, r * tx + c, std::min(s, tx - c), tx * ty});
		}
	}
	return items;
}

// ---------------------------------------------------------------------------------------
// autotuner: CTAs per SM, queue order and item shapes per batch (shapes, PSF sizes, dtype,
// SM count), cached in a text file

struct TuneCache {
	std::mutex lock;
	bool loaded = false;
	std::map<std::string, std::array<int, 3>> choice; // key -> (CTAs per SM, order, grouping)
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

// The batch signature: image count, a 64-bit FNV-1a hash of every (nx, ny, kx, ky), dtype, SMs.
std::string tune_key(const std::vector<int>& nx, const std::vector<int>& ny, const std::vector<int>& kx,
	const std::vector<int>& ky)
{
	uint64_t h = 1469598103934665603ull;
	auto mix = [&](int v) {
		for (int b = 0; b < 4; ++b) {
			h ^= static_cast<uint64_t>((static_cast<uint32_t>(v) >> (8 * b)) & 0xffu);
			h *= 1099511628211ull;
		}
	};
	for (size_t i = 0; i < nx.size(); ++i) {
		mix(nx[i]);
		mix(ny[i]);
		mix(kx[i]);
		mix(ky[i]);
	}
	std::ostringstream k;
	k << "rl2d-batch f32 images " << nx.size() << " shapes " << std::hex << h << std::dec << " sms "
	  << device_sm_count();
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
		// "<key> | <ms per configuration ...> | <CTAs per SM> <order> <grouping>"
		const auto first = line.find(" | ");
		const auto last = line.rfind(" | ");
		if (first == std::string::npos || last == first) continue;
		std::istringstream tail(line.substr(last + 3));
		int bps = 0, order = -1, group = 0;
		if (tail >> bps >> order && bps > 0 && order >= 0 && order < kOrders) {
			if (!(tail >> group) || group < 0 || group >= kGroups) group = 0;
			c.choice[line.substr(0, first)] = {bps, order, group};
		}
	}
}

}  // namespace
}  // namespace iane_gb

struct iane_gb_rl_batch {
	int count = 0;
	std::vector<iane_gb_rl_plan*> plans;
	std::vector<int> nx, ny, kx, ky;
	std::vector<long long> pitch;
	std::vector<size_t> off;               // per image: ratio at off, work at off + image bytes
	std::vector<size_t> img_bytes;
	std::vector<iane_gb::BatchItem> items; // one phase of the queue
	iane_gb::BatchItem* d_items = nullptr;
	size_t smem = 0;                       // dynamic shared memory of the launch
	int blocks_per_sm = 1;                 // resident CTAs per SM the launch uses
	int order = 0;                         // queue order (autotuned)
	int group = 0;                         // item shapes by PSF width (autotuned, tiles_per_item)
	iane_gb::BatchImage* d_images = nullptr;
	iane_gb::InitDesc* d_init = nullptr;
	size_t parts_off = 0, sync_off = 0, scratch_bytes = 0;
	cudaStream_t capture = nullptr;
	cudaGraphExec_t exec = nullptr;
	std::string key;
};

namespace iane_gb {
namespace {

// Device descriptors of every image for a run over `base` (the scratch).
int fill_images(const iane_gb_rl_batch* b, const DevView* obs, const DevView* est, float eps, char* base,
	std::vector<BatchImage>& host, std::vector<InitDesc>& idesc)
{
	const int n = b->count;
	host.assign(n, BatchImage{});
	idesc.assign(n, InitDesc{});
	int* status = device_status_ptr();
	if (!status) return IANE_GB_CUDA_ERROR;
	for (int i = 0; i < n; ++i) {
		const int nx = b->nx[i], ny = b->ny[i], kxi = b->kx[i], kyi = b->ky[i];
		const long long pitch = b->pitch[i], plane = pitch * ny;
		float* ratio = reinterpret_cast<float*>(base + b->off[i]);
		float* work = reinterpret_cast<float*>(base + b->off[i] + b->img_bytes[i]);
		const bool in_place = est && work_layout(est[i], pitch);
		float* e_work = in_place ? reinterpret_cast<float*>(est[i].ptr) : work;
		BatchImage& im = host[i];
		std::memset(&im, 0, sizeof im);
		int st = encode_tensor_map_f32(&im.map_est, e_work, nx, ny, 1, pitch * 4, plane * 4, tile_pitch(kxi, 2),
			kBatchTile + 2 * (kyi / 2));
		if (st) return st;
		st = encode_tensor_map_f32(&im.map_ratio, ratio, nx, ny, 1, pitch * 4, plane * 4, tile_pitch(kxi, 2),
			kBatchTile + 2 * (kyi / 2));
		if (st) return st;
		rl_plan_fill_passes(b->plans[i], &im.pass_a, &im.pass_b, &im.epi_a, &im.epi_b, status);
		im.epi_a.ratio = ratio;
		im.epi_a.obs = obs[i].ptr;
		for (int a = 0; a < 3; ++a) im.epi_a.os[a] = obs[i].stride[a];
		im.epi_a.obs_u8 = obs[i].dtype == IANE_GB_U8;
		im.epi_a.eps = eps;
		im.epi_b.est = e_work;
		im.epi_b.eps = eps;
		if (est) {
			im.epi_b.out = est[i].ptr;
			for (int a = 0; a < 3; ++a) im.epi_b.outs[a] = est[i].stride[a];
			im.epi_b.out_u8 = est[i].dtype == IANE_GB_U8;
		}
		im.kx = kxi;
		im.tiles_x = tiles_of(nx);
		im.tiles = tiles_of(nx) * tiles_of(ny);
		im.write_out_final = in_place || !est ? 0 : 1;
		idesc[i].obs = obs[i];
		if (est) idesc[i].est = est[i];
		idesc[i].work = e_work;
		idesc[i].pitch = pitch;
		idesc[i].in_place = in_place ? 1 : 0;
	}
	return IANE_GB_OK;
}

BatchSync sync_words(const iane_gb_rl_batch* b, char* base)
{
	unsigned int* words = reinterpret_cast<unsigned int*>(base + b->sync_off);
	return BatchSync{words, reinterpret_cast<int*>(words + 1), words + 2};
}

size_t sync_bytes(int count) { return static_cast<size_t>(count + 2) * sizeof(unsigned int); }

// Build descriptors for one run and the graph that performs it: clear the queue, abort flag
// and completion counters, the start values, then the one persistent launch.
int build_graph(iane_gb_rl_batch* b, const DevView* obs, const DevView* est, int iterations, float eps, int init,
	char* base)
{
	const int n = b->count;
	std::vector<BatchImage> host;
	std::vector<InitDesc> idesc;
	int st = fill_images(b, obs, est, eps, base, host, idesc);
	if (st) return st;
	IANE_GB_CUDA(cudaMemcpy(b->d_images, host.data(), n * sizeof(BatchImage), cudaMemcpyHostToDevice),
		"batch: upload image descriptors");
	IANE_GB_CUDA(cudaMemcpy(b->d_init, idesc.data(), n * sizeof(InitDesc), cudaMemcpyHostToDevice),
		"batch: upload start descriptors");
	int* status = device_status_ptr();
	if (!status) return IANE_GB_CUDA_ERROR;

	float* starts = reinterpret_cast<float*>(base + b->parts_off);
	const BatchSync sync = sync_words(b, base);
	cudaStream_t s0 = b->capture;
	cudaGraph_t graph = nullptr;
	IANE_GB_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal), "batch: begin capture");
	auto abort_capture = [&](int code) {
		cudaGraph_t g = nullptr;
		cudaStreamEndCapture(s0, &g);
		if (g) cudaGraphDestroy(g);
		return code;
	};
	if (cudaMemsetAsync(sync.queue, 0, sync_bytes(n), s0) != cudaSuccess) {
		return abort_capture(cuda_fail(cudaGetLastError(), "batch: clear queue"));
	}
	if (init == IANE_GB_RL_INIT_MEAN) {
		batch_mean_kernel<<<n, 256, 0, s0>>>(b->d_init, starts, eps);
	}
	batch_init_kernel<<<dim3(n, 16), 256, 0, s0>>>(b->d_init, starts, eps, init);
	if (iterations > 0) {
		st = launch_batch_persistent(b->d_images, b->d_items, static_cast<int>(b->items.size()), 2 * iterations, sync,
			status, b->blocks_per_sm * device_sm_count(), b->smem, s0);
		if (st) return abort_capture(st);
	} else {
		batch_init_kernel<<<dim3(n, 16), 256, 0, s0>>>(b->d_init, starts, eps, -1);
	}
	if (cudaGetLastError() != cudaSuccess) {
		return abort_capture(cuda_fail(cudaGetLastError(), "batch: capture launches"));
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

// Choose CTAs per SM (1 .. occupancy) and the queue order by timing a two-iteration run of the
// whole batch per candidate on scratch images (observed = 1), once per batch signature.
int autotune(iane_gb_rl_batch* b, cudaStream_t stream)
{
	TuneCache& cache = tune_cache();
	std::lock_guard<std::mutex> guard(cache.lock);
	load_cache(cache);
	const std::string key = tune_key(b->nx, b->ny, b->kx, b->ky);
	const auto hit = cache.choice.find(key);
	const int max_bps = batch_blocks_per_sm(b->smem);
	if (hit != cache.choice.end()) {
		b->blocks_per_sm = std::min(hit->second[0], max_bps);
		b->order = hit->second[1];
		b->group = hit->second[2];
		return IANE_GB_OK;
	}
	int* status = device_status_ptr();
	if (!status) return IANE_GB_CUDA_ERROR;
	const int n = b->count;
	size_t obs_bytes = 0;
	std::vector<size_t> obs_off(n);
	for (int i = 0; i < n; ++i) {
		obs_off[i] = obs_bytes;
		obs_bytes += (static_cast<size_t>(b->pitch[i]) * b->ny[i] * 4 + 255) & ~size_t(255);
	}
	char* buf = nullptr;
	BatchImage* d_images = nullptr;
	BatchItem* d_items = nullptr;
	cudaEvent_t t0 = nullptr, t1 = nullptr;
	auto release = [&](int code) {
		cudaFree(buf);
		cudaFree(d_images);
		cudaFree(d_items);
		if (t0) cudaEventDestroy(t0);
		if (t1) cudaEventDestroy(t1);
		return code;
	};
	const size_t run_bytes = b->scratch_bytes;
	if (cudaMalloc(&buf, run_bytes + obs_bytes) != cudaSuccess || cudaMalloc(&d_images, n * sizeof(BatchImage)) != cudaSuccess ||
	    cudaMalloc(&d_items, b->items.size() * sizeof(BatchItem)) != cudaSuccess || cudaEventCreate(&t0) != cudaSuccess ||
	    cudaEventCreate(&t1) != cudaSuccess) {
		return release(cuda_fail(cudaGetLastError(), "autotune: allocate"));
	}
	char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(buf) + kAlignB - 1) / kAlignB * kAlignB);
	char* obs_base = buf + run_bytes;
	std::vector<float> ones;
	std::vector<DevView> obs(n);
	for (int i = 0; i < n; ++i) {
		DevView& v = obs[i];
		v = DevView{};
		v.ptr = obs_base + obs_off[i];
		v.dtype = IANE_GB_F32;
		v.rank = 2;
		v.ext[0] = b->nx[i];
		v.ext[1] = b->ny[i];
		v.ext[2] = 1;
		v.stride[0] = 4;
		v.stride[1] = b->pitch[i] * 4;
		v.stride[2] = v.stride[1] * b->ny[i];
		ones.assign(static_cast<size_t>(b->pitch[i]) * b->ny[i], 1.0f);
		if (cudaMemcpy(v.ptr, ones.data(), ones.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
			return release(cuda_fail(cudaGetLastError(), "autotune: observed"));
		}
	}
	std::vector<BatchImage> host;
	std::vector<InitDesc> idesc;
	int st = fill_images(b, obs.data(), nullptr, 1e-6f, base, host, idesc);
	if (st) return release(st);
	IANE_GB_CUDA(cudaMemset(base, 0, b->parts_off), "autotune: clear images");
	if (cudaMemcpy(d_images, host.data(), n * sizeof(BatchImage), cudaMemcpyHostToDevice) != cudaSuccess) {
		return release(cuda_fail(cudaGetLastError(), "autotune: upload"));
	}
	const BatchSync sync = sync_words(b, base);
	const int sms = device_sm_count();
	std::ostringstream timings;
	float best = 0.0f;
	// ms of a two-iteration run of the whole batch with one launch configuration
	auto time_config = [&](int order, int group, int bps, float& ms) -> int {
		const std::vector<BatchItem> items = make_items(b->nx, b->ny, b->kx, order, group);
		if (cudaMemcpy(d_items, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice) != cudaSuccess) {
			return cuda_fail(cudaGetLastError(), "autotune: upload items");
		}
		ms = 0.0f;
		for (int rep = 0; rep < 3; ++rep) {
			if (cudaMemsetAsync(sync.queue, 0, sync_bytes(n), stream) != cudaSuccess) {
				return cuda_fail(cudaGetLastError(), "autotune: clear queue");
			}
			cudaEventRecord(t0, stream);
			const int s = launch_batch_persistent(d_images, d_items, static_cast<int>(items.size()), 4, sync, status,
				bps * sms, b->smem, stream);
			if (s) return s;
			cudaEventRecord(t1, stream);
			IANE_GB_CUDA(cudaEventSynchronize(t1), "autotune: time");
			float e = 0.0f;
			cudaEventElapsedTime(&e, t0, t1);
			if (rep > 0) ms += e / 2.0f; // the first run warms up
		}
		timings << ms << ' ';
		return IANE_GB_OK;
	};
	// CTAs per SM x queue order with one tile per item, then the item shapes at the best of those
	for (int order = 0; order < kOrders; ++order) {
		for (int bps = 1; bps <= max_bps; ++bps) {
			float ms = 0.0f;
			st = time_config(order, 0, bps, ms);
			if (st) return release(st);
			if (best == 0.0f || ms < best) {
				best = ms;
				b->blocks_per_sm = bps;
				b->order = order;
			}
		}
	}
	b->group = 0;
	for (int group = 1; group < kGroups; ++group) {
		float ms = 0.0f;
		st = time_config(b->order, group, b->blocks_per_sm, ms);
		if (st) return release(st);
		if (ms < best) {
			best = ms;
			b->group = group;
		}
	}
	cache.choice[key] = {b->blocks_per_sm, b->order, b->group};
	std::ofstream log(cache.path, std::ios::app);
	if (log) {
		log << key << " | " << timings.str() << "| " << b->blocks_per_sm << ' ' << b->order << ' ' << b->group << "\n";
	}
	return release(IANE_GB_OK);
}

}  // namespace
}  // namespace iane_gb

using namespace iane_gb;

extern "C" {

int iane_gb_rl_batch_destroy(iane_gb_rl_batch* b)
{
	if (!b) return IANE_GB_OK;
	for (auto* p : b->plans) iane_gb_rl_destroy(p);
	cudaFree(b->d_items);
	cudaFree(b->d_images);
	cudaFree(b->d_init);
	if (b->exec) cudaGraphExecDestroy(b->exec);
	if (b->capture) cudaStreamDestroy(b->capture);
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
		b->smem = std::max(b->smem, batch_tile_smem(psfs[i].extent[0], psfs[i].extent[1]));
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
	b->sync_off = off;
	off += align_up(sync_bytes(count));
	b->scratch_bytes = off + kAlignB;
	b->blocks_per_sm = batch_blocks_per_sm(b->smem);
	b->order = kOrderLargestFirst;
	b->group = 0;
	b->items = make_items(b->nx, b->ny, b->kx, b->order, b->group);
	if (cudaMalloc(&b->d_items, b->items.size() * sizeof(BatchItem)) != cudaSuccess ||
	    cudaMalloc(&b->d_images, count * sizeof(BatchImage)) != cudaSuccess ||
	    cudaMalloc(&b->d_init, count * sizeof(InitDesc)) != cudaSuccess ||
	    cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking) != cudaSuccess) {
		return cleanup(cuda_fail(cudaGetLastError(), "rl_batch_prepare: allocate descriptors"));
	}
	if (flags & IANE_GB_BATCH_AUTOTUNE) {
		const int st = autotune(b, static_cast<cudaStream_t>(stream));
		if (st) return cleanup(st);
		b->items = make_items(b->nx, b->ny, b->kx, b->order, b->group);
	}
	if (cudaMemcpy(b->d_items, b->items.data(), b->items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice) !=
	    cudaSuccess) {
		return cleanup(cuda_fail(cudaGetLastError(), "rl_batch_prepare: upload work items"));
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
	for (int i = 0; i < b->count; ++i) tile_width[i] = kBatchTile * tiles_per_item(b->kx[i], b->group);
	return IANE_GB_OK;
}

int iane_gb_rl_batch_config(const iane_gb_rl_batch* b, int32_t* blocks_per_sm, int32_t* order, int32_t* grouping)
{
	if (!b || !blocks_per_sm || !order || !grouping) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_batch_config: null argument");
	}
	*blocks_per_sm = b->blocks_per_sm;
	*order = b->order;
	*grouping = b->group;
	return IANE_GB_OK;
}

int iane_gb_rl_batch_configure(iane_gb_rl_batch* b, int blocks_per_sm, int order, int grouping)
{
	if (!b) return fail(IANE_GB_INVALID_ARGUMENT, "rl_batch_configure: null batch");
	if (blocks_per_sm < 1 || blocks_per_sm > batch_blocks_per_sm(b->smem) || order < 0 || order >= kOrders ||
	    grouping < 0 || grouping >= kGroups) {
		return fail(IANE_GB_INVALID_ARGUMENT, "rl_batch_configure: configuration out of range");
	}
	std::vector<BatchItem> items = make_items(b->nx, b->ny, b->kx, order, grouping);
	// a run still in flight may read the queue: wait for the device before replacing it (a
	// grouping never makes more items than one tile per item, for which d_items was sized)
	IANE_GB_CUDA(cudaDeviceSynchronize(), "rl_batch_configure: wait for running work");
	IANE_GB_CUDA(cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice),
		"rl_batch_configure: upload work items");
	b->items.swap(items);
	b->blocks_per_sm = blocks_per_sm;
	b->order = order;
	b->group = grouping;
	b->key.clear(); // the next run captures a graph with the new launch
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
	if (static_cast<long long>(b->items.size()) * 2 * iterations >= (1LL << 31)) {
		return fail(IANE_GB_UNSUPPORTED, "rl_batch_run: more than 2^31 work items (tiles x passes)");
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
