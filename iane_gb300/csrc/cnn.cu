// Kernels of the learned warm start: a small 3-D encoder-decoder CNN, BF16 activations and
// weights, FP32 accumulation.
//
// Activation layout ("C8"): channels in octets, each octet voxel-major with its 8 channels
// contiguous -- element (c, v) of a C-channel volume of V voxels sits at
// ((c / 8) * V + v) * 8 + c % 8 (ceil(C / 8) octets; unused slots of the last octet are
// never read as data). A voxel's octet is one 16-byte vector: the tensor-core kernel
// (cnn_tc.cu) takes it as a row of its K-major operand straight from a TMA box. FP32
// outputs (the network output, test readbacks) are planar [c][v].
//
//   conv3       y[co] = act(b[co] + sum_{ci,t} w[co][ci][t] * x[ci](v + t - 1) (+ residual)),
//               zero padding, inputs given as two tensors concatenated along channels (the
//               decoder's skip connections), optional mask m: y *= (m > 0) (the ReLU of the
//               layer below, fused into input gradients); FP32 or BF16 output
//   conv3_wgrad partial dW[co][ci][t] and db[co] over a chunk of voxels per CTA (split-K),
//               summed in fixed order by conv3_wgrad_reduce (deterministic)
//   flip        wt[ci][co][t] = w[co][ci][26 - t]: the input gradient of a 3x3x3 convolution is
//               the convolution of the output gradient with these weights
//   pool2 / up2 and their gradients, mse (loss and gradient), adam (FP32 master weights)
//
// Direct SIMT implementation (training and input gradients): a CTA computes an 8x8x4 brick
// of output voxels for all output channels, one voxel per thread with CO accumulators; input
// halo bricks and the weights of four input channels are staged in shared memory per step,
// weights read as warp-uniform 128-bit broadcasts.
#include "common.cuh"

#include <cstdint>

namespace iane_gb {
namespace {

constexpr int BX = 8, BY = 8, BZ = 4;        // output brick
constexpr int HX = BX + 2, HY = BY + 2, HZ = BZ + 2;
constexpr int HALO = HX * HY * HZ;           // 600
constexpr int CI_STEP = 4;
constexpr int NT = BX * BY * BZ;             // 256 threads

__device__ __forceinline__ float bf(uint16_t v) { return __uint_as_float(static_cast<uint32_t>(v) << 16); }

// Offset of element (c, v) in a C8 tensor of `vol` voxels.
__host__ __device__ __forceinline__ long long c8(int c, long long v, long long vol)
{
	return ((static_cast<long long>(c >> 3) * vol + v) << 3) + (c & 7);
}
__device__ __forceinline__ uint16_t to_bf(float f)
{
	const __nv_bfloat16 b = __float2bfloat16_rn(f);
	return *reinterpret_cast<const uint16_t*>(&b);
}

struct Conv3Args {
	const uint16_t* x0;
	const uint16_t* x1;
	int c0, c1;
	int d, h, w;
	const uint16_t* wt;     // [co][c0 + c1][27]
	const float* bias;      // [co] or null
	int co;
	uint16_t* y16;          // bf16 output (C8), or null
	float* y32;             // f32 output (planar [co][v]), or null
	const float* residual;  // f32, added before the activation (co == 1 only), or null
	int act;                // 0 none, 1 relu
	const uint16_t* mask;   // C8, co channels: y *= (mask > 0), or null
	int bricks_x, bricks_y;
};

template<int CO>
__global__ void __launch_bounds__(NT) conv3_kernel(const Conv3Args a)
{
	__shared__ float xs[CI_STEP][HALO];
	__shared__ __align__(16) float ws[CI_STEP][27][CO];
	const int tid = threadIdx.x;
	const int lx = tid % BX, ly = (tid / BX) % BY, lz = tid / (BX * BY);
	const int bx = blockIdx.x % a.bricks_x, by = blockIdx.x / a.bricks_x, bz = blockIdx.y;
	const int x0 = bx * BX, y0 = by * BY, z0 = bz * BZ;
	const int x = x0 + lx, y = y0 + ly, z = z0 + lz;
	const long long plane = static_cast<long long>(a.h) * a.w;
	const long long vol = plane * a.d;
	const int ci_total = a.c0 + a.c1;
	float acc[CO];
#pragma unroll
	for (int c = 0; c < CO; ++c) acc[c] = 0.0f;

	for (int ci0 = 0; ci0 < ci_total; ci0 += CI_STEP) {
		__syncthreads();
		for (int i = tid; i < CI_STEP * HALO; i += NT) {
			const int k = i % CI_STEP, r = i / CI_STEP;  // 4 neighbouring threads: 8 contiguous bytes
			const int hx = r % HX, hy = (r / HX) % HY, hz = r / (HX * HY);
			const int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
			const int ci = ci0 + k;
			float v = 0.0f;
			if (ci < ci_total && gx >= 0 && gx < a.w && gy >= 0 && gy < a.h && gz >= 0 && gz < a.d) {
				const long long at = gz * plane + static_cast<long long>(gy) * a.w + gx;
				v = bf(ci < a.c0 ? a.x0[c8(ci, at, vol)] : a.x1[c8(ci - a.c0, at, vol)]);
			}
			xs[k][r] = v;
		}
		for (int i = tid; i < CI_STEP * 27 * CO; i += NT) {
			const int c = i % CO, t = (i / CO) % 27, k = i / (27 * CO);
			const int ci = ci0 + k;
			ws[k][t][c] = (ci < ci_total && c < a.co) ? bf(a.wt[(static_cast<long long>(c) * ci_total + ci) * 27 + t]) : 0.0f;
		}
		__syncthreads();
#pragma unroll
		for (int k = 0; k < CI_STEP; ++k) {
#pragma unroll 3
			for (int t = 0; t < 27; ++t) {
				const int tx = t % 3, ty = (t / 3) % 3, tz = t / 9;
				const float v = xs[k][(lz + tz) * HX * HY + (ly + ty) * HX + lx + tx];
				if constexpr (CO % 4 == 0) {
#pragma unroll
					for (int c = 0; c < CO; c += 4) {
						const float4 w4 = *reinterpret_cast<const float4*>(&ws[k][t][c]);
						acc[c] = fmaf(w4.x, v, acc[c]);
						acc[c + 1] = fmaf(w4.y, v, acc[c + 1]);
						acc[c + 2] = fmaf(w4.z, v, acc[c + 2]);
						acc[c + 3] = fmaf(w4.w, v, acc[c + 3]);
					}
				} else {
#pragma unroll
					for (int c = 0; c < CO; ++c) acc[c] = fmaf(ws[k][t][c], v, acc[c]);
				}
			}
		}
	}
	if (x >= a.w || y >= a.h || z >= a.d) {
		return;
	}
	const long long at = z * plane + static_cast<long long>(y) * a.w + x;
#pragma unroll
	for (int c = 0; c < CO; ++c) {
		if (c >= a.co) break;
		float v = acc[c] + (a.bias ? a.bias[c] : 0.0f);
		if (a.residual) v += a.residual[c * vol + at];
		if (a.act == 1) v = v > 0.0f ? v : 0.0f;
		if (a.mask && !(bf(a.mask[c8(c, at, vol)]) > 0.0f)) v = 0.0f;
		if (a.y32) a.y32[c * vol + at] = v;
		if (a.y16) a.y16[c8(c, at, vol)] = to_bf(v);
	}
}

// Split-K weight gradient: CTA (co tile of 16, input octet, voxel chunk) accumulates, for
// each of its (output channel, tap) pairs and the octet's 8 input channels, the sum over the
// chunk's voxels of dy * x(shifted). The octet's halo brick arrives as one 16-byte vector per
// voxel.
constexpr int WG_CO = 16;
constexpr int WG_THREADS = 448; // >= 16 * 27 pairs, 14 warps

struct WgradArgs {
	const uint16_t* x0;
	const uint16_t* x1;
	int c0, c1;
	int d, h, w;
	const uint16_t* dy;
	int co;
	int chunk_bricks;   // bricks per CTA
	int bricks_x, bricks_y, bricks_total;
	float* partial;     // [chunks][co][ci][27], and [chunks][co] bias partials after that
	int chunks;
};

__global__ void __launch_bounds__(WG_THREADS) conv3_wgrad_kernel(const WgradArgs a)
{
	__shared__ float xs[8][HALO];
	__shared__ float gs[WG_CO][NT + 1];
	const int tid = threadIdx.x;
	const int co0 = blockIdx.x * WG_CO;
	const int ci0 = blockIdx.y * 8;          // this CTA's input octet
	const int chunk = blockIdx.z;
	const int ci_total = a.c0 + a.c1;
	const long long plane = static_cast<long long>(a.h) * a.w;
	const long long vol = plane * a.d;
	const int pc = tid / 27, pt = tid % 27;  // this thread's (output channel, tap)
	const bool active = tid < WG_CO * 27 && co0 + pc < a.co;
	const int tx = pt % 3, ty = (pt / 3) % 3, tz = pt / 9;
	float acc[8], bacc = 0.0f;
#pragma unroll
	for (int k = 0; k < 8; ++k) acc[k] = 0.0f;
	// the octet lies in one input tensor (c0 is a multiple of 8 or the only tensor)
	const uint16_t* xsrc = ci0 < a.c0 ? a.x0 + c8(ci0, 0, vol) : a.x1 + c8(ci0 - a.c0, 0, vol);
	const int b_begin = chunk * a.chunk_bricks;
	const int b_end = min(a.bricks_total, b_begin + a.chunk_bricks);
	for (int b = b_begin; b < b_end; ++b) {
		const int bx = b % a.bricks_x, by = (b / a.bricks_x) % a.bricks_y, bz = b / (a.bricks_x * a.bricks_y);
		const int x0 = bx * BX, y0 = by * BY, z0 = bz * BZ;
		__syncthreads();
		for (int i = tid; i < HALO; i += WG_THREADS) {
			const int hx = i % HX, hy = (i / HX) % HY, hz = i / (HX * HY);
			const int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
			uint4 q = make_uint4(0u, 0u, 0u, 0u);
			if (gx >= 0 && gx < a.w && gy >= 0 && gy < a.h && gz >= 0 && gz < a.d) {
				q = *reinterpret_cast<const uint4*>(xsrc + ((gz * plane + static_cast<long long>(gy) * a.w + gx) << 3));
			}
			const uint32_t wv[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
			for (int k = 0; k < 4; ++k) {
				xs[2 * k][i] = __uint_as_float(wv[k] << 16);
				xs[2 * k + 1][i] = __uint_as_float(wv[k] & 0xFFFF0000u);
			}
		}
		for (int i = tid; i < WG_CO * NT; i += WG_THREADS) {
			const int c = i % WG_CO, r = i / WG_CO;  // 16 neighbouring threads: one voxel's channels
			const int lx = r % BX, ly = (r / BX) % BY, lz = r / (BX * BY);
			const int gx = x0 + lx, gy = y0 + ly, gz = z0 + lz;
			float v = 0.0f;
			if (co0 + c < a.co && gx < a.w && gy < a.h && gz < a.d) {
				v = bf(a.dy[c8(co0 + c, gz * plane + static_cast<long long>(gy) * a.w + gx, vol)]);
			}
			gs[c][r] = v;
		}
		__syncthreads();
		if (active) {
			const float* g = gs[pc];
#pragma unroll 2
			for (int r = 0; r < NT; ++r) {
				const int lx = r % BX, ly = (r / BX) % BY, lz = r / (BX * BY);
				const int at = (lz + tz) * HX * HY + (ly + ty) * HX + lx + tx;
				const float gv = g[r];
#pragma unroll
				for (int k = 0; k < 8; ++k) acc[k] = fmaf(gv, xs[k][at], acc[k]);
				bacc += gv;
			}
		}
	}
	if (active) {
#pragma unroll
		for (int k = 0; k < 8; ++k) {
			const int ci = ci0 + k;
			if (ci < ci_total) {
				a.partial[((static_cast<long long>(chunk) * a.co + co0 + pc) * ci_total + ci) * 27 + pt] = acc[k];
			}
		}
		if (pt == 0 && ci0 == 0) {
			a.partial[static_cast<long long>(a.chunks) * a.co * ci_total * 27 + static_cast<long long>(chunk) * a.co + co0 + pc] =
				bacc;
		}
	}
}

// dw[i] += sum over chunks of partial (fixed order); the bias partials follow the weights.
__global__ void conv3_wgrad_reduce(const float* partial, int chunks, long long nw, int co, float* dw, float* db)
{
	const long long n = nw + co;
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		float s = 0.0f;
		if (i < nw) {
			for (int c = 0; c < chunks; ++c) s += partial[c * nw + i];
			dw[i] += s;
		} else {
			const long long j = i - nw;
			for (int c = 0; c < chunks; ++c) s += partial[chunks * nw + c * co + j];
			if (db) db[j] += s;
		}
	}
}

__global__ void flip_kernel(const uint16_t* w, int co, int ci, uint16_t* wt)
{
	const long long n = static_cast<long long>(co) * ci * 27;
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const int t = static_cast<int>(i % 27);
		const long long oc = i / 27;
		const int o = static_cast<int>(oc / ci), c = static_cast<int>(oc % ci);
		wt[(static_cast<long long>(c) * co + o) * 27 + (26 - t)] = w[i];
	}
}

// Average pooling 2x2x2 (input d, h, w even), nearest upsampling x2 and their gradients on C8
// tensors: one thread per (voxel, octet), 16-byte vector loads and stores. Grid: x over
// blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, (octet, z) folded into blockIdx.z
// (grid-strided); the extents are those of the tensor the thread writes.
__device__ __forceinline__ void unpack8(const uint4 q, float (&f)[8])
{
	const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		f[2 * k] = __uint_as_float(w[k] << 16);
		f[2 * k + 1] = __uint_as_float(w[k] & 0xFFFF0000u);
	}
}

__device__ __forceinline__ uint4 pack8(const float (&f)[8])
{
	uint4 q;
	q.x = static_cast<uint32_t>(to_bf(f[0])) | (static_cast<uint32_t>(to_bf(f[1])) << 16);
	q.y = static_cast<uint32_t>(to_bf(f[2])) | (static_cast<uint32_t>(to_bf(f[3])) << 16);
	q.z = static_cast<uint32_t>(to_bf(f[4])) | (static_cast<uint32_t>(to_bf(f[5])) << 16);
	q.w = static_cast<uint32_t>(to_bf(f[6])) | (static_cast<uint32_t>(to_bf(f[7])) << 16);
	return q;
}

// out-extents (od, oh, ow), octets; x = thread index, y = blockIdx.y, (oct, z) from blockIdx.z
#define IANE_GB_C8_LOOP(od, oh, ow, octets)                                                                    \
	const int x = blockIdx.x * blockDim.x + threadIdx.x;                                                       \
	const int y = blockIdx.y;                                                                                  \
	if (x >= (ow) || y >= (oh)) return;                                                                        \
	for (int zo = blockIdx.z; zo < (od) * (octets); zo += gridDim.z)

__global__ void pool2_kernel(const uint4* x_, int octets, int d, int h, int w, uint4* y_)
{
	const int od = d / 2, oh = h / 2, ow = w / 2;
	const long long ivol = static_cast<long long>(d) * h * w, ovol = static_cast<long long>(od) * oh * ow;
	IANE_GB_C8_LOOP(od, oh, ow, octets)
	{
		const int z = zo % od, oct = zo / od;
		const uint4* src = x_ + oct * ivol;
		float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
		for (int k = 0; k < 8; ++k) {
			float f[8];
			unpack8(src[(2LL * z + (k >> 2)) * h * w + static_cast<long long>(2 * y + ((k >> 1) & 1)) * w + 2 * x + (k & 1)], f);
#pragma unroll
			for (int c = 0; c < 8; ++c) s[c] += f[c];
		}
#pragma unroll
		for (int c = 0; c < 8; ++c) s[c] *= 0.125f;
		y_[oct * ovol + (static_cast<long long>(z) * oh + y) * ow + x] = pack8(s);
	}
}

__global__ void pool2_grad_kernel(const uint4* dy_, int octets, int d, int h, int w, uint4* dx_, const uint4* mask_,
	int accumulate)
{
	const long long ivol = static_cast<long long>(d) * h * w, ovol = ivol / 8;
	IANE_GB_C8_LOOP(d, h, w, octets)
	{
		const int z = zo % d, oct = zo / d;
		const long long at = oct * ivol + (static_cast<long long>(z) * h + y) * w + x;
		float g[8], m[8], prev[8];
		unpack8(dy_[oct * ovol + (static_cast<long long>(z / 2) * (h / 2) + y / 2) * (w / 2) + x / 2], g);
		if (accumulate) unpack8(dx_[at], prev);
		if (mask_) unpack8(mask_[at], m);
#pragma unroll
		for (int c = 0; c < 8; ++c) {
			g[c] *= 0.125f;
			if (accumulate) g[c] += prev[c];
			if (mask_ && !(m[c] > 0.0f)) g[c] = 0.0f;
		}
		dx_[at] = pack8(g);
	}
}

__global__ void up2_kernel(const uint4* x_, int octets, int d, int h, int w, uint4* y_)
{
	const int od = 2 * d, oh = 2 * h, ow = 2 * w;
	const long long ivol = static_cast<long long>(d) * h * w, ovol = 8 * ivol;
	IANE_GB_C8_LOOP(od, oh, ow, octets)
	{
		const int z = zo % od, oct = zo / od;
		y_[oct * ovol + (static_cast<long long>(z) * oh + y) * ow + x] =
			x_[oct * ivol + (static_cast<long long>(z / 2) * h + y / 2) * w + x / 2];
	}
}

__global__ void up2_grad_kernel(const uint4* dy_, int octets, int d, int h, int w, uint4* dx_, const uint4* mask_)
{
	const long long ivol = static_cast<long long>(d) * h * w, ovol = 8 * ivol;
	IANE_GB_C8_LOOP(d, h, w, octets)
	{
		const int z = zo % d, oct = zo / d;
		const uint4* src = dy_ + oct * ovol;
		float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
		for (int k = 0; k < 8; ++k) {
			float f[8];
			unpack8(src[(2LL * z + (k >> 2)) * 4 * h * w + static_cast<long long>(2 * y + ((k >> 1) & 1)) * 2 * w + 2 * x + (k & 1)], f);
#pragma unroll
			for (int c = 0; c < 8; ++c) s[c] += f[c];
		}
		const long long at = oct * ivol + (static_cast<long long>(z) * h + y) * w + x;
		if (mask_) {
			float m[8];
			unpack8(mask_[at], m);
#pragma unroll
			for (int c = 0; c < 8; ++c) if (!(m[c] > 0.0f)) s[c] = 0.0f;
		}
		dx_[at] = pack8(s);
	}
}
#undef IANE_GB_C8_LOOP

// loss = sum (y - t)^2 / n (FP64 accumulation per CTA, atomically added), dy = 2 (y - t) / n
// (a one-channel C8 tensor: slot 0 of each voxel's octet).
__global__ void mse_kernel(const float* y, const float* t, long long n, uint16_t* dy, double* loss)
{
	double s = 0.0;
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const float e = y[i] - t[i];
		s += static_cast<double>(e) * e;
		dy[i * 8] = to_bf(2.0f * e / static_cast<float>(n));  // one channel, C8 layout
	}
	__shared__ double red[32];
	for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
	__syncthreads();
	if (threadIdx.x == 0) {
		double v = 0.0;
		for (int i = 0; i < static_cast<int>(blockDim.x >> 5); ++i) v += red[i];
		atomicAdd(loss, v / static_cast<double>(n));
	}
}

// Adam on FP32 master parameters, refreshing their BF16 copies (grad scaled by `scale`).
__global__ void adam_kernel(float* p, uint16_t* p16, const float* g, float* m, float* v, long long n, float lr, float b1,
	float b2, float eps, float c1, float c2, float scale)
{
	for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
	     i += static_cast<long long>(gridDim.x) * blockDim.x) {
		const float gi = g[i] * scale;
		const float mi = b1 * m[i] + (1.0f - b1) * gi;
		const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
		m[i] = mi;
		v[i] = vi;
		const float upd = lr * (mi / c1) / (sqrtf(vi / c2) + eps);
		p[i] -= upd;
		if (p16) p16[i] = to_bf(p[i]);
	}
}

// Voxel chunks of the split-K weight gradient: about four CTAs per SM in all.
long long wgrad_chunks(int c0, int c1, int d, int h, int w, int co)
{
	const long long bricks = static_cast<long long>((w + BX - 1) / BX) * ((h + BY - 1) / BY) * ((d + BZ - 1) / BZ);
	const int co_tiles = (co + WG_CO - 1) / WG_CO;
	const int octets = (c0 + 7) / 8 + (c1 + 7) / 8;
	long long chunks = (4LL * device_sm_count()) / (co_tiles * octets);
	return chunks < 1 ? 1 : (chunks > bricks ? bricks : chunks);
}

bool aligned16(const void* p) { return reinterpret_cast<uintptr_t>(p) % 16 == 0; }

// Grid of the C8 elementwise kernels: 128 threads along x, one block row per y, (z, octet)
// pairs along grid z (capped; the kernels stride over the rest).
dim3 c8_grid(int ow, int oh, long long zo)
{
	return dim3(static_cast<unsigned>((ow + 127) / 128), static_cast<unsigned>(oh),
		static_cast<unsigned>(zo < 65535 ? zo : 65535));
}

int grid1(long long n)
{
	const long long b = (n + 255) / 256;
	const long long cap = 16LL * device_sm_count();
	return static_cast<int>(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace
}  // namespace iane_gb

using namespace iane_gb;

extern "C" {

int iane_gb_cnn_conv3(const uint16_t* x0, int c0, const uint16_t* x1, int c1, int d, int h, int w, const uint16_t* weights,
	const float* bias, int co, uint16_t* y16, float* y32, const float* residual, int act, const uint16_t* mask,
	void* stream)
{
	if (!x0 || c0 < 1 || c1 < 0 || (c1 > 0 && !x1) || d < 1 || h < 1 || w < 1 || !weights || co < 1 || co > 64 ||
	    (!y16 && !y32) || (residual && co != 1)) {
		return fail(IANE_GB_INVALID_ARGUMENT, "cnn_conv3: bad arguments");
	}
	Conv3Args a{x0, x1, c0, c1, d, h, w, weights, bias, co, y16, y32, residual, act, mask, (w + BX - 1) / BX,
		(h + BY - 1) / BY};
	const dim3 grid(a.bricks_x * a.bricks_y, (d + BZ - 1) / BZ);
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	if (grid.y > 65535) return fail(IANE_GB_UNSUPPORTED, "cnn_conv3: volume too deep");
	if (co <= 4) {
		conv3_kernel<4><<<grid, NT, 0, st>>>(a);
	} else if (co <= 16) {
		conv3_kernel<16><<<grid, NT, 0, st>>>(a);
	} else if (co <= 32) {
		conv3_kernel<32><<<grid, NT, 0, st>>>(a);
	} else {
		conv3_kernel<64><<<grid, NT, 0, st>>>(a);
	}
	IANE_GB_CUDA(cudaGetLastError(), "cnn_conv3: launch");
	return IANE_GB_OK;
}

size_t iane_gb_cnn_wgrad_scratch_bytes(int c0, int c1, int d, int h, int w, int co)
{
	const long long chunks = wgrad_chunks(c0, c1, d, h, w, co);
	return static_cast<size_t>(chunks) * co * ((c0 + c1) * 27 + 1) * sizeof(float);
}

int iane_gb_cnn_conv3_wgrad(const uint16_t* x0, int c0, const uint16_t* x1, int c1, int d, int h, int w,
	const uint16_t* dy, int co, float* dw, float* db, void* scratch, size_t scratch_bytes, void* stream)
{
	if (!x0 || c0 < 1 || c1 < 0 || (c1 > 0 && (!x1 || c0 % 8 != 0)) || !dy || !dw || co < 1 || co > 64 || !scratch ||
	    d < 1 || h < 1 || w < 1) {
		return fail(IANE_GB_INVALID_ARGUMENT, "cnn_conv3_wgrad: bad arguments");
	}
	if (reinterpret_cast<uintptr_t>(x0) % 16 || reinterpret_cast<uintptr_t>(x1) % 16) {
		return fail(IANE_GB_INVALID_ARGUMENT, "cnn_conv3_wgrad: inputs must be 16-byte aligned");
	}
	if (scratch_bytes < iane_gb_cnn_wgrad_scratch_bytes(c0, c1, d, h, w, co)) {
		return fail(IANE_GB_LENGTH_ERROR, "cnn_conv3_wgrad: scratch too small");
	}
	const int bx = (w + BX - 1) / BX, by = (h + BY - 1) / BY, bz = (d + BZ - 1) / BZ;
	const long long bricks = static_cast<long long>(bx) * by * bz;
	const int co_tiles = (co + WG_CO - 1) / WG_CO;
	const int ci_total = c0 + c1;
	const int octets = (c0 + 7) / 8 + (c1 + 7) / 8;
	const long long chunks = wgrad_chunks(c0, c1, d, h, w, co);
	WgradArgs a{};
	a.x0 = x0;
	a.x1 = x1;
	a.c0 = c0;
	a.c1 = c1;
	a.d = d;
	a.h = h;
	a.w = w;
	a.dy = dy;
	a.co = co;
	a.chunk_bricks = static_cast<int>((bricks + chunks - 1) / chunks);
	a.bricks_x = bx;
	a.bricks_y = by;
	a.bricks_total = static_cast<int>(bricks);
	a.partial = static_cast<float*>(scratch);
	a.chunks = static_cast<int>(chunks);
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	conv3_wgrad_kernel<<<dim3(co_tiles, octets, static_cast<unsigned>(chunks)), WG_THREADS, 0, st>>>(a);
	const long long nw = static_cast<long long>(co) * ci_total * 27;
	conv3_wgrad_reduce<<<grid1(nw + co), 256, 0, st>>>(a.partial, a.chunks, nw, co, dw, db);
	IANE_GB_CUDA(cudaGetLastError(), "cnn_conv3_wgrad: launch");
	return IANE_GB_OK;
}

int iane_gb_cnn_flip(const uint16_t* weights, int co, int ci, uint16_t* flipped, void* stream)
{
	if (!weights || !flipped || co < 1 || ci < 1) return fail(IANE_GB_INVALID_ARGUMENT, "cnn_flip: bad arguments");
	const long long n = static_cast<long long>(co) * ci * 27;
	flip_kernel<<<grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(weights, co, ci, flipped);
	IANE_GB_CUDA(cudaGetLastError(), "cnn_flip: launch");
	return IANE_GB_OK;
}

int iane_gb_cnn_pool2(const uint16_t* x, int c, int d, int h, int w, uint16_t* y, void* stream)
{
	if (!x || !y || c < 1 || d % 2 || h % 2 || w % 2 || d < 2 || !aligned16(x) || !aligned16(y) || h / 2 > 65535) {
		return fail(IANE_GB_INVALID_ARGUMENT, "cnn_pool2: even extents, 16-byte aligned C8 tensors");
	}
	const int oct = (c + 7) / 8;
	pool2_kernel<<<c8_grid(w / 2, h / 2, d / 2 * oct), 128, 0, static_cast<cudaStream_t>(stream)>>>(
		reinterpret_cast<const uint4*>(x), oct, d, h, w, reinterpret_cast<uint4*>(y));
	IANE_GB_CUDA(cudaGetLastError(), "cnn_pool2: launch");
	return IANE_GB_OK;
}

int iane_gb_cnn_pool2_grad(const uint16_t* dy, int c, int d, int h, int w, uint16_t* dx, const uint16_t* mask,
	int accumulate, void* stream)
{
	if (!dy || !dx || c < 1 || d % 2 || h % 2 || w % 2 || !aligned16(dy) || !aligned16(dx) || !aligned16(mask) || h > 65535) {
		return fail(IANE_GB_INVALID_ARGUMENT, "cnn_pool2_grad: even extents, 16-byte aligned C8 tensors");
	}
	const int oct = (c + 7) / 8;
	pool2_grad_kernel<<<c8_grid(w, h, d * oct), 128, 0, static_cast<cudaStream_t>(stream)>>>(
		reinterpret_cast<const uint4*>(dy), oct, d, h, w, reinterpret_cast<uint4*>(dx), reinterpret_cast<const uint4*>(mask),
		accumulate);
	IANE_GB_CUDA(cudaGetLastError(), "cnn_pool2_grad: launch");
	return IANE_GB_OK;
}

int iane_gb_cnn_up2(const uint16_t* x, int c, int d, int h, int w, uint16_t* y, void* stream)
{
	if (!x || !y || c < 1 || d < 1 || h < 1 || w < 1 || !aligned16(x) || !aligned16(y) || 2 * h > 65535) {
		return fail(IANE_GB_INVALID_ARGUMENT, "cnn_up2: bad arguments");
	}
	const int oct = (c + 7) / 8;
	up2_kernel<<<c8_grid(2 * w, 2 * h, 2 * d * oct), 128, 0, static_cast<cudaStream_t>(stream)>>>(
		reinterpret_cast<const uint4*>(x), oct, d, h, w, reinterpret_cast<uint4*>(y));
	IANE_GB_CUDA(cudaGetLastError(), "cnn_up2: launch");
	return IANE_GB_OK;
}

int iane_gb_cnn_up2_grad(const uint16_t* dy, int c, int d, int h, int w, uint16_t* dx, const uint16_t* mask,
	void* stream)
{
	if (!dy || !dx || c < 1 || d < 1 || h < 1 || w < 1 || !aligned16(dy) || !aligned16(dx) || !aligned16(mask) ||
	    h > 65535) {
		return fail(IANE_GB_INVALID_ARGUMENT, "cnn_up2_grad: bad arguments");
	}
	const int oct = (c + 7) / 8;
	up2_grad_kernel<<<c8_grid(w, h, d * oct), 128, 0, static_cast<cudaStream_t>(stream)>>>(
		reinterpret_cast<const uint4*>(dy), oct, d, h, w, reinterpret_cast<uint4*>(dx), reinterpret_cast<const uint4*>(mask));
	IANE_GB_CUDA(cudaGetLastError(), "cnn_up2_grad: launch");
	return IANE_GB_OK;
}

int iane_gb_cnn_mse(const float* y, const float* target, long long n, uint16_t* dy, double* loss, void* stream)
{
	if (!y || !target || !dy || !loss || n < 1) return fail(IANE_GB_INVALID_ARGUMENT, "cnn_mse: bad arguments");
	mse_kernel<<<grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(y, target, n, dy, loss);
	IANE_GB_CUDA(cudaGetLastError(), "cnn_mse: launch");
	return IANE_GB_OK;
}

int iane_gb_cnn_adam(float* params, uint16_t* params16, const float* grads, float* m, float* v, long long n, float lr,
	float beta1, float beta2, float eps, int step, float grad_scale, void* stream)
{
	if (!params || !grads || !m || !v || n < 1 || step < 1) return fail(IANE_GB_INVALID_ARGUMENT, "cnn_adam: bad arguments");
	const float c1 = 1.0f - powf(beta1, static_cast<float>(step));
	const float c2 = 1.0f - powf(beta2, static_cast<float>(step));
	adam_kernel<<<grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(params, params16, grads, m, v, n, lr, beta1,
		beta2, eps, c1, c2, grad_scale);
	IANE_GB_CUDA(cudaGetLastError(), "cnn_adam: launch");
	return IANE_GB_OK;
}

}  // extern "C"
