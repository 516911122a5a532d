// Richardson-Lucy epilogues for the tiled convolution core (conv_tile.cuh): the pointwise
// steps of the reference's RL example (examples/rl_deconvolution/main.cu:22-49) fused into
// the convolution that produces their operand, so one iteration is two passes over HBM:
//
//   pass A:  ratio    = observed / max(conv(estimate, psf), eps)               (EpiRatio)
//   pass B:  estimate = estimate * edge(conv(ratio, adjoint), sensitivity)     (EpiUpdate)
//
// with edge(c, s) = s > 0 ? c / max(s, eps) : 0. Both divisions are IEEE (no fast math), as
// in the reference. The sensitivity image is never stored: it is exactly the zero-border
// response of the adjoint to an image of ones, which depends only on how far each voxel
// is from the faces, so it is read from a small per-class table outside the interior and
// is a single constant inside.
#pragma once

#include "conv_tile.cuh"

namespace iane_gb {

struct EpiRatio {
	float* ratio;       // packed-pitch work image
	long long pitch;    // floats per row
	long long plane;    // floats per plane
	const char* obs;    // observed view (u8 or f32, any strides)
	long long os[3];
	int obs_u8;
	float eps;
	int nx, ny;

	__device__ __forceinline__ float observed(int x, int y, int z) const
	{
		const char* p = obs + x * os[0] + y * os[1] + z * os[2];
		return obs_u8 ? static_cast<float>(*reinterpret_cast<const uint8_t*>(p)) : *reinterpret_cast<const float*>(p);
	}

	// N outputs of one row starting at xo (N a multiple of 4; xo a multiple of 4)
	template<int N>
	__device__ __forceinline__ void row(int xo, int y, int z, const float (&v)[N]) const
	{
		if (y >= ny) {
			return;
		}
		float r[N];
#pragma unroll
		for (int i = 0; i < N; ++i) {
			const float p = v[i];
			r[i] = xo + i < nx ? observed(xo + i, y, z) / (p > eps ? p : eps) : 0.0f;
		}
		float* out = ratio + z * plane + y * pitch + xo;
		if (xo + N <= nx) {
#pragma unroll
			for (int m = 0; m < N / 4; ++m) {
				reinterpret_cast<float4*>(out)[m] = make_float4(r[4 * m], r[4 * m + 1], r[4 * m + 2], r[4 * m + 3]);
			}
		} else {
#pragma unroll
			for (int i = 0; i < N; ++i) {
				if (xo + i < nx) out[i] = r[i];
			}
		}
	}
	__device__ __forceinline__ void finish() const {}
};

__device__ __forceinline__ void kahan_add(float& sum, float& comp, float value)
{
	const float y = value - comp;
	const float t = sum + y;
	comp = (t - sum) - y;
	sum = t;
}

__device__ __forceinline__ uint8_t to_gray8(float v)
{
	// examples/common/deconvolution.hpp:43-55
	if (!(v > 0.0f)) return 0;
	if (v >= 255.0f) return 255;
	const unsigned int integer = static_cast<unsigned int>(v);
	return static_cast<uint8_t>(integer + (v - integer >= 0.5f));
}

struct EpiUpdate {
	float* est;          // packed-pitch work estimate, read and written in place
	long long pitch, plane;
	float eps;
	int nx, ny, nz;
	// sensitivity: class index per coordinate (x at 0, y at nx, z at nx + ny) and table
	const int* cls;
	const float* sens;
	int cx_count, cy_count;
	int ilo[3], ihi[3];  // interior coordinate range per axis (empty if ilo > ihi)
	float s_interior;
	// statistics (optional)
	int want_stats;
	double* partials;    // 3 doubles per block
	unsigned int* counter;
	double* stats;       // 2 doubles for this iteration
	// final output (optional): the caller's view when it is not the work estimate
	int write_out;
	char* out;
	long long outs[3];
	int out_u8;
	// per-thread Kahan state
	float f_s, f_c, c_s, c_c, n_s, n_c;

	// N outputs of one row starting at xo (N a multiple of 4; xo a multiple of 4)
	template<int N>
	__device__ __forceinline__ void row(int xo, int y, int z, const float (&v)[N])
	{
		if (y >= ny) {
			return;
		}
		const bool interior = xo >= ilo[0] && xo + N - 1 <= ihi[0] && y >= ilo[1] && y <= ihi[1] &&
			z >= ilo[2] && z <= ihi[2];
		float* e = est + z * plane + y * pitch + xo;
		float old[N];
		const bool full = xo + N <= nx;
		if (full) {
#pragma unroll
			for (int m = 0; m < N / 4; ++m) {
				const float4 a = reinterpret_cast<const float4*>(e)[m];
				old[4 * m] = a.x; old[4 * m + 1] = a.y; old[4 * m + 2] = a.z; old[4 * m + 3] = a.w;
			}
		} else {
#pragma unroll
			for (int i = 0; i < N; ++i) old[i] = xo + i < nx ? e[i] : 0.0f;
		}
		float upd[N];
		const int cyz = interior ? 0 : cx_count * (cls[nx + y] + cy_count * cls[nx + ny + z]);
#pragma unroll
		for (int i = 0; i < N; ++i) {
			float s = s_interior;
			if (!interior && xo + i < nx) {
				s = sens[cls[xo + i] + cyz];
			}
			const float factor = s > 0.0f ? v[i] / (s > eps ? s : eps) : 0.0f;
			upd[i] = old[i] * factor;
		}
		if (full) {
#pragma unroll
			for (int m = 0; m < N / 4; ++m) {
				reinterpret_cast<float4*>(e)[m] = make_float4(upd[4 * m], upd[4 * m + 1], upd[4 * m + 2], upd[4 * m + 3]);
			}
		} else {
#pragma unroll
			for (int i = 0; i < N; ++i) {
				if (xo + i < nx) e[i] = upd[i];
			}
		}
#pragma unroll
		for (int i = 0; i < N; ++i) {
			if (xo + i < nx) {
				if (want_stats) {
					kahan_add(f_s, f_c, upd[i]);
					const float d = upd[i] - old[i];
					kahan_add(c_s, c_c, d * d);
					kahan_add(n_s, n_c, old[i] * old[i]);
				}
				if (write_out) {
					char* p = out + (xo + i) * outs[0] + y * outs[1] + z * outs[2];
					if (out_u8) {
						*reinterpret_cast<uint8_t*>(p) = to_gray8(upd[i]);
					} else {
						*reinterpret_cast<float*>(p) = upd[i];
					}
				}
			}
		}
	}

	// Block partials in FP64, then the last block to finish combines all partials in block
	// order (deterministic) and writes this iteration's flux and relative change.
	__device__ void finish()
	{
		if (!want_stats) {
			return;
		}
		extern __shared__ __align__(128) unsigned char smem_raw[];
		double* red = reinterpret_cast<double*>(smem_raw); // the halo tiles are no longer read
		int& last_block = *reinterpret_cast<int*>(red + 3 * 32);
		double v[3] = {static_cast<double>(f_s) - static_cast<double>(f_c),
			static_cast<double>(c_s) - static_cast<double>(c_c), static_cast<double>(n_s) - static_cast<double>(n_c)};
#pragma unroll
		for (int k = 0; k < 3; ++k) {
#pragma unroll
			for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
		}
		const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
		__syncthreads();
		if (lane == 0) {
			for (int k = 0; k < 3; ++k) red[warp * 3 + k] = v[k];
		}
		__syncthreads();
		const unsigned int nblocks = gridDim.x * gridDim.y * gridDim.z;
		const unsigned int block = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
		if (threadIdx.x == 0) {
			double t[3] = {0.0, 0.0, 0.0};
			for (int w = 0; w < warps; ++w)
				for (int k = 0; k < 3; ++k) t[k] += red[w * 3 + k];
			for (int k = 0; k < 3; ++k) partials[block * 3 + k] = t[k];
			__threadfence();
			const unsigned int ticket = atomicAdd(counter, 1u);
			last_block = ticket == nblocks - 1;
		}
		__syncthreads();
		if (!last_block) {
			return;
		}
		__threadfence();
		double t[3] = {0.0, 0.0, 0.0};
		for (unsigned int b = threadIdx.x; b < nblocks; b += blockDim.x) {
			for (int k = 0; k < 3; ++k) t[k] += __ldcg(&partials[b * 3 + k]);
		}
#pragma unroll
		for (int k = 0; k < 3; ++k) {
#pragma unroll
			for (int off = 16; off > 0; off >>= 1) t[k] += __shfl_down_sync(0xffffffffu, t[k], off);
		}
		__syncthreads();
		if (lane == 0) {
			for (int k = 0; k < 3; ++k) red[warp * 3 + k] = t[k];
		}
		__syncthreads();
		if (threadIdx.x == 0) {
			double s[3] = {0.0, 0.0, 0.0};
			for (int w = 0; w < warps; ++w)
				for (int k = 0; k < 3; ++k) s[k] += red[w * 3 + k];
			stats[0] = s[0];
			stats[1] = s[2] > 0.0 ? sqrt(s[1] / s[2]) : 0.0;
			*counter = 0u;
		}
	}
};

// Pitch (floats) of the shared-memory halo tile, i.e. the TMA box width, for a kernel
// width kx and WX warps along x. Mirrors TileWidth<KX, WX>::P.
inline int tile_pitch(int kx, int wx)
{
	const int rx = kx / 2;
	const int rxa = (rx + 3) & ~3;
	const int d = rxa - rx;
	const int segn = (d + kRX + kx - 1 + 3) & ~3;
	const int w = 32 * wx - kRX + segn;
	return (w % 8 == 0) ? w + 4 : w;
}

// Launch pass A / pass B for a runtime kx (rl_pass_*.cu). small = 32x32 tiles.
int launch_rl_pass_a(int kx, bool small, const CUtensorMap& map, const TileArgs& a, const EpiRatio& e,
	cudaStream_t stream);
int launch_rl_pass_b(int kx, bool small, const CUtensorMap& map, const TileArgs& a, const EpiUpdate& e,
	cudaStream_t stream);

}  // namespace iane_gb
