// Host-side launchers shared between the library's translation units.
#pragma once

#include "common.cuh"

#include <algorithm>

namespace iane_gb {

// Row chunks per strip for the row-marching kernels (a block per strip and chunk, marching
// down the chunk in steps of `step_rows` rows): the grid of strips x chunks blocks is sized to
// fill whole waves of `slots` resident blocks as closely as possible -- the blocks of a partly
// filled last wave run while most of the GPU idles -- and each chunk loads about one step of
// rows beyond its own, so longer chunks are preferred where the fill is equal. Chunks are at
// least four steps tall.
inline int strip_chunks(long long strips, int ny, long long slots, int step_rows)
{
	int best = 1;
	double best_score = -1.0;
	const long long most = std::max(1, ny / (4 * step_rows));
	for (long long waves = 1; waves <= 8; ++waves) {
		const long long chunks = std::min(most, std::max(1LL, waves * slots / strips));
		const long long blocks = strips * chunks;
		const long long used = (blocks + slots - 1) / slots;
		const double fill = static_cast<double>(blocks) / static_cast<double>(used * slots);
		const double score = fill / (1.0 + static_cast<double>(step_rows) * static_cast<double>(chunks) / ny);
		if (score > best_score + 1e-9) {
			best_score = score;
			best = static_cast<int>(chunks);
		}
	}
	return best;
}

// Generic direct convolution (conv_generic.cu): any supported element types, border and
// strides; exact = FP64 fma in kernel raster order.
int launch_conv_generic(const DevView& src, const DevView& kernel, const DevView& dst, int border, bool exact,
	cudaStream_t stream, const TexSource* tex = nullptr);

// Spectral convolution (conv_fft.cu): cuFFT FP64 transforms over the border-padded source.
bool conv_fft_supported(const DevView& src, const DevView& kernel, const DevView& dst);
void conv_cost_model(const DevView& src, const DevView& kernel, double& direct_s, double& fft_s);
int launch_conv_fft(const DevView& src, const DevView& kernel, const DevView& dst, int border, cudaStream_t stream);

// iane_gb_convolve after view normalisation: argument checks and dispatch; `tex` (if set)
// is the source of samples, `s` then gives its extents and texel type.
int convolve_checked(const DevView& s, const DevView& k, const DevView& d, int border, unsigned flags, void* stream,
	const TexSource* tex);

// The tiled FP32 fast path for an f32 kernel; `tex` (if set) replaces src as the source of
// samples (src then only gives extents and the texel type). IANE_GB_UNSUPPORTED when the
// combination is not its own (the caller falls back to the generic kernel).
int launch_conv_f32_tiled(const DevView& src, const DevView& kernel, const DevView& dst, int border,
	cudaStream_t stream, const TexSource* tex = nullptr);

// Row-strip direct FP32 convolution of large 2-D f32 images (or stacks of 2-D planes under a
// kernel one plane deep) with kernels of odd extents up to 7, line filters included
// (direct_rows.cu); the same bits as the tiled kernel. IANE_GB_UNSUPPORTED without an error
// when the views or the kernel do not qualify.
int launch_direct_rows(const DevView& src, const DevView& kernel, const DevView& dst, int border,
	cudaStream_t stream);

// Bandwidth-oriented fused separable FP32 convolution for radii <= 7 (separable_fast.cu);
// IANE_GB_UNSUPPORTED without an error when it does not apply.
int launch_conv_separable_fast(const DevView& src, const DevView* taps, const DevView& dst, int border,
	cudaStream_t stream);

// Large 2-D f32 images (separable_rows.cu): IANE_GB_UNSUPPORTED when the view or radius does
// not qualify.
int launch_separable_rows(const DevView& src, const DevView* taps, const DevView& dst, int border,
	cudaStream_t stream);

// Fused separable FP32 convolution, any tap length (separable.cu).
int launch_conv_separable(const DevView& src, const DevView* taps, const DevView& dst, int border,
	cudaStream_t stream);

}  // namespace iane_gb
