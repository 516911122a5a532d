// Host-side launchers shared between the library's translation units.
#pragma once

#include "common.cuh"

namespace iane_gb {

// Generic direct convolution (conv_generic.cu): any supported element types, border and
// strides; exact = FP64 fma in kernel raster order.
int launch_conv_generic(const DevView& src, const DevView& kernel, const DevView& dst, int border, bool exact,
	cudaStream_t stream, const TexSource* tex = nullptr);

// Register-tiled FP32 convolution (conv_f32.cu). Returns IANE_GB_UNSUPPORTED (without
// recording an error) when the shapes are outside what the tiled path takes, so that the
// caller falls back to the generic kernel.
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

// Bandwidth-oriented fused separable FP32 convolution for radii <= 7 (separable_fast.cu);
// IANE_GB_UNSUPPORTED without an error when it does not apply.
int launch_conv_separable_fast(const DevView& src, const DevView* taps, const DevView& dst, int border,
	cudaStream_t stream);

// Fused separable FP32 convolution, any tap length (separable.cu).
// Large 2-D f32 images (separable_rows.cu): IANE_GB_UNSUPPORTED when the view or radius does
// not qualify.
int launch_separable_rows(const DevView& src, const DevView* taps, const DevView& dst, int border,
	cudaStream_t stream);
int launch_conv_separable(const DevView& src, const DevView* taps, const DevView& dst, int border,
	cudaStream_t stream);

}  // namespace iane_gb
