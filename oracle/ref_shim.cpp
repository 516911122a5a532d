// extern "C" entry points around the reference's own CPU convolution, compiled from the
// reference headers where they lie (never copied) into oracle/_ref/libiane_ref.so by
// oracle/build.py. TEST INFRASTRUCTURE ONLY: it pins the C oracle (oracle/iane_oracle.c)
// and generates the golden vectors in tests/golden/. It is built only where the
// reference sources are present; the GPU host uses the C oracle instead.
//
// ref_convolve calls iane::convolve (include/iane/algorithms/convolution.hpp:97-117)
// on host views with the caller's byte strides and iane::cpu_policy{threads}.
// ref_rl restates prepare_rl (examples/rl_deconvolution/main.cu:51-81) from the
// reference's own convolve / constant_view / zip_view / copy / transform on
// host_image<float, N>, with float observed data and a selectable start.
#include "../include/iane_gb/capi.h"

#include <iane/algorithms/convolution.hpp>
#include <iane/algorithms/copy.hpp>
#include <iane/algorithms/morphology/morphology.hpp>
#include <iane/image/image.hpp>
#include <iane/resource/host/resource_host.hpp>
#include <iane/view/make_view.hpp>
#include <iane/view/procedural.hpp>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <exception>
#include <type_traits>

namespace {

template<int tDim>
using extents_t = typename iane::math::dim_traits<tDim>::extents_t;

template<int tDim>
extents_t<tDim> to_extents(const int32_t* values)
{
	extents_t<tDim> out{};
	for (int i = 0; i < tDim; ++i) {
		iane::math::detail::axis(out, i) = values[i];
	}
	return out;
}

template<int tDim>
extents_t<tDim> to_strides(const int64_t* values)
{
	extents_t<tDim> out{};
	for (int i = 0; i < tDim; ++i) {
		iane::math::detail::axis(out, i) = static_cast<int>(values[i]);
	}
	return out;
}

// A packed byte (r, g, b) pixel and its per-channel double sum, with the element semantics of
// the custom pixel in the reference's convolution example (examples/convolution/main.cu:20-56):
// the product with a float tap is taken in double per channel, sums add channel by channel,
// and the conversion back rounds each channel half up and saturates to a byte.
struct pixel3 {
	std::uint8_t c[3];
};
static_assert(sizeof(pixel3) == 3);

struct pixel3_sum {
	double c[3];

	pixel3_sum operator+(const pixel3_sum& aOther) const
	{
		return {{c[0] + aOther.c[0], c[1] + aOther.c[1], c[2] + aOther.c[2]}};
	}

	explicit operator pixel3() const
	{
		pixel3 out{};
		for (int i = 0; i < 3; ++i) {
			const double v = c[i];
			if (!(v > 0.0)) {
				out.c[i] = 0;
			} else if (v >= 255.0) {
				out.c[i] = 255;
			} else {
				const auto whole = static_cast<unsigned int>(v);
				out.c[i] = static_cast<std::uint8_t>(whole + (v - whole >= 0.5 ? 1u : 0u));
			}
		}
		return out;
	}
};

pixel3_sum operator*(pixel3 aPixel, float aTap)
{
	const double tap = aTap;
	return {{aPixel.c[0] * tap, aPixel.c[1] * tap, aPixel.c[2] * tap}};
}

template<class TSrc, class TKernel, class TDst, int tDim>
int convolve_typed(const iane_gb_view& aSrc, const iane_gb_view& aKernel, const iane_gb_view& aDst,
	int aBorder, int aThreads)
{
	const iane::const_host_image_view<TSrc, tDim> src(static_cast<const TSrc*>(aSrc.ptr),
		to_extents<tDim>(aSrc.extent), to_strides<tDim>(aSrc.stride));
	const iane::const_host_image_view<TKernel, tDim> kernel(static_cast<const TKernel*>(aKernel.ptr),
		to_extents<tDim>(aKernel.extent), to_strides<tDim>(aKernel.stride));
	const iane::host_image_view<TDst, tDim> dst(static_cast<TDst*>(aDst.ptr),
		to_extents<tDim>(aDst.extent), to_strides<tDim>(aDst.stride));
	const iane::convolution_options options{
		.border = aBorder == IANE_GB_BORDER_ZERO ? iane::border_mode::zero : iane::border_mode::clamp};
	iane::convolve(src, kernel, dst, options,
		iane::cpu_policy{.threads = static_cast<std::size_t>(aThreads < 1 ? 1 : aThreads)}).wait();
	return 0;
}

template<class TSrc, class TKernel, class TDst>
int convolve_rank(const iane_gb_view& aSrc, const iane_gb_view& aKernel, const iane_gb_view& aDst,
	int aBorder, int aThreads)
{
	switch (aSrc.rank) {
	case 1: return convolve_typed<TSrc, TKernel, TDst, 1>(aSrc, aKernel, aDst, aBorder, aThreads);
	case 2: return convolve_typed<TSrc, TKernel, TDst, 2>(aSrc, aKernel, aDst, aBorder, aThreads);
	case 3: return convolve_typed<TSrc, TKernel, TDst, 3>(aSrc, aKernel, aDst, aBorder, aThreads);
	default: return IANE_GB_UNSUPPORTED;
	}
}

#define IANE_REF_COMBO(S, K, D, TS, TK, TD) \
	if (aSrc.dtype == S && aKernel.dtype == K && aDst.dtype == D) \
		return convolve_rank<TS, TK, TD>(aSrc, aKernel, aDst, aBorder, aThreads);

int dispatch(const iane_gb_view& aSrc, const iane_gb_view& aKernel, const iane_gb_view& aDst,
	int aBorder, int aThreads)
{
	IANE_REF_COMBO(IANE_GB_F32, IANE_GB_F32, IANE_GB_F32, float, float, float)
	IANE_REF_COMBO(IANE_GB_F64, IANE_GB_F64, IANE_GB_F64, double, double, double)
	IANE_REF_COMBO(IANE_GB_F32, IANE_GB_F32, IANE_GB_F64, float, float, double)
	IANE_REF_COMBO(IANE_GB_U8, IANE_GB_F32, IANE_GB_U8, std::uint8_t, float, std::uint8_t)
	IANE_REF_COMBO(IANE_GB_U8, IANE_GB_F32, IANE_GB_F32, std::uint8_t, float, float)
	IANE_REF_COMBO(IANE_GB_U8, IANE_GB_I32, IANE_GB_U8, std::uint8_t, std::int32_t, std::uint8_t)
	IANE_REF_COMBO(IANE_GB_U16, IANE_GB_I32, IANE_GB_U16, std::uint16_t, std::int32_t, std::uint16_t)
	IANE_REF_COMBO(IANE_GB_I16, IANE_GB_I32, IANE_GB_I16, std::int16_t, std::int32_t, std::int16_t)
	IANE_REF_COMBO(IANE_GB_I32, IANE_GB_I32, IANE_GB_I32, std::int32_t, std::int32_t, std::int32_t)
	IANE_REF_COMBO(IANE_GB_F32, IANE_GB_F32, IANE_GB_U8, float, float, std::uint8_t)
	IANE_REF_COMBO(IANE_GB_F32, IANE_GB_F32, IANE_GB_I32, float, float, std::int32_t)
	IANE_REF_COMBO(IANE_GB_U16, IANE_GB_F32, IANE_GB_F32, std::uint16_t, float, float)
	IANE_REF_COMBO(IANE_GB_I8, IANE_GB_F32, IANE_GB_I8, std::int8_t, float, std::int8_t)
	IANE_REF_COMBO(IANE_GB_I8, IANE_GB_I32, IANE_GB_I8, std::int8_t, std::int32_t, std::int8_t)
	IANE_REF_COMBO(IANE_GB_U32, IANE_GB_F32, IANE_GB_U32, std::uint32_t, float, std::uint32_t)
	IANE_REF_COMBO(IANE_GB_U32, IANE_GB_I32, IANE_GB_U32, std::uint32_t, std::int32_t, std::uint32_t)
	IANE_REF_COMBO(IANE_GB_F32, IANE_GB_F32, IANE_GB_I8, float, float, std::int8_t)
	IANE_REF_COMBO(IANE_GB_F32, IANE_GB_F32, IANE_GB_U32, float, float, std::uint32_t)
	IANE_REF_COMBO(IANE_GB_RGB8, IANE_GB_F32, IANE_GB_RGB8, pixel3, float, pixel3)
	return IANE_GB_UNSUPPORTED;
}

// The pointwise steps of examples/rl_deconvolution/main.cu:12-49 for float data.
struct observation_ratio {
	float epsilon;
	float operator()(float aObserved, float aPredicted) const
	{
		return aObserved / (aPredicted > epsilon ? aPredicted : epsilon);
	}
};

struct edge_correction {
	float epsilon;
	float operator()(float aBackprojection, float aSensitivity) const
	{
		return aSensitivity > 0.0f
			? aBackprojection / (aSensitivity > epsilon ? aSensitivity : epsilon)
			: 0.0f;
	}
};

struct multiply_estimate {
	float operator()(float aEstimate, float aCorrection) const { return aEstimate * aCorrection; }
};

template<int tDim>
int rl_typed(const float* aObserved, const int32_t* aExtent, const float* aPsf, const int32_t* aPsfExtent,
	int aIterations, float aEpsilon, int aInit, float* aEstimate, int aThreads)
{
	const auto size = to_extents<tDim>(aExtent);
	const auto psf_size = to_extents<tDim>(aPsfExtent);
	const iane::cpu_policy policy{.threads = static_cast<std::size_t>(aThreads < 1 ? 1 : aThreads)};
	const auto source = iane::host::make_const_view<float, tDim>(aObserved, size);
	const auto psf = iane::host::make_const_view<float, tDim>(aPsf, psf_size);
	const auto taps = iane::math::detail::element_count<tDim>(psf_size);
	iane::host_image<float, tDim> adjoint(psf_size);
	std::reverse_copy(aPsf, aPsf + taps, adjoint.pointer());
	const auto estimate = iane::host::make_view<float, tDim>(aEstimate, size);
	iane::host_image<float, tDim> predicted(size);
	iane::host_image<float, tDim> correction(size);
	iane::host_image<float, tDim> sensitivity(size);
	constexpr iane::convolution_options options{.border = iane::border_mode::zero};
	iane::convolve(iane::constant_view(sensitivity.view(), 1.0f), adjoint.const_view(),
		sensitivity.view(), options, policy).wait();
	const auto count = iane::math::detail::element_count<tDim>(size);
	if (aInit == IANE_GB_RL_INIT_MEAN) {
		double total = 0.0;
		for (std::size_t i = 0; i < count; ++i) {
			total += static_cast<double>(aObserved[i]);
		}
		const float mean = static_cast<float>(total / static_cast<double>(count));
		std::fill(aEstimate, aEstimate + count, mean > aEpsilon ? mean : aEpsilon);
	} else if (aInit == IANE_GB_RL_INIT_OBSERVED) {
		const float epsilon = aEpsilon;
		iane::transform(source, estimate,
			[epsilon](float aValue) { return aValue > epsilon ? aValue : epsilon; }, policy);
	}
	for (int iteration = 0; iteration < aIterations; ++iteration) {
		iane::convolve(iane::host::make_const_view<float, tDim>(aEstimate, size), psf,
			predicted.view(), options, policy);
		iane::copy(iane::zip_view(source, predicted.const_view(), observation_ratio{aEpsilon}),
			predicted.view(), policy);
		iane::convolve(predicted.const_view(), adjoint.const_view(), correction.view(), options, policy);
		const auto factor = iane::zip_view(correction.const_view(), sensitivity.const_view(),
			edge_correction{aEpsilon});
		iane::copy(iane::zip_view(iane::host::make_const_view<float, tDim>(aEstimate, size), factor,
			multiply_estimate{}), estimate, policy);
	}
	return 0;
}

// A footprint predicate over a mask of (2 r + 1) per axis in raster order.
template<int tDim>
struct mask_predicate {
	const std::uint8_t* mask;
	extents_t<tDim> radius;

	template<class TCoord>
	bool operator()(const TCoord& aOffset) const
	{
		long long index = 0, stride = 1;
		for (int i = 0; i < tDim; ++i) {
			const int r = iane::math::detail::axis(radius, i);
			index += (iane::math::detail::axis(aOffset, i) + r) * stride;
			stride *= 2 * r + 1;
		}
		return mask[index] != 0;
	}
};

template<class T, int tDim>
int morphology_typed(const iane_gb_view& aSrc, const iane_gb_view& aDst, const int32_t* aRadius,
	const std::uint8_t* aMask, int aDilate, int aBorder)
{
	const iane::const_host_image_view<T, tDim> src(static_cast<const T*>(aSrc.ptr),
		to_extents<tDim>(aSrc.extent), to_strides<tDim>(aSrc.stride));
	const iane::host_image_view<T, tDim> dst(static_cast<T*>(aDst.ptr),
		to_extents<tDim>(aDst.extent), to_strides<tDim>(aDst.stride));
	typename iane::math::dim_traits<tDim>::coord_t radius{};
	for (int i = 0; i < tDim; ++i) iane::math::detail::axis(radius, i) = aRadius[i];
	const iane::morphology_options options{
		.border = aBorder == IANE_GB_BORDER_ZERO ? iane::border_mode::zero : iane::border_mode::clamp};
	if (aMask) {
		const auto footprint = iane::make_flat_footprint(radius, mask_predicate<tDim>{aMask, to_extents<tDim>(aRadius)});
		if (aDilate) iane::dilate(src, dst, footprint, options).wait();
		else iane::erode(src, dst, footprint, options).wait();
	} else {
		const auto footprint = iane::box_footprint(radius);
		if (aDilate) iane::dilate(src, dst, footprint, options).wait();
		else iane::erode(src, dst, footprint, options).wait();
	}
	return 0;
}

template<class T>
int morphology_rank(const iane_gb_view& aSrc, const iane_gb_view& aDst, const int32_t* aRadius,
	const std::uint8_t* aMask, int aDilate, int aBorder)
{
	switch (aSrc.rank) {
	case 1: return morphology_typed<T, 1>(aSrc, aDst, aRadius, aMask, aDilate, aBorder);
	case 2: return morphology_typed<T, 2>(aSrc, aDst, aRadius, aMask, aDilate, aBorder);
	case 3: return morphology_typed<T, 3>(aSrc, aDst, aRadius, aMask, aDilate, aBorder);
	default: return IANE_GB_UNSUPPORTED;
	}
}

} // namespace

extern "C" {

// iane::erode / iane::dilate (include/iane/algorithms/morphology/morphology.hpp:172-206) on
// host views, box footprint (mask NULL) or a mask predicate.
int ref_morphology(const iane_gb_view* aSrc, const iane_gb_view* aDst, const int32_t* aRadius,
	const std::uint8_t* aMask, int aDilate, int aBorder)
{
	if (!aSrc || !aDst || !aRadius || aSrc->rank != aDst->rank || aSrc->dtype != aDst->dtype ||
	    (aBorder != IANE_GB_BORDER_ZERO && aBorder != IANE_GB_BORDER_CLAMP)) {
		return IANE_GB_INVALID_ARGUMENT;
	}
	try {
		switch (aSrc->dtype) {
		case IANE_GB_U8: return morphology_rank<std::uint8_t>(*aSrc, *aDst, aRadius, aMask, aDilate, aBorder);
		case IANE_GB_I16: return morphology_rank<std::int16_t>(*aSrc, *aDst, aRadius, aMask, aDilate, aBorder);
		case IANE_GB_I32: return morphology_rank<std::int32_t>(*aSrc, *aDst, aRadius, aMask, aDilate, aBorder);
		case IANE_GB_U32: return morphology_rank<std::uint32_t>(*aSrc, *aDst, aRadius, aMask, aDilate, aBorder);
		case IANE_GB_F32: return morphology_rank<float>(*aSrc, *aDst, aRadius, aMask, aDilate, aBorder);
		case IANE_GB_F64: return morphology_rank<double>(*aSrc, *aDst, aRadius, aMask, aDilate, aBorder);
		default: return IANE_GB_UNSUPPORTED;
		}
	} catch (const std::exception&) {
		return IANE_GB_INVALID_ARGUMENT;
	}
}

int ref_convolve(const iane_gb_view* aSrc, const iane_gb_view* aKernel, const iane_gb_view* aDst,
	int aBorder, int aThreads)
{
	if (!aSrc || !aKernel || !aDst || aSrc->rank != aKernel->rank || aSrc->rank != aDst->rank ||
	    (aBorder != IANE_GB_BORDER_ZERO && aBorder != IANE_GB_BORDER_CLAMP)) {
		return IANE_GB_INVALID_ARGUMENT;
	}
	try {
		return dispatch(*aSrc, *aKernel, *aDst, aBorder, aThreads);
	} catch (const std::exception&) {
		return IANE_GB_INVALID_ARGUMENT;
	}
}

int ref_rl(const float* aObserved, int aRank, const int32_t* aExtent, const float* aPsf,
	const int32_t* aPsfExtent, int aIterations, float aEpsilon, int aInit, float* aEstimate, int aThreads)
{
	try {
		switch (aRank) {
		case 1: return rl_typed<1>(aObserved, aExtent, aPsf, aPsfExtent, aIterations, aEpsilon, aInit, aEstimate, aThreads);
		case 2: return rl_typed<2>(aObserved, aExtent, aPsf, aPsfExtent, aIterations, aEpsilon, aInit, aEstimate, aThreads);
		case 3: return rl_typed<3>(aObserved, aExtent, aPsf, aPsfExtent, aIterations, aEpsilon, aInit, aEstimate, aThreads);
		default: return IANE_GB_UNSUPPORTED;
		}
	} catch (const std::exception&) {
		return IANE_GB_INVALID_ARGUMENT;
	}
}

} // extern "C"
