// Drop-in GB300 dispatch for IANE's convolution and a prepared Richardson-Lucy algorithm.
//
// Include this header after (or instead of) <iane/algorithms/convolution.hpp> and link
// libiane_gb300.so. Existing call sites
//
//     iane::convolve(src, kernel, dst, {.border = iane::border_mode::zero}, iane::cuda_policy{stream});
//
// on CUDA memory views (const_device_image_view / device_image_view) of u8, i8, u16, i16,
// i32, u32, f32 or f64 elements (or a packed rgb8 pixel type opted in through
// iane::gb::packed_rgb8), rank 1 to 3, then resolve to the overload below, which carries the
// reference template's constraints (include/iane/algorithms/convolution.hpp:91-96) plus
// native_view on all three views and therefore wins overload resolution as the more
// constrained candidate; texture_image_view sources with memory kernels and destinations
// resolve to the texture overload at the end. Procedural views, other custom element types
// and host views keep resolving to the reference's generic template. The call is asynchronous on
// the policy's stream, returns an execution handle whose wait() synchronises it, and
// reports errors with the reference's exception types: std::invalid_argument for kernel
// extents that are not positive and odd or for mismatched image extents, std::runtime_error
// for CUDA failures (include/iane/execution/context.hpp:36-41).
//
// iane::gb::richardson_lucy plugs the RL loop of examples/rl_deconvolution/main.cu:51-81
// into the prepared-algorithm protocol (include/iane/execution/prepared.hpp:120-146):
//
//     auto exec = iane::make_execution_context(iane::cuda_policy{stream});
//     auto op = exec.prepare(iane::gb::richardson_lucy{psf, 50, 1e-6f}, observed, estimate);
//     exec.run(op, observed, estimate).wait();
#pragma once

#include <iane/algorithms/convolution.hpp>
#include <iane/algorithms/copy.hpp>
#include <iane/execution/context.hpp>
#include <iane/execution/prepared.hpp>
#include <iane/view/make_view.hpp>
#include <iane/view/texture_image_view.hpp>
#include <iane_gb/capi.h>

#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>

namespace iane::gb {

/// Completion handle of a GB300 launch; a cuda_execution for all uses.
struct execution : cuda_execution {};

/// Accumulation for the convolution overload: fast (FP32, or int64 for integer pairs) or
/// exact (FP64 in the reference's tap order, bit-identical to the reference).
enum class accumulation { fast, exact };

/// Accumulation used by iane::convolve on native views in the calling thread.
inline accumulation& thread_accumulation()
{
	thread_local accumulation mode = accumulation::fast;
	return mode;
}

/// Method for float convolution in fast accumulation: direct (tiled FP32), fft (cuFFT in
/// FP64 over the border-padded source) or automatic (whichever a cost model predicts faster:
/// the spectral path pays off for kernels of many thousands of taps).
enum class method { direct, fft, automatic };

/// Method used by iane::convolve on native views in the calling thread.
inline method& thread_method()
{
	thread_local method m = method::direct;
	return m;
}

namespace detail {

template<class T> inline constexpr int dtype_code = 0;
template<> inline constexpr int dtype_code<std::uint8_t> = IANE_GB_U8;
template<> inline constexpr int dtype_code<std::uint16_t> = IANE_GB_U16;
template<> inline constexpr int dtype_code<std::int16_t> = IANE_GB_I16;
template<> inline constexpr int dtype_code<std::int32_t> = IANE_GB_I32;
template<> inline constexpr int dtype_code<float> = IANE_GB_F32;
template<> inline constexpr int dtype_code<double> = IANE_GB_F64;
template<> inline constexpr int dtype_code<std::int8_t> = IANE_GB_I8;
template<> inline constexpr int dtype_code<std::uint32_t> = IANE_GB_U32;

} // namespace detail

/// Opt-in for a user's packed byte (r, g, b) pixel type: specialise to std::true_type for a
/// 3-byte type whose product with a float tap is a per-channel double sum converted back with
/// the byte rule, like the pixel of the reference's convolution example
/// (examples/convolution/main.cu:20-56). Views of it then take the GB300 rgb8 path.
template<class T>
struct packed_rgb8 : std::false_type {};

namespace detail {

template<class T>
constexpr int element_code()
{
	if constexpr (packed_rgb8<T>::value) {
		static_assert(sizeof(T) == 3, "a packed rgb8 pixel is 3 bytes");
		return IANE_GB_RGB8;
	} else {
		return dtype_code<T>;
	}
}

/// A CUDA memory view whose element type and rank the GB300 kernels take.
template<class TView>
concept native_view = concepts::DeviceView<TView> && concepts::MemoryView<TView> &&
	(TView::dimension >= 1) && (TView::dimension <= IANE_GB_MAX_RANK) &&
	(element_code<std::remove_cv_t<typename TView::value_type>>() != 0);

template<class TView>
iane_gb_view to_view(const TView& aView)
{
	iane_gb_view v{};
	v.ptr = const_cast<void*>(static_cast<const void*>(aView.pointer()));
	v.dtype = element_code<std::remove_cv_t<typename TView::value_type>>();
	v.rank = TView::dimension;
	const auto size = aView.dimensions();
	const auto strides = aView.strides();
	for (int i = 0; i < TView::dimension; ++i) {
		v.extent[i] = math::detail::axis(size, i);
		v.stride[i] = math::detail::axis(strides, i);
	}
	return v;
}

inline std::string last_error()
{
	char buffer[512];
	iane_gb_last_error(buffer, sizeof buffer);
	return buffer;
}

/// Map a C-ABI status to the exception the reference throws in the same situation.
inline void check(int aStatus)
{
	switch (aStatus) {
	case IANE_GB_OK: return;
	case IANE_GB_INVALID_ARGUMENT: throw std::invalid_argument(last_error());
	case IANE_GB_LENGTH_ERROR: throw std::length_error(last_error());
	case IANE_GB_OUT_OF_MEMORY: throw std::bad_alloc();
	default: throw std::runtime_error(last_error());
	}
}

inline int border_code(border_mode aBorder)
{
	return aBorder == border_mode::zero ? IANE_GB_BORDER_ZERO : IANE_GB_BORDER_CLAMP;
}

} // namespace detail

/// Start value of a Richardson-Lucy run.
enum class rl_start {
	observed = IANE_GB_RL_INIT_OBSERVED, ///< max(observed, eps), as examples/rl_deconvolution
	mean = IANE_GB_RL_INIT_MEAN,         ///< flat start at max(mean(observed), eps)
	given = IANE_GB_RL_INIT_GIVEN        ///< the estimate view's current contents
};

/// Prepared state: owns the plan (PSF copies, adjoint, edge-sensitivity table).
class richardson_lucy_state {
public:
	richardson_lucy_state(iane_gb_rl_plan* aPlan, int aIterations, float aEpsilon, rl_start aStart)
		: mPlan(aPlan), mIterations(aIterations), mEpsilon(aEpsilon), mStart(aStart) {}

	std::size_t scratch_bytes() const { return iane_gb_rl_scratch_bytes(mPlan.get()); }

	template<class TSrc, class TDst>
	requires (detail::native_view<TSrc> && detail::native_view<TDst> && concepts::MatchingViewRank<TSrc, TDst>)
	execution run(TSrc aSource, TDst aDestination, iane::detail::scratch_space<cuda_policy>& aScratch,
		cuda_policy aPolicy)
	{
		const auto bytes = scratch_bytes();
		void* scratch = aScratch.bytes(bytes, alignof(std::max_align_t));
		const auto src = detail::to_view(aSource);
		const auto dst = detail::to_view(aDestination);
		detail::check(iane_gb_rl_run(mPlan.get(), &src, &dst, mIterations, mEpsilon, static_cast<int>(mStart),
			scratch, bytes, nullptr, aPolicy.stream));
		return {{aPolicy.stream}};
	}

private:
	struct plan_deleter {
		void operator()(iane_gb_rl_plan* aPlan) const noexcept { iane_gb_rl_destroy(aPlan); }
	};
	std::unique_ptr<iane_gb_rl_plan, plan_deleter> mPlan;
	int mIterations;
	float mEpsilon;
	rl_start mStart;
};

/**
 * @brief Richardson-Lucy deconvolution as a prepared algorithm for CUDA contexts.
 * @tparam TPsf An f32 CUDA memory view of odd extents with the image rank; normalise it to
 * sum 1 beforehand, as examples/common/deconvolution.hpp:10-30 does.
 *
 * Each iteration is two fused passes: convolve(estimate, psf) with the guarded ratio
 * observed / max(pred, eps) in its epilogue, then convolve(ratio, adjoint) with the edge
 * correction and the multiplicative update in its epilogue (zero border throughout).
 */
template<class TPsf>
requires detail::native_view<TPsf>
struct richardson_lucy {
	TPsf psf;
	int iterations = 20;
	float epsilon = 1e-6f;
	rl_start start = rl_start::observed;

	template<class TSrc, class TDst>
	requires (detail::native_view<TSrc> && detail::native_view<TDst> && concepts::MatchingViewRank<TSrc, TDst>)
	richardson_lucy_state prepare(TSrc aSource, TDst aDestination, cuda_policy aPolicy) const
	{
		const auto psf_view = detail::to_view(psf);
		const auto size = aSource.dimensions();
		const auto out = aDestination.dimensions();
		std::int32_t extent[3] = {1, 1, 1};
		for (int i = 0; i < TSrc::dimension; ++i) {
			extent[i] = math::detail::axis(size, i);
			if (math::detail::axis(out, i) != extent[i]) {
				throw std::invalid_argument("Source and destination require matching nonnegative dimensions");
			}
		}
		if (iterations < 0 || !(epsilon > 0.0f)) {
			throw std::invalid_argument("Iterations and finite epsilon must be positive");
		}
		iane_gb_rl_plan* plan = nullptr;
		detail::check(iane_gb_rl_prepare(&psf_view, TSrc::dimension, extent, aPolicy.stream, &plan));
		return richardson_lucy_state(plan, iterations, epsilon, start);
	}
};

template<class TPsf>
richardson_lucy(TPsf, int, float) -> richardson_lucy<TPsf>;
template<class TPsf>
richardson_lucy(TPsf, int, float, rl_start) -> richardson_lucy<TPsf>;

} // namespace iane::gb

namespace iane {

/**
 * @brief GB300 convolution for CUDA memory views (see the file comment).
 *
 * Same contract as the reference's iane::convolve. Accumulation follows
 * iane::gb::thread_accumulation(): FP32 by default, FP64 in the reference's order when set
 * to accumulation::exact. In fast accumulation, iane::gb::thread_method() selects the
 * direct or the spectral (FFT) method for float views.
 */
template<class TSrc, class TKernel, class TDst>
requires (concepts::TransformViews<TSrc, TDst> &&
	concepts::ReadableView<TKernel> &&
	concepts::MatchingViewRank<TKernel, TSrc> &&
	concepts::SameViewBackend<TKernel, TSrc> &&
	concepts::ConvolutionElements<typename TSrc::value_type, typename TKernel::value_type,
		typename TDst::value_type> &&
	gb::detail::native_view<TSrc> && gb::detail::native_view<TKernel> && gb::detail::native_view<TDst>)
gb::execution convolve(TSrc aSource, TKernel aKernel, TDst aDestination,
	convolution_options aOptions = {}, view_policy<TDst> aPolicy = {})
{
	const auto src = gb::detail::to_view(aSource);
	const auto kernel = gb::detail::to_view(aKernel);
	const auto dst = gb::detail::to_view(aDestination);
	unsigned flags = gb::thread_accumulation() == gb::accumulation::exact ? IANE_GB_ACC_EXACT : IANE_GB_ACC_FAST;
	if (flags == IANE_GB_ACC_FAST && gb::thread_method() != gb::method::direct) {
		flags |= gb::thread_method() == gb::method::fft ? IANE_GB_CONV_FFT : IANE_GB_CONV_AUTO;
	}
	gb::detail::check(iane_gb_convolve(&src, &kernel, &dst, gb::detail::border_code(aOptions.border), flags,
		aPolicy.stream));
	return {{aPolicy.stream}};
}

#if defined(__CUDACC__)
/**
 * @brief GB300 convolution with a texture source (texture_image_view, rank 1-3, of a scalar
 * texel type), a CUDA memory kernel and destination.
 *
 * The view keeps its texture object private, so the texels are first gathered into a
 * stream-ordered linear buffer by the reference's own copy (texture_image_view::operator[],
 * include/iane/view/texture_image_view.hpp:45-53) and the buffer is convolved by the GB300
 * kernels; the buffer is freed in stream order. Callers that hold the texture object use
 * iane_gb_convolve_texture, which reads the texels directly.
 */
template<class TElement, int tDim, class TKernel, class TDst>
requires (gb::detail::native_view<TKernel> && gb::detail::native_view<TDst> &&
	TKernel::dimension == tDim && TDst::dimension == tDim &&
	(gb::detail::dtype_code<TElement> != 0) &&
	concepts::ConvolutionElements<TElement, typename TKernel::value_type, typename TDst::value_type>)
gb::execution convolve(texture_image_view<TElement, tDim> aSource, TKernel aKernel, TDst aDestination,
	convolution_options aOptions = {}, view_policy<TDst> aPolicy = {})
{
	const auto size = aSource.dimensions();
	const auto count = math::detail::element_count<tDim>(size);
	if (count == 0) {
		return convolve(device::make_const_view<TElement, tDim>(nullptr, size), aKernel, aDestination, aOptions,
			aPolicy);
	}
	TElement* linear = nullptr;
	detail::check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&linear), count * sizeof(TElement), aPolicy.stream),
		"GB300 texture convolution: gather buffer");
	struct release {
		TElement* ptr;
		cudaStream_t stream;
		~release() { cudaFreeAsync(ptr, stream); }
	} guard{linear, aPolicy.stream};
	copy(aSource, device::make_view<TElement, tDim>(linear, size), cuda_policy{.stream = aPolicy.stream});
	return convolve(device::make_const_view<TElement, tDim>(linear, size), aKernel, aDestination, aOptions, aPolicy);
}
#endif

} // namespace iane
