// Drop-in GB300 dispatch for IANE's flat morphology.
//
// Include after (or instead of) <iane/algorithms/morphology/morphology.hpp> and link
// libiane_gb300.so. Existing calls
//
//     iane::erode(src, dst, iane::box_footprint(radius), {.border = iane::border_mode::zero}, iane::cuda_policy{s});
//     iane::dilate(src, dst, iane::make_flat_footprint(radius, predicate));
//
// on CUDA memory views of u8, i8, u16, i16, i32, u32, f32 or f64 (rank 1-3) resolve to the
// overloads below: they carry the reference's constraints
// (include/iane/algorithms/morphology/morphology.hpp:172-206) plus native_view on both views,
// so they win overload resolution as the more constrained candidates. A box footprint is
// passed as the whole box; any other predicate is evaluated on the host over the box and
// uploaded as a byte mask (stream-ordered, freed after the launch). Results are bit-identical
// to the reference's, NaN and signed zeros included.
//
// iane::gb::opening / iane::gb::closing are the prepared compound algorithms
// (morphology.hpp:216-232) for execution_context::prepare / run, with the GB300 kernels.
#pragma once

#include <iane/algorithms/morphology/morphology.hpp>
#include <iane/gb/convolution.hpp>

#include <cstdint>
#include <memory>
#include <type_traits>
#include <vector>

namespace iane::gb::detail {

template<int tDim, class TCoord>
void radius_array(const TCoord& aRadius, std::int32_t (&aOut)[3])
{
	for (int i = 0; i < 3; ++i) aOut[i] = 0;
	for (int i = 0; i < tDim; ++i) {
		aOut[i] = static_cast<std::int32_t>(math::detail::axis(aRadius, i));
		if (aOut[i] < 0) {
			throw std::invalid_argument("Morphology requires a nonnegative radius with representable width");
		}
	}
}

struct device_buffer_deleter {
	void operator()(std::uint8_t* aPtr) const noexcept { cudaFree(aPtr); }
};
using device_mask = std::unique_ptr<std::uint8_t, device_buffer_deleter>;

/// The footprint as a byte mask over its box in raster order; empty for a box footprint.
template<int tDim, class TCoord, class TPredicate>
std::vector<std::uint8_t> footprint_bytes(const flat_footprint<TCoord, TPredicate>& aFootprint)
{
	if constexpr (std::is_same_v<TPredicate, iane::detail::include_offset>) {
		return {};
	} else {
		std::int32_t r[3];
		radius_array<tDim>(aFootprint.radius, r);
		const long long w0 = 2LL * r[0] + 1, w1 = 2LL * r[1] + 1, w2 = 2LL * r[2] + 1;
		std::vector<std::uint8_t> mask(static_cast<std::size_t>(w0 * w1 * w2));
		std::size_t q = 0;
		for (long long p2 = 0; p2 < w2; ++p2) {
			for (long long p1 = 0; p1 < w1; ++p1) {
				for (long long p0 = 0; p0 < w0; ++p0, ++q) {
					TCoord offset{};
					const long long pos[3] = {p0, p1, p2};
					for (int i = 0; i < tDim; ++i) {
						math::detail::axis(offset, i) = static_cast<int>(pos[i] - r[i]);
					}
					mask[q] = aFootprint.contains(static_cast<const TCoord&>(offset)) ? 1 : 0;
				}
			}
		}
		return mask;
	}
}

/// The footprint's mask in device memory owned by the caller (null for a box footprint).
template<int tDim, class TCoord, class TPredicate>
device_mask footprint_mask(const flat_footprint<TCoord, TPredicate>& aFootprint)
{
	const auto bytes = footprint_bytes<tDim>(aFootprint);
	if (bytes.empty()) {
		return device_mask(nullptr);
	}
	std::uint8_t* device = nullptr;
	iane::detail::check_cuda(cudaMalloc(reinterpret_cast<void**>(&device), bytes.size()), "GB300 morphology: mask");
	device_mask owned(device);
	iane::detail::check_cuda(cudaMemcpy(device, bytes.data(), bytes.size(), cudaMemcpyHostToDevice),
		"GB300 morphology: mask upload");
	return owned;
}

template<class TSrc, class TDst, class TCoord, class TPredicate>
execution morphology_call(TSrc aSource, TDst aDestination, const flat_footprint<TCoord, TPredicate>& aFootprint,
	morphology_options aOptions, cudaStream_t aStream, int aOp)
{
	std::int32_t r[3];
	radius_array<TSrc::dimension>(aFootprint.radius, r);
	const auto bytes = footprint_bytes<TSrc::dimension>(aFootprint);
	std::uint8_t* mask = nullptr;
	if (!bytes.empty()) {
		// stream-ordered: the upload copies the pageable host mask before it returns, and the
		// buffer is freed after the launch that reads it
		iane::detail::check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&mask), bytes.size(), aStream),
			"GB300 morphology: mask");
		iane::detail::check_cuda(cudaMemcpyAsync(mask, bytes.data(), bytes.size(), cudaMemcpyHostToDevice, aStream),
			"GB300 morphology: mask upload");
	}
	const auto src = to_view(aSource);
	const auto dst = to_view(aDestination);
	const int status = iane_gb_morphology(&src, &dst, r, mask, aOp, border_code(aOptions.border), aStream);
	if (mask) {
		cudaFreeAsync(mask, aStream);
	}
	check(status);
	return {{aStream}};
}

} // namespace iane::gb::detail

namespace iane {

/// GB300 erosion for CUDA memory views; the reference's contract (morphology.hpp:172-190).
template<class TSrc, class TDst, class TCoord, class TPredicate>
requires (detail::morphology_views<TSrc, TDst, TCoord, TPredicate> && gb::detail::native_view<TSrc> &&
	gb::detail::native_view<TDst>)
gb::execution erode(TSrc aSource, TDst aDestination, flat_footprint<TCoord, TPredicate> aFootprint,
	morphology_options aOptions = {}, view_policy<TDst> aPolicy = {})
{
	return gb::detail::morphology_call(aSource, aDestination, aFootprint, aOptions, aPolicy.stream, IANE_GB_ERODE);
}

/// GB300 dilation for CUDA memory views; the reference's contract (morphology.hpp:192-206).
template<class TSrc, class TDst, class TCoord, class TPredicate>
requires (detail::morphology_views<TSrc, TDst, TCoord, TPredicate> && gb::detail::native_view<TSrc> &&
	gb::detail::native_view<TDst>)
gb::execution dilate(TSrc aSource, TDst aDestination, flat_footprint<TCoord, TPredicate> aFootprint,
	morphology_options aOptions = {}, view_policy<TDst> aPolicy = {})
{
	return gb::detail::morphology_call(aSource, aDestination, aFootprint, aOptions, aPolicy.stream, IANE_GB_DILATE);
}

} // namespace iane

namespace iane::gb {

/// Prepared opening / closing: the mask and radius, the prepared shape and element type.
template<int tDim>
class compound_morphology_state {
public:
	compound_morphology_state(detail::device_mask aMask, const std::int32_t (&aRadius)[3], const std::int32_t (&aExtent)[3],
		int aDtype, int aOp, int aBorder)
		: mMask(std::move(aMask)), mDtype(aDtype), mOp(aOp), mBorder(aBorder)
	{
		for (int i = 0; i < 3; ++i) {
			mRadius[i] = aRadius[i];
			mExtent[i] = aExtent[i];
		}
	}

	std::size_t scratch_bytes() const { return iane_gb_morphology_scratch_bytes(mDtype, tDim, mExtent); }

	template<class TSrc, class TDst>
	requires (detail::native_view<TSrc> && detail::native_view<TDst> && TSrc::dimension == tDim)
	execution run(TSrc aSource, TDst aDestination, iane::detail::scratch_space<cuda_policy>& aScratch,
		cuda_policy aPolicy)
	{
		const auto src = detail::to_view(aSource);
		const auto dst = detail::to_view(aDestination);
		for (int i = 0; i < tDim; ++i) {
			if (src.extent[i] != mExtent[i] || dst.extent[i] != mExtent[i]) {
				throw std::invalid_argument("Morphology views must match the prepared shape");
			}
		}
		const auto bytes = scratch_bytes();
		void* scratch = aScratch.bytes(bytes, 256);
		detail::check(iane_gb_morphology_compound(&src, &dst, mRadius, mMask.get(), mOp, mBorder, scratch, bytes,
			aPolicy.stream));
		return {{aPolicy.stream}};
	}

private:
	detail::device_mask mMask;
	std::int32_t mRadius[3];
	std::int32_t mExtent[3];
	int mDtype;
	int mOp;
	int mBorder;
};

/// The prepared compound algorithm: iane::opening / iane::closing on the GB300 kernels.
template<class TCoord, class TPredicate>
struct compound_morphology {
	flat_footprint<TCoord, TPredicate> footprint;
	morphology_options options;
	int op;

	template<class TSrc, class TDst>
	requires (detail::native_view<TSrc> && detail::native_view<TDst> &&
		iane::detail::morphology_views<TSrc, TDst, TCoord, TPredicate>)
	compound_morphology_state<TSrc::dimension> prepare(TSrc aSource, TDst aDestination, cuda_policy) const
	{
		std::int32_t r[3], extent[3] = {1, 1, 1};
		detail::radius_array<TSrc::dimension>(footprint.radius, r);
		const auto size = aSource.dimensions();
		const auto out = aDestination.dimensions();
		for (int i = 0; i < TSrc::dimension; ++i) {
			extent[i] = math::detail::axis(size, i);
			if (math::detail::axis(out, i) != extent[i]) {
				throw std::invalid_argument("Source and destination require matching nonnegative dimensions");
			}
		}
		return compound_morphology_state<TSrc::dimension>(detail::footprint_mask<TSrc::dimension>(footprint), r, extent,
			detail::to_view(aSource).dtype, op, detail::border_code(options.border));
	}
};

/// Prepared flat opening (erosion, then dilation) on the GB300 kernels.
template<class TCoord, class TPredicate>
compound_morphology<TCoord, TPredicate> opening(flat_footprint<TCoord, TPredicate> aFootprint,
	morphology_options aOptions = {})
{
	return {aFootprint, aOptions, IANE_GB_OPENING};
}

/// Prepared flat closing (dilation, then erosion) on the GB300 kernels.
template<class TCoord, class TPredicate>
compound_morphology<TCoord, TPredicate> closing(flat_footprint<TCoord, TPredicate> aFootprint,
	morphology_options aOptions = {})
{
	return {aFootprint, aOptions, IANE_GB_CLOSING};
}

} // namespace iane::gb
