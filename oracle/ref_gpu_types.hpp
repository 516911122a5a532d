/*
 * Types of the reference's CUDA convolution of f32 3-D memory views -- TEST INFRASTRUCTURE ONLY.
 *
 * iane::convolve on CUDA views (include/iane/algorithms/convolution.hpp:97-117) hands
 * transform_locator (include/iane/algorithms/transform.hpp:94-102) a convolution_filter; that
 * reaches for_each_position, which wraps it in a pixel_visitor and launches visit_positions
 * (include/iane/algorithms/for_each.hpp:19-29, 143-160). These aliases name exactly that
 * functor for f32 source, kernel and destination views of rank 3. Compiled only against the
 * reference's own headers (oracle/build.py); nothing here restates them.
 */
#pragma once

#include <iane/algorithms/convolution.hpp>
#include <iane/view/const_device_image_view.hpp>
#include <iane/view/device_image_view.hpp>

namespace ref_gpu {

using Src = iane::const_device_image_view<float, 3>;
using Ker = iane::const_device_image_view<float, 3>;
using Dst = iane::device_image_view<float, 3>;
using Filter = iane::detail::convolution_filter<Ker, float>;
using Transform = iane::detail::locator_transform<Src, Filter>;
using Fn = iane::detail::pixel_visitor<Dst, Transform>;

}  // namespace ref_gpu
