/*
 * The reference's own CUDA convolution kernel -- TEST INFRASTRUCTURE ONLY (the GPU baseline
 * and a checker). oracle/build.py compiles this file with nvcc against the reference's headers
 * in place into oracle/_ref/ref_conv_f32_3d.cubin. The cubin holds one kernel: the reference's
 * visit_positions (include/iane/algorithms/for_each.hpp:19-29) instantiated with the functor
 * iane::convolve builds for f32 3-D CUDA views (ref_gpu_types.hpp). oracle/ref_gpu.py loads it
 * through the CUDA driver API and launches it the way visit_coordinates does
 * (for_each.hpp:143-160): one thread per output voxel, 256-thread blocks.
 */
#include "ref_gpu_types.hpp"

template __global__ void iane::detail::visit_positions<ref_gpu::Dst, ref_gpu::Fn>(ref_gpu::Fn, std::size_t,
	ref_gpu::Dst::extents_t);
