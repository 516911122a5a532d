// Compile-and-run check of the C++ drop-in (include/iane/gb/convolution.hpp) against the
// reference's own headers: overload selection, exception mapping, and -- where a GPU is
// present -- a convolution and a prepared Richardson-Lucy run through iane's own API.
#include <iane/algorithms/convolution.hpp>
#include <iane/algorithms/copy.hpp>
#include <iane/image/image.hpp>
#include <iane/resource/cuda/resource_cuda.hpp>
#include <iane/resource/host/resource_host.hpp>
#include <iane/gb/convolution.hpp>
#include <iane/gb/morphology.hpp>

#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <type_traits>
#include <utility>

// A packed byte pixel with per-channel double sums (the element of the reference's
// convolution example), opted in to the GB300 rgb8 path.
struct pixel3 {
	std::uint8_t r, g, b;
};
struct pixel3_sum {
	double r, g, b;
	IANE_DECL_HYBRID pixel3_sum operator+(pixel3_sum o) const { return {r + o.r, g + o.g, b + o.b}; }
	IANE_DECL_HYBRID static std::uint8_t byte(double v)
	{
		if (!(v > 0.0)) return 0;
		if (v >= 255.0) return 255;
		const auto w = static_cast<unsigned int>(v);
		return static_cast<std::uint8_t>(w + (v - w >= 0.5));
	}
	IANE_DECL_HYBRID explicit operator pixel3() const { return {byte(r), byte(g), byte(b)}; }
};
IANE_DECL_HYBRID inline pixel3_sum operator*(pixel3 p, float k)
{
	const double d = k;
	return {p.r * d, p.g * d, p.b * d};
}
template<>
struct iane::gb::packed_rgb8<pixel3> : std::true_type {};

namespace {

using dev_src = iane::const_device_image_view<float, 3>;
using dev_dst = iane::device_image_view<float, 3>;
using dev_src8 = iane::const_device_image_view<std::uint8_t, 2>;
using dev_dst8 = iane::device_image_view<std::uint8_t, 2>;
using dev_k2 = iane::const_device_image_view<float, 2>;
using host_src = iane::const_host_image_view<float, 2>;
using host_dst = iane::host_image_view<float, 2>;

// CUDA memory views of supported types resolve to the GB300 overload ...
static_assert(std::is_same_v<decltype(iane::convolve(std::declval<dev_src>(), std::declval<dev_src>(),
	std::declval<dev_dst>())), iane::gb::execution>);
static_assert(std::is_same_v<decltype(iane::convolve(std::declval<dev_src8>(), std::declval<dev_k2>(),
	std::declval<dev_dst8>(), iane::convolution_options{}, iane::cuda_policy{})), iane::gb::execution>);
// ... so do opted-in rgb8 pixels, and texture sources with memory kernels and destinations ...
static_assert(std::is_same_v<decltype(iane::convolve(std::declval<iane::const_device_image_view<pixel3, 2>>(),
	std::declval<dev_k2>(), std::declval<iane::device_image_view<pixel3, 2>>())), iane::gb::execution>);
static_assert(std::is_same_v<decltype(iane::convolve(std::declval<iane::texture_image_view<std::uint8_t, 2>>(),
	std::declval<dev_k2>(), std::declval<dev_dst8>())), iane::gb::execution>);
// ... and erosion / dilation of CUDA memory views, box or predicate footprints ...
struct cross_predicate {
	IANE_DECL_HYBRID bool operator()(const iane::math::vec2i& o) const { return o[0] == 0 || o[1] == 0; }
};
static_assert(std::is_same_v<decltype(iane::erode(std::declval<dev_src8>(), std::declval<dev_dst8>(),
	iane::box_footprint(iane::math::vec2i{1, 2}))), iane::gb::execution>);
static_assert(std::is_same_v<decltype(iane::dilate(std::declval<dev_src8>(), std::declval<dev_dst8>(),
	iane::make_flat_footprint(iane::math::vec2i{1, 1}, cross_predicate{}))), iane::gb::execution>);
// ... host views keep the reference's template.
static_assert(!std::is_same_v<decltype(iane::convolve(std::declval<host_src>(), std::declval<host_src>(),
	std::declval<host_dst>())), iane::gb::execution>);

int failures = 0;

template<class F>
void expect_invalid_argument(const char* what, F&& f)
{
	try {
		f();
		std::printf("FAIL %s: no exception\n", what);
		++failures;
	} catch (const std::invalid_argument&) {
		std::printf("ok   %s\n", what);
	} catch (const std::exception& e) {
		std::printf("FAIL %s: wrong exception %s\n", what, e.what());
		++failures;
	}
}

} // namespace

int main()
{
	// Argument errors are detected before any CUDA call, so they need no device.
	float storage[64] = {};
	using v3 = iane::math::vec3i;
	const dev_src src(storage, v3{4, 4, 4}, v3{4, 16, 64});
	const dev_dst dst(storage, v3{4, 4, 4}, v3{4, 16, 64});
	const dev_src even(storage, v3{2, 3, 3}, v3{4, 8, 24});
	const dev_dst smaller(storage, v3{4, 4, 3}, v3{4, 16, 64});
	expect_invalid_argument("even kernel extent", [&] { iane::convolve(src, even, dst); });
	expect_invalid_argument("mismatched extents", [&] { iane::convolve(src, src, smaller); });

	int devices = 0;
	if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) {
		std::printf("no CUDA device: GPU part skipped\n");
		return failures == 0 ? 0 : 1;
	}
	// GPU part: 3-D convolution against the reference's CPU convolution, then prepared RL.
	iane::host_image<float, 3> h_src(20, 18, 9), h_ref(20, 18, 9), h_out(20, 18, 9);
	iane::host_image<float, 3> h_k(5, 3, 3);
	for (int i = 0; i < 20 * 18 * 9; ++i) h_src.pointer()[i] = static_cast<float>((i * 37) % 101) / 7.0f;
	for (int i = 0; i < 45; ++i) h_k.pointer()[i] = static_cast<float>(i % 7 + 1) / 100.0f;
	iane::convolve(h_src.const_view(), h_k.const_view(), h_ref.view(), {iane::border_mode::zero});
	iane::device_image<float, 3> d_src(20, 18, 9), d_out(20, 18, 9), d_k(5, 3, 3);
	iane::copy(h_src.const_view(), d_src.view()).wait();
	iane::copy(h_k.const_view(), d_k.view()).wait();
	iane::gb::thread_accumulation() = iane::gb::accumulation::exact;
	iane::convolve(d_src.const_view(), d_k.const_view(), d_out.view(), {iane::border_mode::zero}).wait();
	iane::copy(d_out.const_view(), h_out.view()).wait();
	for (int i = 0; i < 20 * 18 * 9; ++i) {
		if (h_out.pointer()[i] != h_ref.pointer()[i]) {
			std::printf("FAIL exact convolution differs at %d\n", i);
			return 1;
		}
	}
	std::printf("ok   exact convolution matches the reference\n");
	iane::gb::thread_accumulation() = iane::gb::accumulation::fast;
	iane::gb::thread_method() = iane::gb::method::fft;
	iane::convolve(d_src.const_view(), d_k.const_view(), d_out.view(), {iane::border_mode::zero}).wait();
	iane::gb::thread_method() = iane::gb::method::direct;
	iane::copy(d_out.const_view(), h_out.view()).wait();
	for (int i = 0; i < 20 * 18 * 9; ++i) {
		const float want = h_ref.pointer()[i];
		if (std::fabs(h_out.pointer()[i] - want) > 1e-5f * (1.0f + std::fabs(want))) {
			std::printf("FAIL FFT convolution differs at %d\n", i);
			return 1;
		}
	}
	std::printf("ok   FFT convolution matches the reference\n");
	{
		// a texture source: the reference's own texture test shape
		// (test/unit/algorithms/test_convolution_cuda.cu:53-86) against its CPU convolution
		iane::host_image<float, 2> source(iane::math::vec2i{5, 4}), kernel(iane::math::vec2i{3, 3});
		iane::host_image<float, 2> reference(iane::math::vec2i{3, 3}), output(iane::math::vec2i{3, 3});
		for (int i = 0; i < 20; ++i) source.pointer()[i] = static_cast<float>(i - 6);
		for (int i = 0; i < 9; ++i) kernel.pointer()[i] = static_cast<float>(i - 3) / 8.0f;
		iane::texture_image<float> texture(source.dimensions());
		iane::device_image<float, 2> device_kernel(kernel.dimensions()), device_output(iane::math::vec2i{3, 3});
		iane::copy(source.const_view(), texture).wait();
		iane::copy(kernel.const_view(), device_kernel.view()).wait();
		const iane::math::vec2i origin{1, 1}, crop{3, 3};
		iane::convolve(source.const_view().subview(origin, crop), kernel.const_view(), reference.view(),
			{.border = iane::border_mode::clamp});
		iane::convolve(texture.const_view().subview(origin, crop), device_kernel.const_view(), device_output.view(),
			{.border = iane::border_mode::clamp}).wait();
		iane::copy(device_output.const_view(), output.view()).wait();
		for (int i = 0; i < 9; ++i) {
			if (output.pointer()[i] != reference.pointer()[i]) {
				std::printf("FAIL texture convolution differs at %d\n", i);
				return 1;
			}
		}
		std::printf("ok   texture convolution matches the reference\n");
	}
	{
		// erosion with a predicate footprint and a prepared opening against the reference's CPU
		iane::host_image<float, 3> ref_e(20, 18, 9), ref_o(20, 18, 9), mid(20, 18, 9);
		struct odd_sum {
			IANE_DECL_HYBRID bool operator()(const iane::math::vec3i& o) const { return ((o[0] + o[1] + o[2]) & 1) == 0; }
		};
		const auto fp = iane::make_flat_footprint(iane::math::vec3i{1, 2, 1}, odd_sum{});
		iane::erode(h_src.const_view(), ref_e.view(), fp, {.border = iane::border_mode::zero});
		iane::erode(h_src.const_view(), mid.view(), iane::box_footprint(iane::math::vec3i{1, 1, 1}));
		iane::dilate(mid.const_view(), ref_o.view(), iane::box_footprint(iane::math::vec3i{1, 1, 1}));
		iane::erode(d_src.const_view(), d_out.view(), fp, {.border = iane::border_mode::zero}).wait();
		iane::copy(d_out.const_view(), h_out.view()).wait();
		for (int i = 0; i < 20 * 18 * 9; ++i) {
			if (h_out.pointer()[i] != ref_e.pointer()[i]) {
				std::printf("FAIL erosion differs at %d\n", i);
				return 1;
			}
		}
		auto mexec = iane::make_execution_context(iane::cuda_policy{});
		auto plan = mexec.prepare(iane::gb::opening(iane::box_footprint(iane::math::vec3i{1, 1, 1})), d_src.const_view(),
			d_out.view());
		mexec.run(plan, d_src.const_view(), d_out.view()).wait();
		iane::copy(d_out.const_view(), h_out.view()).wait();
		for (int i = 0; i < 20 * 18 * 9; ++i) {
			if (h_out.pointer()[i] != ref_o.pointer()[i]) {
				std::printf("FAIL opening differs at %d\n", i);
				return 1;
			}
		}
		std::printf("ok   morphology matches the reference\n");
	}
	auto exec = iane::make_execution_context(iane::cuda_policy{});
	auto op = exec.prepare(iane::gb::richardson_lucy{d_k.const_view(), 5, 1e-6f, iane::gb::rl_start::mean},
		d_src.const_view(), d_out.view());
	exec.run(op, d_src.const_view(), d_out.view()).wait();
	std::printf("ok   prepared Richardson-Lucy ran\n");
	return failures == 0 ? 0 : 1;
}
