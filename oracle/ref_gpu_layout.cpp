/*
 * Byte layout of the functor argument of the reference kernel in ref_gpu.cu -- TEST
 * INFRASTRUCTURE ONLY. Built and run where the reference's headers are (oracle/build.py); it
 * constructs the functor with a distinct marker in every field, finds each marker in the
 * object's bytes and prints the offsets as JSON, so that a host without those headers can fill
 * in device pointers, extents and strides. Exits 1 unless every marker occurs exactly once.
 */
#include "ref_gpu_types.hpp"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>

namespace {

template<class T>
int find_once(const unsigned char* bytes, size_t size, T marker)
{
	int found = -1;
	for (size_t o = 0; o + sizeof(T) <= size; ++o) {
		if (std::memcmp(bytes + o, &marker, sizeof(T)) == 0) {
			if (found >= 0) return -2;
			found = static_cast<int>(o);
		}
	}
	return found;
}

ref_gpu::Fn make(iane::border_mode border)
{
	using ext = ref_gpu::Dst::extents_t;
	ref_gpu::Dst dst(reinterpret_cast<float*>(0x1a1a1a1a1a1a1a10ull), ext{0x11000001, 0x11000002, 0x11000003},
		ext{0x12000001, 0x12000002, 0x12000003});
	ref_gpu::Src src(reinterpret_cast<const float*>(0x2b2b2b2b2b2b2b20ull), ext{0x21000001, 0x21000002, 0x21000003},
		ext{0x22000001, 0x22000002, 0x22000003});
	ref_gpu::Ker ker(reinterpret_cast<const float*>(0x3c3c3c3c3c3c3c30ull), ext{0x31000001, 0x31000002, 0x31000003},
		ext{0x32000001, 0x32000002, 0x32000003});
	return ref_gpu::Fn{dst, ref_gpu::Transform{src, ref_gpu::Filter{ker, ext{0x41000001, 0x41000002, 0x41000003}},
		border}};
}

}  // namespace

int main()
{
	// objects built in zeroed storage, so padding bytes compare equal
	alignas(ref_gpu::Fn) unsigned char ba[sizeof(ref_gpu::Fn)] = {};
	alignas(ref_gpu::Fn) unsigned char bb[sizeof(ref_gpu::Fn)] = {};
	new (ba) ref_gpu::Fn(make(iane::border_mode::clamp));
	new (bb) ref_gpu::Fn(make(iane::border_mode::zero));
	int border = -1, diffs = 0;
	for (size_t o = 0; o < sizeof ba; ++o) {
		if (ba[o] != bb[o]) {
			border = static_cast<int>(o);
			++diffs;
		}
	}
	struct { const char* name; int offset; } fields[] = {
		{"dst_ptr", find_once<uint64_t>(ba, sizeof ba, 0x1a1a1a1a1a1a1a10ull)},
		{"dst_size", find_once<int32_t>(ba, sizeof ba, 0x11000001)},
		{"dst_strides", find_once<int32_t>(ba, sizeof ba, 0x12000001)},
		{"src_ptr", find_once<uint64_t>(ba, sizeof ba, 0x2b2b2b2b2b2b2b20ull)},
		{"src_size", find_once<int32_t>(ba, sizeof ba, 0x21000001)},
		{"src_strides", find_once<int32_t>(ba, sizeof ba, 0x22000001)},
		{"ker_ptr", find_once<uint64_t>(ba, sizeof ba, 0x3c3c3c3c3c3c3c30ull)},
		{"ker_size", find_once<int32_t>(ba, sizeof ba, 0x31000001)},
		{"ker_strides", find_once<int32_t>(ba, sizeof ba, 0x32000001)},
		{"filter_size", find_once<int32_t>(ba, sizeof ba, 0x41000001)},
	};
	if (diffs != 1) {
		std::fprintf(stderr, "border differs in %d bytes\n", diffs);
		return 1;
	}
	std::printf("{\"size\": %zu, \"align\": %zu, \"extents_bytes\": %zu, \"border\": %d, \"border_zero\": %d",
		sizeof(ref_gpu::Fn), alignof(ref_gpu::Fn), sizeof(ref_gpu::Dst::extents_t), border, static_cast<int>(bb[border]));
	for (const auto& f : fields) {
		if (f.offset < 0) {
			std::fprintf(stderr, "marker of %s found %s\n", f.name, f.offset == -1 ? "nowhere" : "twice");
			return 1;
		}
		std::printf(", \"%s\": %d", f.name, f.offset);
	}
	std::printf("}\n");
	return 0;
}
