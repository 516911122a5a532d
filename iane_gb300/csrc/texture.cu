// Texture sources for convolution: the reference's texture_image (a CUDA array and its
// point-sampled texture object, include/iane/resource/cuda/texture_image.hpp:20-96), its
// upload (texture_image.hpp:98-140) and convolve over a texture_image_view
// (include/iane/view/texture_image_view.hpp:26-98).
//
// A texture view reads texel origin + p at the texel centre; the border rule is applied to p
// in view coordinates first, as the reference's locator does, so only texels inside the view
// are read and the texture's own addressing mode never matters. Samples feed the same two
// kernels as memory views: the tiled FP32 kernel (fast mode, f32 kernels) and the generic
// kernel (exact mode and integer kernels), through texel fetches instead of loads.
#include "common.cuh"
#include "kernels.h"

#include <map>
#include <mutex>
#include <string>

namespace iane_gb {
namespace {

struct TextureRecord {
	cudaArray_t array;
	int dtype;
	int rank;
	int ext[3];
};

std::mutex& registry_mutex()
{
	static std::mutex m;
	return m;
}

std::map<uint64_t, TextureRecord>& registry()
{
	static std::map<uint64_t, TextureRecord> r;
	return r;
}

bool texel_dtype(int dtype, cudaChannelFormatDesc* desc)
{
	switch (dtype) {
	case IANE_GB_U8: *desc = cudaCreateChannelDesc(8, 0, 0, 0, cudaChannelFormatKindUnsigned); return true;
	case IANE_GB_I8: *desc = cudaCreateChannelDesc(8, 0, 0, 0, cudaChannelFormatKindSigned); return true;
	case IANE_GB_U16: *desc = cudaCreateChannelDesc(16, 0, 0, 0, cudaChannelFormatKindUnsigned); return true;
	case IANE_GB_I16: *desc = cudaCreateChannelDesc(16, 0, 0, 0, cudaChannelFormatKindSigned); return true;
	case IANE_GB_I32: *desc = cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindSigned); return true;
	case IANE_GB_U32: *desc = cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindUnsigned); return true;
	case IANE_GB_F32: *desc = cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindFloat); return true;
	default: return false;
	}
}

// Array extents of a texture object's array (unused axes 1), or false for a texture that is
// not a point-sampled, unnormalised, element-read array texture.
int array_texture_extents(cudaTextureObject_t tex, int ext[3])
{
	cudaResourceDesc res{};
	IANE_GB_CUDA(cudaGetTextureObjectResourceDesc(&res, tex), "convolve texture: resource of the texture");
	if (res.resType != cudaResourceTypeArray) {
		return fail(IANE_GB_UNSUPPORTED, "convolve texture: the texture must read a CUDA array");
	}
	cudaTextureDesc desc{};
	IANE_GB_CUDA(cudaGetTextureObjectTextureDesc(&desc, tex), "convolve texture: sampler of the texture");
	if (desc.filterMode != cudaFilterModePoint || desc.readMode != cudaReadModeElementType || desc.normalizedCoords) {
		return fail(IANE_GB_UNSUPPORTED,
			"convolve texture: the texture must use point sampling, element reads and unnormalised coordinates");
	}
	cudaChannelFormatDesc ch{};
	cudaExtent e{};
	unsigned int flags = 0;
	IANE_GB_CUDA(cudaArrayGetInfo(&ch, &e, &flags, res.res.array.array), "convolve texture: array extents");
	ext[0] = static_cast<int>(e.width);
	ext[1] = e.height ? static_cast<int>(e.height) : 1;
	ext[2] = e.depth ? static_cast<int>(e.depth) : 1;
	return IANE_GB_OK;
}

}  // namespace
}  // namespace iane_gb

using namespace iane_gb;

extern "C" {

int iane_gb_texture_create(int dtype, int rank, const int32_t* extent, uint64_t* texture)
{
	if (!texture || !extent) {
		return fail(IANE_GB_INVALID_ARGUMENT, "texture create: null argument");
	}
	*texture = 0;
	cudaChannelFormatDesc channel{};
	if (!texel_dtype(dtype, &channel)) {
		return fail(IANE_GB_UNSUPPORTED, std::string("texture create: element type ") + dtype_name(dtype) +
			" (textures hold u8, i8, u16, i16, i32, u32 or f32)");
	}
	if (rank < 1 || rank > 3) {
		return fail(IANE_GB_UNSUPPORTED, "texture create: rank must be 1..3");
	}
	int ext[3] = {1, 1, 1};
	long long count = 1;
	for (int i = 0; i < rank; ++i) {
		if (extent[i] < 0) {
			return fail(IANE_GB_INVALID_ARGUMENT, "texture create: negative extent");
		}
		ext[i] = extent[i];
		count *= extent[i];
	}
	if (count == 0) {
		return IANE_GB_OK; // texture_image.hpp:55-57: an empty extent allocates nothing
	}
	cudaArray_t array = nullptr;
	if (rank == 1) {
		IANE_GB_CUDA(cudaMallocArray(&array, &channel, ext[0]), "texture create: array");
	} else if (rank == 2) {
		IANE_GB_CUDA(cudaMallocArray(&array, &channel, ext[0], ext[1]), "texture create: array");
	} else {
		IANE_GB_CUDA(cudaMalloc3DArray(&array, &channel, make_cudaExtent(ext[0], ext[1], ext[2])), "texture create: array");
	}
	cudaResourceDesc resource{};
	resource.resType = cudaResourceTypeArray;
	resource.res.array.array = array;
	cudaTextureDesc sampler{};
	for (int axis = 0; axis < rank; ++axis) {
		sampler.addressMode[axis] = cudaAddressModeClamp;
	}
	sampler.filterMode = cudaFilterModePoint;
	sampler.readMode = cudaReadModeElementType;
	sampler.normalizedCoords = 0;
	cudaTextureObject_t tex = 0;
	const cudaError_t e = cudaCreateTextureObject(&tex, &resource, &sampler, nullptr);
	if (e != cudaSuccess) {
		cudaFreeArray(array);
		return cuda_fail(e, "texture create: texture object");
	}
	{
		const std::lock_guard<std::mutex> lock(registry_mutex());
		registry()[static_cast<uint64_t>(tex)] = TextureRecord{array, dtype, rank, {ext[0], ext[1], ext[2]}};
	}
	*texture = static_cast<uint64_t>(tex);
	return IANE_GB_OK;
}

int iane_gb_texture_upload(uint64_t texture, const iane_gb_view* src, void* stream)
{
	TextureRecord rec{};
	{
		const std::lock_guard<std::mutex> lock(registry_mutex());
		auto it = registry().find(texture);
		if (it == registry().end()) {
			return fail(IANE_GB_INVALID_ARGUMENT, "texture upload: not a texture made by iane_gb_texture_create");
		}
		rec = it->second;
	}
	if (!src || src->rank != rec.rank || src->dtype != rec.dtype) {
		return fail(IANE_GB_INVALID_ARGUMENT, "texture upload: the view needs the texture's rank and element type");
	}
	for (int i = 0; i < rec.rank; ++i) {
		if (src->extent[i] != rec.ext[i]) {
			return fail(IANE_GB_INVALID_ARGUMENT, "CUDA texture upload requires matching dimensions");
		}
	}
	const long long elem = dtype_size(rec.dtype);
	if (src->stride[0] != elem) {
		return fail(IANE_GB_INVALID_ARGUMENT, "CUDA texture upload requires contiguous rows");
	}
	const long long row_bytes = elem * rec.ext[0];
	const long long pitch = rec.rank > 1 && rec.ext[1] > 1 ? src->stride[1] : row_bytes;
	long long slice_rows = rec.ext[1];
	if (rec.rank > 2 && rec.ext[2] > 1) {
		if (pitch <= 0 || src->stride[2] % pitch != 0 || src->stride[2] / pitch < rec.ext[1]) {
			return fail(IANE_GB_INVALID_ARGUMENT, "texture upload: plane stride must be a multiple of the row stride");
		}
		slice_rows = src->stride[2] / pitch;
	}
	if (pitch < row_bytes) {
		return fail(IANE_GB_INVALID_ARGUMENT, "texture upload: rows overlap");
	}
	cudaMemcpy3DParms copy{};
	copy.srcPtr = make_cudaPitchedPtr(const_cast<void*>(static_cast<const void*>(src->ptr)), static_cast<size_t>(pitch),
		static_cast<size_t>(rec.ext[0]), static_cast<size_t>(slice_rows));
	copy.dstArray = rec.array;
	copy.extent = make_cudaExtent(static_cast<size_t>(rec.ext[0]), static_cast<size_t>(rec.ext[1]),
		static_cast<size_t>(rec.ext[2]));
	copy.kind = cudaMemcpyDefault;
	IANE_GB_CUDA(cudaMemcpy3DAsync(&copy, static_cast<cudaStream_t>(stream)), "CUDA texture upload");
	return IANE_GB_OK;
}

int iane_gb_texture_destroy(uint64_t texture)
{
	if (texture == 0) {
		return IANE_GB_OK;
	}
	TextureRecord rec{};
	{
		const std::lock_guard<std::mutex> lock(registry_mutex());
		auto it = registry().find(texture);
		if (it == registry().end()) {
			return fail(IANE_GB_INVALID_ARGUMENT, "texture destroy: not a texture made by iane_gb_texture_create");
		}
		rec = it->second;
		registry().erase(it);
	}
	// texture_image.hpp:33-40: the texture object before its array
	const cudaError_t e1 = cudaDestroyTextureObject(static_cast<cudaTextureObject_t>(texture));
	const cudaError_t e2 = cudaFreeArray(rec.array);
	IANE_GB_CUDA(e1, "texture destroy: texture object");
	IANE_GB_CUDA(e2, "texture destroy: array");
	return IANE_GB_OK;
}

int iane_gb_convolve_texture(const iane_gb_texture_view* src, const iane_gb_view* kernel, const iane_gb_view* dst,
	int border, unsigned flags, void* stream)
{
	if (!src) {
		return fail(IANE_GB_INVALID_ARGUMENT, "convolve texture: null source");
	}
	cudaChannelFormatDesc unused{};
	if (!texel_dtype(src->dtype, &unused)) {
		return fail(IANE_GB_UNSUPPORTED, std::string("convolve texture: element type ") + dtype_name(src->dtype));
	}
	if (src->rank < 1 || src->rank > 3) {
		return fail(IANE_GB_UNSUPPORTED, "convolve texture source: rank must be 1..3");
	}
	DevView s{};
	s.ptr = nullptr;
	s.dtype = src->dtype;
	s.rank = src->rank;
	TexSource t{};
	t.tex = static_cast<cudaTextureObject_t>(src->texture);
	t.dtype = src->dtype;
	t.rank = src->rank;
	long long count = 1;
	for (int i = 0; i < 3; ++i) {
		s.ext[i] = i < src->rank ? src->extent[i] : 1;
		t.origin[i] = i < src->rank ? src->origin[i] : 0;
		s.stride[i] = 0;
		if (s.ext[i] < 0 || t.origin[i] < 0) {
			return fail(IANE_GB_INVALID_ARGUMENT, "convolve texture source: negative extent or origin");
		}
		count *= s.ext[i];
	}
	DevView k{}, d{};
	int status = normalise_view(kernel, "convolve kernel", &k);
	if (status) return status;
	status = normalise_view(dst, "convolve destination", &d);
	if (status) return status;
	if (count > 0) {
		if (src->texture == 0) {
			return fail(IANE_GB_INVALID_ARGUMENT, "convolve texture: no texture for a nonempty view");
		}
		int ext[3];
		status = array_texture_extents(t.tex, ext);
		if (status) return status;
		for (int i = 0; i < 3; ++i) {
			if (static_cast<long long>(t.origin[i]) + s.ext[i] > ext[i]) {
				return fail(IANE_GB_INVALID_ARGUMENT, "convolve texture source: the view reaches outside the texture");
			}
		}
	}
	return convolve_checked(s, k, d, border, flags, stream, &t);
}

}  // extern "C"
