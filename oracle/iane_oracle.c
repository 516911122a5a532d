/*
 * CPU oracle for the IANE convolution and Richardson-Lucy path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker: it is loaded by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and by nothing on the
 * product path. It restates, in plain C, the reference algorithm so that the GPU
 * kernels can be compared with it on the GPU host, where the reference sources are
 * not available. It is pinned against the reference itself (the reference's headers
 * compiled here by oracle/build.py into oracle/_ref, see tests/test_oracle.py)
 * and against the golden vectors in tests/golden/.
 *
 * Reference (JanKolomaznik/iane) citations:
 *   per-output filter   include/iane/algorithms/convolution.hpp:23-77
 *   argument checks     include/iane/algorithms/convolution.hpp:107-113,
 *                       include/iane/algorithms/transform.hpp:51-63
 *   border rule         include/iane/locator/image_locator.hpp:14,40-56
 *   raster order        include/iane/math/index.hpp:53-64 (axis 0 fastest)
 *   strided addressing  include/iane/math/offset.hpp:11-21
 *   RL iteration        examples/rl_deconvolution/main.cu:12-81
 *   to_gray8            examples/common/deconvolution.hpp:43-55
 *   CPU worker split    include/iane/algorithms/for_each.hpp:75-134
 *
 * Mirror border and separable convolution are not in the reference; they are defined
 * here the way the GPU library defines them (half-sample symmetric reflection; axis 0
 * pass, then axis 1, then axis 2, with an f32 intermediate).
 *
 * Build with -ffp-contract=off so that no a*b+c outside the explicit fma() calls is
 * contracted differently on x86-64 and aarch64.
 */
#include "../include/iane_gb/capi.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_OK 0
#define ORACLE_EINVAL -1
#define ORACLE_EUNSUP -2
#define ORACLE_ENOMEM -5

/* ------------------------------------------------------------------------------------ */
/* element access                                                                         */

static float bf16_to_float(uint16_t h)
{
	uint32_t u = (uint32_t)h << 16;
	float f;
	memcpy(&f, &u, sizeof f);
	return f;
}

static uint16_t float_to_bf16(float f)
{
	uint32_t u;
	memcpy(&u, &f, sizeof u);
	if ((u & 0x7fffffffu) > 0x7f800000u) {
		return (uint16_t)((u >> 16) | 0x40u); /* quiet NaN */
	}
	const uint32_t rounding = 0x7fffu + ((u >> 16) & 1u);
	return (uint16_t)((u + rounding) >> 16);
}

static int dtype_size(int dtype)
{
	switch (dtype) {
	case IANE_GB_U8: return 1;
	case IANE_GB_U16: return 2;
	case IANE_GB_I16: return 2;
	case IANE_GB_I32: return 4;
	case IANE_GB_F32: return 4;
	case IANE_GB_F64: return 8;
	case IANE_GB_BF16: return 2;
	case IANE_GB_I8: return 1;
	case IANE_GB_U32: return 4;
	case IANE_GB_RGB8: return 3;
	default: return 0;
	}
}

static double load_double(const char* p, int dtype)
{
	switch (dtype) {
	case IANE_GB_U8: return (double)*(const uint8_t*)p;
	case IANE_GB_U16: { uint16_t v; memcpy(&v, p, 2); return (double)v; }
	case IANE_GB_I16: { int16_t v; memcpy(&v, p, 2); return (double)v; }
	case IANE_GB_I32: { int32_t v; memcpy(&v, p, 4); return (double)v; }
	case IANE_GB_F32: { float v; memcpy(&v, p, 4); return (double)v; }
	case IANE_GB_F64: { double v; memcpy(&v, p, 8); return v; }
	case IANE_GB_BF16: { uint16_t v; memcpy(&v, p, 2); return (double)bf16_to_float(v); }
	case IANE_GB_I8: return (double)*(const int8_t*)p;
	case IANE_GB_U32: { uint32_t v; memcpy(&v, p, 4); return (double)v; }
	default: return 0.0;
	}
}

/* The reference's result conversion, include/iane/algorithms/convolution.hpp:51-75. */
static void store_double(char* p, int dtype, double sum)
{
	switch (dtype) {
	case IANE_GB_U8: {
		uint8_t r;
		if (!(sum > 0.0)) {
			r = 0;
		} else if (sum >= 255.0) {
			r = 255;
		} else {
			const unsigned int integer = (unsigned int)sum;
			r = (uint8_t)(integer + (sum - integer >= 0.5));
		}
		*(uint8_t*)p = r;
		return;
	}
	case IANE_GB_U16: {
		uint16_t r;
		if (sum != sum) r = 0;
		else if (sum <= 0.0) r = 0;
		else if (sum >= 65535.0) r = 65535;
		else r = (uint16_t)sum;
		memcpy(p, &r, 2);
		return;
	}
	case IANE_GB_I16: {
		int16_t r;
		if (sum != sum) r = 0;
		else if (sum <= -32768.0) r = -32768;
		else if (sum >= 32767.0) r = 32767;
		else r = (int16_t)sum;
		memcpy(p, &r, 2);
		return;
	}
	case IANE_GB_I32: {
		int32_t r;
		if (sum != sum) r = 0;
		else if (sum <= -2147483648.0) r = INT32_MIN;
		else if (sum >= 2147483647.0) r = INT32_MAX;
		else r = (int32_t)sum;
		memcpy(p, &r, 4);
		return;
	}
	case IANE_GB_I8: {
		int8_t r;
		if (sum != sum) r = 0;
		else if (sum <= -128.0) r = -128;
		else if (sum >= 127.0) r = 127;
		else r = (int8_t)sum;
		*(int8_t*)p = r;
		return;
	}
	case IANE_GB_U32: {
		uint32_t r;
		if (sum != sum) r = 0;
		else if (sum <= 0.0) r = 0;
		else if (sum >= 4294967295.0) r = UINT32_MAX;
		else r = (uint32_t)sum;
		memcpy(p, &r, 4);
		return;
	}
	case IANE_GB_F32: { float r = (float)sum; memcpy(p, &r, 4); return; }
	case IANE_GB_F64: memcpy(p, &sum, 8); return;
	case IANE_GB_BF16: { uint16_t r = float_to_bf16((float)sum); memcpy(p, &r, 2); return; }
	default: return;
	}
}

/* ------------------------------------------------------------------------------------ */
/* border rule                                                                            */

/* Map one coordinate into [0, n) or report that the sample is zero.
 * clamp/zero: include/iane/locator/image_locator.hpp:44-52. mirror: half-sample
 * symmetric, period 2n. */
static int map_coordinate(int64_t c, int64_t n, int border, int64_t* out)
{
	if (c >= 0 && c < n) {
		*out = c;
		return 1;
	}
	if (border == IANE_GB_BORDER_ZERO || n <= 0) {
		return 0;
	}
	if (border == IANE_GB_BORDER_CLAMP) {
		*out = c < 0 ? 0 : n - 1;
		return 1;
	}
	const int64_t period = 2 * n;
	int64_t m = c % period;
	if (m < 0) {
		m += period;
	}
	*out = m < n ? m : period - 1 - m;
	return 1;
}

/* ------------------------------------------------------------------------------------ */
/* convolution                                                                            */

typedef struct conv_job {
	const iane_gb_view* src;
	const iane_gb_view* kernel;
	const iane_gb_view* dst;
	int border;
	int64_t ext[3];
	int64_t kext[3];
	int64_t rows;       /* ext[1] * ext[2] */
	int64_t next_row;   /* shared work counter */
	pthread_mutex_t lock;
	const double* coef; /* kernel coefficients as double, packed raster order */
} conv_job;

static int check_view(const iane_gb_view* v)
{
	if (!v || v->rank < 1 || v->rank > 3 || dtype_size(v->dtype) == 0) {
		return 0;
	}
	for (int i = 0; i < v->rank; ++i) {
		if (v->extent[i] < 0) {
			return 0;
		}
	}
	return 1;
}

static void view_extents(const iane_gb_view* v, int64_t ext[3])
{
	for (int i = 0; i < 3; ++i) {
		ext[i] = i < v->rank ? v->extent[i] : 1;
	}
}

static const char* view_at(const iane_gb_view* v, int64_t x, int64_t y, int64_t z)
{
	int64_t offset = x * v->stride[0];
	if (v->rank > 1) offset += y * v->stride[1];
	if (v->rank > 2) offset += z * v->stride[2];
	return (const char*)v->ptr + offset;
}

/* One output: the taps in kernel raster order, fma in double, starting from +0.0
 * (convolution.hpp:37-49). Out-of-range zero-border samples contribute fma(0, k, sum)
 * exactly as the reference's value-initialised sample does. */
static double convolve_one(const conv_job* job, int64_t x, int64_t y, int64_t z)
{
	const iane_gb_view* src = job->src;
	const int border = job->border;
	const int64_t cx = job->kext[0] / 2, cy = job->kext[1] / 2, cz = job->kext[2] / 2;
	double sum = 0.0;
	const double* coef = job->coef;
	for (int64_t qz = 0; qz < job->kext[2]; ++qz) {
		int64_t sz = 0;
		const int okz = map_coordinate(z + cz - qz, job->ext[2], border, &sz);
		for (int64_t qy = 0; qy < job->kext[1]; ++qy) {
			int64_t sy = 0;
			const int oky = okz && map_coordinate(y + cy - qy, job->ext[1], border, &sy);
			for (int64_t qx = 0; qx < job->kext[0]; ++qx, ++coef) {
				int64_t sx = 0;
				double value = 0.0;
				if (oky && map_coordinate(x + cx - qx, job->ext[0], border, &sx)) {
					value = load_double(view_at(src, sx, sy, sz), src->dtype);
				}
				sum = fma(value, *coef, sum);
			}
		}
	}
	return sum;
}

/* The same loop with typed f32 loads, for the timed CPU baseline. */
static double convolve_one_f32(const conv_job* job, int64_t x, int64_t y, int64_t z)
{
	const iane_gb_view* src = job->src;
	const int border = job->border;
	const int64_t cx = job->kext[0] / 2, cy = job->kext[1] / 2, cz = job->kext[2] / 2;
	double sum = 0.0;
	const double* coef = job->coef;
	const char* base = (const char*)src->ptr;
	const int64_t s0 = src->stride[0];
	const int64_t s1 = src->rank > 1 ? src->stride[1] : 0;
	const int64_t s2 = src->rank > 2 ? src->stride[2] : 0;
	for (int64_t qz = 0; qz < job->kext[2]; ++qz) {
		int64_t sz = 0;
		const int okz = map_coordinate(z + cz - qz, job->ext[2], border, &sz);
		for (int64_t qy = 0; qy < job->kext[1]; ++qy) {
			int64_t sy = 0;
			const int oky = okz && map_coordinate(y + cy - qy, job->ext[1], border, &sy);
			const char* row = base + sy * s1 + sz * s2;
			for (int64_t qx = 0; qx < job->kext[0]; ++qx, ++coef) {
				int64_t sx = 0;
				float value = 0.0f;
				if (oky && map_coordinate(x + cx - qx, job->ext[0], border, &sx)) {
					memcpy(&value, row + sx * s0, sizeof value);
				}
				sum = fma((double)value, *coef, sum);
			}
		}
	}
	return sum;
}

static void* conv_worker(void* arg)
{
	conv_job* job = (conv_job*)arg;
	const int fast = job->src->dtype == IANE_GB_F32;
	for (;;) {
		pthread_mutex_lock(&job->lock);
		const int64_t row = job->next_row;
		job->next_row += 4;
		pthread_mutex_unlock(&job->lock);
		if (row >= job->rows) {
			break;
		}
		const int64_t end = row + 4 < job->rows ? row + 4 : job->rows;
		for (int64_t r = row; r < end; ++r) {
			const int64_t y = r % job->ext[1];
			const int64_t z = r / job->ext[1];
			for (int64_t x = 0; x < job->ext[0]; ++x) {
				const double sum = fast ? convolve_one_f32(job, x, y, z) : convolve_one(job, x, y, z);
				store_double((char*)view_at(job->dst, x, y, z), job->dst->dtype, sum);
			}
		}
	}
	return NULL;
}

static int run_workers(void* (*fn)(void*), void* job, int threads)
{
	if (threads < 1) {
		threads = 1;
	}
	if (threads == 1) {
		fn(job);
		return ORACLE_OK;
	}
	pthread_t* ids = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
	if (!ids) {
		return ORACLE_ENOMEM;
	}
	int started = 0;
	for (int t = 1; t < threads; ++t) {
		if (pthread_create(&ids[t], NULL, fn, job) == 0) {
			++started;
		} else {
			ids[t] = 0;
		}
	}
	fn(job);
	for (int t = 1; t < threads; ++t) {
		if (ids[t]) {
			pthread_join(ids[t], NULL);
		}
	}
	(void)started;
	free(ids);
	return ORACLE_OK;
}

/* Convolve src with kernel into dst (all host memory). Returns 0 or a negative status.
 * Argument rules of convolution.hpp:107-113 and transform.hpp:51-63. */
int oracle_convolve(const iane_gb_view* src, const iane_gb_view* kernel, const iane_gb_view* dst,
	int border, int threads)
{
	if (!check_view(src) || !check_view(kernel) || !check_view(dst) ||
	    src->rank != kernel->rank || src->rank != dst->rank) {
		return ORACLE_EINVAL;
	}
	if (border < IANE_GB_BORDER_CLAMP || border > IANE_GB_BORDER_MIRROR) {
		return ORACLE_EINVAL;
	}
	for (int i = 0; i < kernel->rank; ++i) {
		if (kernel->extent[i] <= 0 || kernel->extent[i] % 2 == 0) {
			return ORACLE_EINVAL;
		}
		if (src->extent[i] != dst->extent[i]) {
			return ORACLE_EINVAL;
		}
	}
	if (src->dtype == IANE_GB_RGB8 || dst->dtype == IANE_GB_RGB8) {
		/* Packed (r, g, b) pixels (examples/convolution/main.cu:20-56): the sum of pixel * tap
		 * is per channel, each channel's byte-times-f32 product is exact in double, so each
		 * channel is the u8 convolution of that channel. */
		if (src->dtype != dst->dtype || kernel->dtype != IANE_GB_F32) {
			return ORACLE_EINVAL;
		}
		for (int c = 0; c < 3; ++c) {
			iane_gb_view sc = *src, dc = *dst;
			sc.dtype = dc.dtype = IANE_GB_U8;
			sc.ptr = (char*)src->ptr + c;
			dc.ptr = (char*)dst->ptr + c;
			const int status = oracle_convolve(&sc, kernel, &dc, border, threads);
			if (status) {
				return status;
			}
		}
		return ORACLE_OK;
	}
	conv_job job;
	memset(&job, 0, sizeof job);
	job.src = src;
	job.kernel = kernel;
	job.dst = dst;
	job.border = border;
	view_extents(src, job.ext);
	view_extents(kernel, job.kext);
	if (job.ext[0] == 0 || job.ext[1] == 0 || job.ext[2] == 0) {
		return ORACLE_OK;
	}
	const int64_t taps = job.kext[0] * job.kext[1] * job.kext[2];
	double* coef = (double*)malloc((size_t)taps * sizeof(double));
	if (!coef) {
		return ORACLE_ENOMEM;
	}
	int64_t i = 0;
	for (int64_t qz = 0; qz < job.kext[2]; ++qz)
		for (int64_t qy = 0; qy < job.kext[1]; ++qy)
			for (int64_t qx = 0; qx < job.kext[0]; ++qx)
				coef[i++] = load_double(view_at(kernel, qx, qy, qz), kernel->dtype);
	job.coef = coef;
	job.rows = job.ext[1] * job.ext[2];
	pthread_mutex_init(&job.lock, NULL);
	const int status = run_workers(conv_worker, &job, threads);
	pthread_mutex_destroy(&job.lock);
	free(coef);
	return status;
}

/* Separable convolution: successive 1-D convolutions along axis 0, 1, 2 with an f32
 * intermediate, each pass exactly an oracle_convolve with a unit-extent kernel. */
int oracle_convolve_separable(const iane_gb_view* src, const iane_gb_view* const* taps,
	const iane_gb_view* dst, int border, int threads)
{
	if (!check_view(src) || !check_view(dst) || src->rank != dst->rank ||
	    src->dtype != IANE_GB_F32 || dst->dtype != IANE_GB_F32 || !taps) {
		return ORACLE_EINVAL;
	}
	const int rank = src->rank;
	int64_t ext[3];
	view_extents(src, ext);
	const int64_t count = ext[0] * ext[1] * ext[2];
	float* work[2] = {NULL, NULL};
	if (count > 0) {
		work[0] = (float*)malloc((size_t)count * sizeof(float));
		work[1] = (float*)malloc((size_t)count * sizeof(float));
		if (!work[0] || !work[1]) {
			free(work[0]);
			free(work[1]);
			return ORACLE_ENOMEM;
		}
	}
	int status = ORACLE_OK;
	const iane_gb_view* in = src;
	iane_gb_view packed[2];
	for (int axis = 0; axis < rank && status == ORACLE_OK; ++axis) {
		const iane_gb_view* t = taps[axis];
		if (!check_view(t) || t->rank != 1 || t->dtype != IANE_GB_F32) {
			status = ORACLE_EINVAL;
			break;
		}
		iane_gb_view k;
		memset(&k, 0, sizeof k);
		k.ptr = t->ptr;
		k.dtype = IANE_GB_F32;
		k.rank = rank;
		for (int i = 0; i < rank; ++i) {
			k.extent[i] = i == axis ? t->extent[0] : 1;
			k.stride[i] = i == axis ? t->stride[0] : 4;
		}
		const iane_gb_view* out = dst;
		if (axis + 1 < rank) {
			iane_gb_view* p = &packed[axis % 2];
			memset(p, 0, sizeof *p);
			p->ptr = work[axis % 2];
			p->dtype = IANE_GB_F32;
			p->rank = rank;
			int64_t stride = 4;
			for (int i = 0; i < rank; ++i) {
				p->extent[i] = src->extent[i];
				p->stride[i] = stride;
				stride *= src->extent[i];
			}
			out = p;
		}
		status = oracle_convolve(in, &k, out, border, threads);
		in = out;
	}
	free(work[0]);
	free(work[1]);
	return status;
}

/* ------------------------------------------------------------------------------------ */
/* Richardson-Lucy (examples/rl_deconvolution/main.cu:12-81)                             */

static iane_gb_view packed_view(void* ptr, int dtype, int rank, const int64_t ext[3])
{
	iane_gb_view v;
	memset(&v, 0, sizeof v);
	v.ptr = ptr;
	v.dtype = dtype;
	v.rank = rank;
	int64_t stride = dtype_size(dtype);
	for (int i = 0; i < rank; ++i) {
		v.extent[i] = (int32_t)ext[i];
		v.stride[i] = stride;
		stride *= ext[i];
	}
	return v;
}

/*
 * observed: packed host image of `observed_dtype` (u8 or f32); psf: packed f32 of
 * psf_extent; estimate: packed f32, in/out (read only for init == GIVEN).
 * stats (optional): 2*iterations doubles, per iteration flux and relative L2 change.
 * init: 0 = max(observed, eps) (main.cu:12-19), 1 = flat max(mean, eps), 2 = given.
 */
int oracle_rl(const void* observed, int observed_dtype, int rank, const int32_t* extent,
	const float* psf, const int32_t* psf_extent, int iterations, float epsilon, int init,
	float* estimate, double* stats, int threads)
{
	if (rank < 1 || rank > 3 || iterations < 0 || !(epsilon > 0.0f) || !isfinite(epsilon) ||
	    (observed_dtype != IANE_GB_U8 && observed_dtype != IANE_GB_F32) || init < 0 || init > 2) {
		return ORACLE_EINVAL;
	}
	int64_t ext[3] = {1, 1, 1};
	int64_t kext[3] = {1, 1, 1};
	for (int i = 0; i < rank; ++i) {
		ext[i] = extent[i];
		kext[i] = psf_extent[i];
		if (ext[i] < 0 || kext[i] <= 0 || kext[i] % 2 == 0) {
			return ORACLE_EINVAL;
		}
	}
	const int64_t count = ext[0] * ext[1] * ext[2];
	const int64_t taps = kext[0] * kext[1] * kext[2];
	if (count == 0) {
		return ORACLE_OK;
	}
	float* adjoint = (float*)malloc((size_t)taps * sizeof(float));
	float* ones = (float*)malloc((size_t)count * sizeof(float));
	float* sensitivity = (float*)malloc((size_t)count * sizeof(float));
	float* predicted = (float*)malloc((size_t)count * sizeof(float));
	float* correction = (float*)malloc((size_t)count * sizeof(float));
	if (!adjoint || !ones || !sensitivity || !predicted || !correction) {
		free(adjoint); free(ones); free(sensitivity); free(predicted); free(correction);
		return ORACLE_ENOMEM;
	}
	/* adjoint = reverse_copy of the packed PSF (main.cu:106-107): every axis flipped. */
	for (int64_t i = 0; i < taps; ++i) {
		adjoint[i] = psf[taps - 1 - i];
	}
	for (int64_t i = 0; i < count; ++i) {
		ones[i] = 1.0f;
	}
	iane_gb_view psf_v = packed_view((void*)psf, IANE_GB_F32, rank, kext);
	iane_gb_view adj_v = packed_view(adjoint, IANE_GB_F32, rank, kext);
	iane_gb_view ones_v = packed_view(ones, IANE_GB_F32, rank, ext);
	iane_gb_view sens_v = packed_view(sensitivity, IANE_GB_F32, rank, ext);
	iane_gb_view est_v = packed_view(estimate, IANE_GB_F32, rank, ext);
	iane_gb_view pred_v = packed_view(predicted, IANE_GB_F32, rank, ext);
	iane_gb_view corr_v = packed_view(correction, IANE_GB_F32, rank, ext);
	int status = oracle_convolve(&ones_v, &adj_v, &sens_v, IANE_GB_BORDER_ZERO, threads);
	free(ones);

	const uint8_t* obs8 = (const uint8_t*)observed;
	const float* obs32 = (const float*)observed;
#define OBS(i) (observed_dtype == IANE_GB_U8 ? (float)obs8[i] : obs32[i])
	if (status == ORACLE_OK && init != IANE_GB_RL_INIT_GIVEN) {
		float start = 0.0f;
		if (init == IANE_GB_RL_INIT_MEAN) {
			double total = 0.0;
			for (int64_t i = 0; i < count; ++i) {
				total += (double)OBS(i);
			}
			const float mean = (float)(total / (double)count);
			start = mean > epsilon ? mean : epsilon;
		}
		for (int64_t i = 0; i < count; ++i) {
			if (init == IANE_GB_RL_INIT_MEAN) {
				estimate[i] = start;
			} else {
				const float o = OBS(i);
				estimate[i] = o > epsilon ? o : epsilon;
			}
		}
	}
	for (int it = 0; it < iterations && status == ORACLE_OK; ++it) {
		status = oracle_convolve(&est_v, &psf_v, &pred_v, IANE_GB_BORDER_ZERO, threads);
		if (status != ORACLE_OK) {
			break;
		}
		for (int64_t i = 0; i < count; ++i) {
			const float p = predicted[i];
			predicted[i] = OBS(i) / (p > epsilon ? p : epsilon);
		}
		status = oracle_convolve(&pred_v, &adj_v, &corr_v, IANE_GB_BORDER_ZERO, threads);
		if (status != ORACLE_OK) {
			break;
		}
		double flux = 0.0, change = 0.0, norm = 0.0;
		for (int64_t i = 0; i < count; ++i) {
			const float s = sensitivity[i];
			const float factor = s > 0.0f ? correction[i] / (s > epsilon ? s : epsilon) : 0.0f;
			const float old = estimate[i];
			const float updated = old * factor;
			estimate[i] = updated;
			flux += (double)updated;
			const double d = (double)updated - (double)old;
			change += d * d;
			norm += (double)old * (double)old;
		}
		if (stats) {
			stats[2 * it] = flux;
			stats[2 * it + 1] = norm > 0.0 ? sqrt(change / norm) : 0.0;
		}
	}
#undef OBS
	free(adjoint); free(sensitivity); free(predicted); free(correction);
	return status;
}

/* The reference's final byte conversion (examples/common/deconvolution.hpp:43-55). */
void oracle_to_gray8(const float* values, uint8_t* out, int64_t count)
{
	for (int64_t i = 0; i < count; ++i) {
		const float v = values[i];
		if (!(v > 0.0f)) {
			out[i] = 0;
		} else if (v >= 255.0f) {
			out[i] = 255;
		} else {
			const unsigned int integer = (unsigned int)v;
			out[i] = (uint8_t)(integer + (v - integer >= 0.5f));
		}
	}
}

/* Boundary sensitivity of a zero-border convolution with `kernel` applied to an image of
 * ones, i.e. the first step of main.cu:62-64, exposed for direct checks. */
int oracle_sensitivity(const float* kernel, const int32_t* kernel_extent, int rank,
	const int32_t* extent, float* out, int threads)
{
	int64_t ext[3] = {1, 1, 1}, kext[3] = {1, 1, 1};
	for (int i = 0; i < rank; ++i) {
		ext[i] = extent[i];
		kext[i] = kernel_extent[i];
	}
	const int64_t count = ext[0] * ext[1] * ext[2];
	float* ones = (float*)malloc((size_t)(count > 0 ? count : 1) * sizeof(float));
	if (!ones) {
		return ORACLE_ENOMEM;
	}
	for (int64_t i = 0; i < count; ++i) {
		ones[i] = 1.0f;
	}
	iane_gb_view k = packed_view((void*)kernel, IANE_GB_F32, rank, kext);
	iane_gb_view s = packed_view(ones, IANE_GB_F32, rank, ext);
	iane_gb_view d = packed_view(out, IANE_GB_F32, rank, ext);
	const int status = oracle_convolve(&s, &k, &d, IANE_GB_BORDER_ZERO, threads);
	free(ones);
	return status;
}

/* ------------------------------------------------------------------------------------ */
/* flat morphology                                                                        */

/* erode / dilate (include/iane/algorithms/morphology/morphology.hpp:44-71): the footprint
 * box of (2 r + 1) per axis scanned in raster order, offsets o = position - r, mask[q]
 * selecting positions (NULL: all); erosion takes the minimum of src(p + o), dilation the
 * maximum of src(p - o), with the rule `value < result` (`>`) from +inf / -inf (the type's
 * max / lowest for integers), so NaN never replaces the running value and the first of
 * equal values stays. Out-of-range zero-border samples are the value 0. Values are compared
 * as doubles, which every supported element type converts to exactly. Single-threaded. */
int oracle_morphology(const iane_gb_view* src, const iane_gb_view* dst, const int32_t* radius,
	const uint8_t* mask, int dilate, int border)
{
	if (!check_view(src) || !check_view(dst) || src->rank != dst->rank || src->dtype != dst->dtype || !radius ||
	    border < IANE_GB_BORDER_CLAMP || border > IANE_GB_BORDER_MIRROR) {
		return ORACLE_EINVAL;
	}
	int64_t ext[3], r[3];
	view_extents(src, ext);
	for (int i = 0; i < 3; ++i) {
		r[i] = i < src->rank ? radius[i] : 0;
		if (r[i] < 0 || (i < src->rank && dst->extent[i] != src->extent[i])) {
			return ORACLE_EINVAL;
		}
	}
	double start;
	switch (src->dtype) {
	case IANE_GB_F32: case IANE_GB_F64: start = dilate ? -INFINITY : INFINITY; break;
	case IANE_GB_U8: start = dilate ? 0.0 : 255.0; break;
	case IANE_GB_I8: start = dilate ? -128.0 : 127.0; break;
	case IANE_GB_U16: start = dilate ? 0.0 : 65535.0; break;
	case IANE_GB_I16: start = dilate ? -32768.0 : 32767.0; break;
	case IANE_GB_I32: start = dilate ? -2147483648.0 : 2147483647.0; break;
	case IANE_GB_U32: start = dilate ? 0.0 : 4294967295.0; break;
	default: return ORACLE_EINVAL;
	}
	for (int64_t z = 0; z < ext[2]; ++z)
		for (int64_t y = 0; y < ext[1]; ++y)
			for (int64_t x = 0; x < ext[0]; ++x) {
				double m = start;
				int64_t q = 0;
				for (int64_t pz = 0; pz <= 2 * r[2]; ++pz)
					for (int64_t py = 0; py <= 2 * r[1]; ++py)
						for (int64_t px = 0; px <= 2 * r[0]; ++px, ++q) {
							if (mask && !mask[q]) {
								continue;
							}
							const int64_t ox = px - r[0], oy = py - r[1], oz = pz - r[2];
							const int64_t sx = dilate ? x - ox : x + ox;
							const int64_t sy = dilate ? y - oy : y + oy;
							const int64_t sz = dilate ? z - oz : z + oz;
							int64_t mx = 0, my = 0, mz = 0;
							double v = 0.0;
							if (map_coordinate(sx, ext[0], border, &mx) && map_coordinate(sy, ext[1], border, &my) &&
							    map_coordinate(sz, ext[2], border, &mz)) {
								v = load_double(view_at(src, mx, my, mz), src->dtype);
							}
							if (dilate ? v > m : v < m) {
								m = v;
							}
						}
				store_double((char*)view_at(dst, x, y, z), dst->dtype, m);
			}
	return ORACLE_OK;
}
