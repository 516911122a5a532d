/*
 * iane_gb C ABI: GB300 (sm_103a) kernels for IANE's N-dimensional convolution and the
 * Richardson-Lucy (RL) deconvolution iteration built on it.
 *
 * Every entry point takes plain pointers, sizes and a CUDA stream handle (passed as
 * `void*`, a `cudaStream_t`); no C++ or PyTorch type crosses this boundary. All image
 * pointers are device pointers borrowed for the duration of the stream-ordered work;
 * the caller keeps the storage alive until the stream has completed it, exactly as
 * IANE requires for CUDA views (include/iane/algorithms/convolution.hpp:88-89 of the
 * reference: "Keep all view storage valid until completion").
 *
 * Functions return IANE_GB_OK (0) or a negative iane_gb_status. The message of the
 * last failure on the calling thread is available through iane_gb_last_error(). No
 * entry point traps on the device; device-side waits are bounded and reported as
 * IANE_GB_DEVICE_TIMEOUT.
 *
 * Layout: a view is IANE's strided view (include/iane/view/const_device_image_view.hpp:8-50,
 * include/iane/math/offset.hpp:11-21): a base pointer to element (0,...,0), a rank
 * (1..3), extents with axis 0 fastest, and byte strides per axis. Strides may pad rows
 * and planes and may describe crops of larger allocations; the view extent is the
 * sampling boundary even for crops (include/iane/locator/image_locator.hpp:18-21).
 */
#ifndef IANE_GB_CAPI_H
#define IANE_GB_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IANE_GB_ABI_VERSION 2
#define IANE_GB_MAX_RANK 3

/* Element types. */
typedef enum iane_gb_dtype {
	IANE_GB_U8 = 1,
	IANE_GB_U16 = 2,
	IANE_GB_I16 = 3,
	IANE_GB_I32 = 4,
	IANE_GB_F32 = 5,
	IANE_GB_F64 = 6,
	IANE_GB_BF16 = 7,
	IANE_GB_I8 = 8,
	IANE_GB_U32 = 9,
	/* Packed 3-byte (r, g, b) pixel. Convolution treats each channel as its own u8 image
	 * with a float kernel and writes packed pixels: the custom element of the reference's
	 * convolution example (examples/convolution/main.cu:20-56, a per-channel double sum
	 * converted with the byte rule). */
	IANE_GB_RGB8 = 10
} iane_gb_dtype;

/* Boundary rules. clamp and zero are the reference's border_mode
 * (include/iane/locator/image_locator.hpp:14); mirror is an addition: half-sample
 * symmetric reflection (... c b a | a b c d | d c b ...), repeated with period 2n
 * for kernels wider than the image. */
typedef enum iane_gb_border {
	IANE_GB_BORDER_CLAMP = 0,
	IANE_GB_BORDER_ZERO = 1,
	IANE_GB_BORDER_MIRROR = 2
} iane_gb_border;

typedef enum iane_gb_status {
	IANE_GB_OK = 0,
	IANE_GB_INVALID_ARGUMENT = -1, /* the reference throws std::invalid_argument */
	IANE_GB_UNSUPPORTED = -2,      /* a type, rank or layout this library does not take */
	IANE_GB_CUDA_ERROR = -3,       /* the reference throws std::runtime_error (check_cuda) */
	IANE_GB_DEVICE_TIMEOUT = -4,   /* a bounded device wait gave up */
	IANE_GB_OUT_OF_MEMORY = -5,
	IANE_GB_LENGTH_ERROR = -6      /* scratch smaller than required (std::length_error) */
} iane_gb_status;

/* Convolution flags. */
#define IANE_GB_ACC_FAST 0u  /* FP32 accumulation for float kernels, int64 for integer pairs */
#define IANE_GB_ACC_EXACT 1u /* FP64 fma in kernel raster order: bit-identical to the reference */
/* Spectral convolution (no counterpart in the reference's convolve; the reference has FFTs in
 * include/iane/algorithms/fft/): f32/f64 source, kernel and destination; the border-padded
 * source and the kernel are transformed with cuFFT in FP64, multiplied and transformed back,
 * so results stay within the direct path's per-element bar while the work grows as
 * L log L (L = padded size) instead of voxels x taps. */
#define IANE_GB_CONV_FFT 2u  /* always the spectral path */
#define IANE_GB_CONV_AUTO 4u /* direct FP32 or spectral, whichever a cost model predicts faster */

typedef struct iane_gb_view {
	void* ptr;              /* device address of element (0,...,0) */
	int32_t dtype;          /* iane_gb_dtype */
	int32_t rank;           /* 1..IANE_GB_MAX_RANK */
	int32_t extent[3];      /* axis 0 fastest; unused axes ignored */
	int32_t reserved;
	int64_t stride[3];      /* byte strides; unused axes ignored */
} iane_gb_view;

/* Library identification. */
int iane_gb_abi_version(void);

/* Copy the calling thread's last error message into buf (NUL-terminated, truncated to
 * size). Returns the full message length. */
size_t iane_gb_last_error(char* buf, size_t size);

/* Read and clear the current device's status word after waiting for `stream`. Returns
 * IANE_GB_DEVICE_TIMEOUT if a bounded device-side wait of an earlier launch gave up. */
int iane_gb_device_status(void* stream);

/* Diagnostic: launch a kernel with one device-side wait of the given kind, bounded to
 * `limit_us` microseconds (1 .. 10^7):
 *   IANE_GB_PROBE_MBARRIER: an mbarrier nobody arrives on;
 *   IANE_GB_PROBE_COUNTER: a completion counter nothing raises (the persistent queues' wait);
 *     the wait also raises the run's abort flag;
 *   IANE_GB_PROBE_COUNTER_ABORT: the same counter, with another warp raising the abort flag
 *     after 1 ms -- the wait returns then and records nothing.
 * A wait that gives up records IANE_GB_DEVICE_TIMEOUT in the status word and the kernel ends;
 * the next iane_gb_device_status reports it, and the context stays usable. Every device-side
 * wait of this library has the same kind of bound (two seconds). */
#define IANE_GB_PROBE_MBARRIER 0
#define IANE_GB_PROBE_COUNTER 1
#define IANE_GB_PROBE_COUNTER_ABORT 2
int iane_gb_wait_probe(unsigned int limit_us, int kind, void* stream);

/* Diagnostic: measured FP32 fused multiply-add throughput of the current device in TFLOP/s
 * (2 flops per FMA), the ceiling of FP32-pipe-bound convolutions. paired = 0 issues scalar
 * FFMA, 1 the packed two-lane fma.rn.f32x2; independent chains on every lane of 8 blocks of
 * 256 threads per SM, best of three timed launches after a warm-up. Synchronises `stream`.
 * No counterpart in the reference. */
int iane_gb_fp32_peak_probe(int paired, double* tflops, void* stream);

/*
 * Direct N-D convolution. Replaces iane::convolve for CUDA memory views
 * (reference include/iane/algorithms/convolution.hpp:97-117, with the extent check of
 * include/iane/algorithms/transform.hpp:51-63):
 *
 *   dst[p] = sum_q kernel[q] * sample(src, p + size/2 - q)
 *
 * with the kernel flipped (true convolution), kernel extents positive and odd, dst of
 * the same extents as src and disjoint from both inputs. The kernel is a device view of
 * the same rank. Results follow the reference's casts (convolution.hpp:51-75):
 * u8 rounds half up and saturates; other integers saturate and map NaN to 0.
 * Supported: src u8/i8/u16/i16/i32/u32/f32/bf16/f64, kernel i32/f32/f64,
 * dst u8/i8/u16/i16/i32/u32/f32/f64; and rgb8 src and dst with an f32 kernel.
 */
int iane_gb_convolve(const iane_gb_view* src, const iane_gb_view* kernel,
	const iane_gb_view* dst, int border, unsigned flags, void* stream);

/*
 * A point-sampled CUDA texture as a convolution source: the reference's
 * texture_image_view<T, N> (include/iane/view/texture_image_view.hpp:26-98), which reads
 * texel origin + p at the texel centre. `texture` is a cudaTextureObject_t over a CUDA array
 * of `dtype` elements (u8, i8, u16, i16, i32, u32 or f32) with unnormalised coordinates,
 * point filtering and element-type reads, as iane_gb_texture_create makes it (and as the
 * reference's texture_image does, include/iane/resource/cuda/texture_image.hpp:49-80); the
 * view covers extent[] texels from origin[] (axis 0 fastest; unused axes ignored).
 */
typedef struct iane_gb_texture_view {
	uint64_t texture;
	int32_t dtype;
	int32_t rank;
	int32_t extent[3];
	int32_t origin[3];
} iane_gb_texture_view;

/* The reference's texture_image (include/iane/resource/cuda/texture_image.hpp:20-96): a
 * CUDA array of `extent` elements of `dtype` and its texture object on the current device.
 * An empty extent allocates nothing and yields texture 0. */
int iane_gb_texture_create(int dtype, int rank, const int32_t* extent, uint64_t* texture);

/* Upload a host or device view of the texture's dtype and extents into its array (the
 * reference's copy(view, texture_image), texture_image.hpp:98-140): rows must be contiguous
 * (stride[0] = element size), rows and planes may be padded. Asynchronous on `stream`. */
int iane_gb_texture_upload(uint64_t texture, const iane_gb_view* src, void* stream);

/* Destroy a texture made by iane_gb_texture_create and free its array. Waits for nothing:
 * the caller keeps it alive until work that reads it has finished. */
int iane_gb_texture_destroy(uint64_t texture);

/* iane_gb_convolve with a texture source: same formula, borders, flags (exact mode gives the
 * reference's bits; spectral flags are refused) and destination rules. */
int iane_gb_convolve_texture(const iane_gb_texture_view* src, const iane_gb_view* kernel,
	const iane_gb_view* dst, int border, unsigned flags, void* stream);

/*
 * Separable convolution: the convolution with the outer-product kernel
 * K[a,b,c] = taps[0][a] * taps[1][b] * taps[2][c], evaluated as one fused pass (axis 0,
 * then 1, then 2, intermediate rows kept on chip). taps[i] is a 1-D f32 device view of
 * odd length for axis i; there are exactly src->rank of them. src and dst are f32.
 * No counterpart in the reference (it has no separable path); its result equals
 * iane::convolve with the outer-product kernel, and equals successive convolve calls
 * with unit-extent kernels up to FP32 rounding.
 */
int iane_gb_convolve_separable(const iane_gb_view* src, const iane_gb_view* const* taps,
	const iane_gb_view* dst, int border, void* stream);

/*
 * Richardson-Lucy deconvolution as an IANE prepared algorithm
 * (reference include/iane/execution/prepared.hpp:120-146 for the prepare/run/scratch
 * protocol; examples/rl_deconvolution/main.cu:51-81 for the iteration):
 *
 *   sensitivity = convolve(1, adjoint, zero border)           (once, at prepare)
 *   estimate    = init(observed)
 *   repeat:  ratio    = observed / max(convolve(estimate, psf, zero), eps)
 *            estimate = estimate * (sens > 0 ? convolve(ratio, adjoint, zero) / max(sens, eps) : 0)
 *
 * adjoint = the PSF reversed along every axis. Each iteration is two fused passes over
 * HBM. The PSF is an f32 device view of odd extents with the image's rank; it is used as
 * given (callers normalise it, as examples/common/deconvolution.hpp:10-30 does).
 */
typedef struct iane_gb_rl_plan iane_gb_rl_plan;

#define IANE_GB_RL_INIT_OBSERVED 0 /* max(observed, eps): the reference example's start */
#define IANE_GB_RL_INIT_MEAN 1     /* flat start at max(mean(observed), eps) */
#define IANE_GB_RL_INIT_GIVEN 2    /* start from the values already in the estimate view */

/* Prepare for images of `extent` (rank 1..3). Copies the PSF, builds its adjoint and the
 * exact boundary-sensitivity table. Blocks until the copies are done. */
int iane_gb_rl_prepare(const iane_gb_view* psf, int rank, const int32_t* extent,
	void* stream, iane_gb_rl_plan** plan);

/* Precision path: images and PSF in BF16 for the convolutions, which run as implicit GEMMs
 * on the tcgen05 tensor cores with FP32 accumulation; the ratio, the division guard, the
 * update and the statistics stay FP32 (the estimate keeps an FP32 master copy). PSFs up to
 * 17 wide. No counterpart in the reference, which convolves in FP64. */
#define IANE_GB_RL_BF16_TENSOR 1u

/* FP32 path: one launch per pass (two per iteration) instead of one persistent launch for the
 * whole run. The estimates are the same bits (the statistics agree to rounding: the two
 * schedules group the FP32 partial sums differently); images small enough for 32 x 32 tiles
 * always take one launch per pass. */
#define IANE_GB_RL_PER_PASS 2u

/* iane_gb_rl_prepare with flags (0, or IANE_GB_RL_BF16_TENSOR and/or IANE_GB_RL_PER_PASS). */
int iane_gb_rl_prepare_ex(const iane_gb_view* psf, int rank, const int32_t* extent,
	unsigned flags, void* stream, iane_gb_rl_plan** plan);

/* Scratch bytes iane_gb_rl_run needs (ratio image, statistics), 256-byte aligned. */
size_t iane_gb_rl_scratch_bytes(const iane_gb_rl_plan* plan);

/* Run `iterations` RL iterations. observed: f32 or u8; estimate: f32 (the result,
 * packed or strided) or u8 (converted at the end with the reference's to_gray8,
 * examples/common/deconvolution.hpp:43-55; then scratch also holds the float estimate).
 * If stats is non-NULL it is a DEVICE array of 2*iterations doubles that receives, per
 * iteration, the flux sum(estimate) and the relative L2 change
 * ||e_new - e_old|| / ||e_old||, from FP32 Kahan partials combined in FP64. */
int iane_gb_rl_run(iane_gb_rl_plan* plan, const iane_gb_view* observed,
	const iane_gb_view* estimate, int iterations, float epsilon, int init,
	void* scratch, size_t scratch_bytes, double* stats, void* stream);

/* Bytes of device scratch iane_gb_rl_run_host needs: run scratch plus packed device
 * copies of the observed and estimate images. */
size_t iane_gb_rl_host_scratch_bytes(const iane_gb_rl_plan* plan, int observed_dtype);

/* End-to-end run from packed HOST images (the reference's run_prepared_on staging,
 * include/iane/execution/run_on.hpp:86-178): upload observed, run, download the f32
 * estimate, then wait for the stream. Host buffers should be pinned for full speed. */
int iane_gb_rl_run_host(iane_gb_rl_plan* plan, const void* host_observed, int observed_dtype,
	float* host_estimate, int iterations, float epsilon, int init,
	void* scratch, size_t scratch_bytes, void* stream);

/* Release a plan (after the stream has finished work that uses it). NULL is accepted. */
int iane_gb_rl_destroy(iane_gb_rl_plan* plan);

/*
 * Flat morphology (the reference's include/iane/algorithms/morphology/morphology.hpp, rank 1-3
 * here): erode(p) = min over footprint offsets o of src(p + o), dilate(p) = max of src(p - o),
 * o = position - radius over the (2 radius + 1)-box in raster order, with the border rule
 * (clamp, zero -- out-of-range samples are the value 0 -- or mirror), NaN ignored (an all-NaN
 * neighbourhood gives +inf / -inf) and the first of equal values in scan order kept, so
 * results are bit-identical to the reference's. `footprint` is NULL for the whole box, or a
 * device mask of prod(2 radius + 1) bytes in raster order (axis 0 fastest, nonzero =
 * contained; the reference's flat_footprint predicate). src and dst have the same extents and
 * element type (u8, i8, u16, i16, i32, u32, f32, f64) and do not overlap.
 */
#define IANE_GB_ERODE 0
#define IANE_GB_DILATE 1
#define IANE_GB_OPENING 2 /* erosion, then dilation (morphology.hpp:216-221) */
#define IANE_GB_CLOSING 3 /* dilation, then erosion */
int iane_gb_morphology(const iane_gb_view* src, const iane_gb_view* dst, const int32_t* radius,
	const uint8_t* footprint, int op, int border, void* stream);

/* Opening or closing through a packed intermediate in `scratch` (device, at least
 * iane_gb_morphology_scratch_bytes for the image's element type and extents); src and dst may
 * be the same view (exact in-place execution, as the reference's prepared compound). */
size_t iane_gb_morphology_scratch_bytes(int dtype, int rank, const int32_t* extent);
int iane_gb_morphology_compound(const iane_gb_view* src, const iane_gb_view* dst, const int32_t* radius,
	const uint8_t* footprint, int op, int border, void* scratch, size_t scratch_bytes, void* stream);

/*
 * Wiener deconvolution, prepared (the reference's examples/wiener/main.cu:44-83, 2-D there;
 * rank 1-3 here). prepare: `psf` is an f32 device view of the image's rank and no larger than
 * `extent` on any axis (the example normalises it to sum one first; it is used as given
 * here); it is centred at the origin with periodic wrap-around, transformed, and turned into
 * the filter conj(H) / (|H|^2 + noise); noise must be finite and positive. Synchronous.
 * run: restored = IFFT(FFT(observed) * filter) / N, periodic boundary, FP32 transforms;
 * observed is any scalar view except f64, restored u8 (the example's to_gray8: round half
 * up, saturate) or another scalar type (the reference's casts from the FP32 value).
 * `scratch` (device, >= iane_gb_wiener_scratch_bytes) holds the buffers and the FFT work
 * area. A plan runs on one stream at a time.
 */
typedef struct iane_gb_wiener_plan iane_gb_wiener_plan;
int iane_gb_wiener_prepare(const iane_gb_view* psf, int rank, const int32_t* extent, float noise, void* stream,
	iane_gb_wiener_plan** plan);
size_t iane_gb_wiener_scratch_bytes(const iane_gb_wiener_plan* plan);
int iane_gb_wiener_run(iane_gb_wiener_plan* plan, const iane_gb_view* observed, const iane_gb_view* restored,
	void* scratch, size_t scratch_bytes, void* stream);
int iane_gb_wiener_destroy(iane_gb_wiener_plan* plan);

/*
 * Batched Richardson-Lucy over many 2-D images of uneven size, each with its own PSF. No
 * counterpart in the reference (its example runs one image per process). The whole run --
 * every pass of every iteration of every image -- is ONE persistent launch over a device work
 * queue of (image, 64x64 tile) items in pass order; an image's pass waits only until that
 * image's previous pass is complete (per-image completion counters, bounded waits), never for
 * the rest of the batch. The run is captured into a CUDA graph on the first call and replayed
 * while the views, scratch and parameters stay the same. A work item is a run of 1, 2 or 4
 * consecutive tiles along x of one image (items of narrow PSFs carry the per-item queue,
 * dependency and completion work over several tiles).
 * psfs: `count` f32 2-D device views (odd extents up to 31 x 63); extents: 2*count ints
 * (nx, ny per image). IANE_GB_BATCH_AUTOTUNE times the launch's CTAs per SM, its queue order
 * (largest images first, or grouped by PSF width) and the work items' shapes (the grouping level:
 * 0 one tile per item; 1 two tiles for PSFs up to 11 wide; 2 four tiles for PSFs up to 11 wide;
 * 3 four tiles up to 7 wide and two up to 15) on this batch and caches the choice per (image
 * shapes, PSF sizes, dtype, SM count) in the file named by the environment variable
 * IANE_GB_TUNE_CACHE (default $HOME/.cache/iane_gb300_tune.txt).
 */
typedef struct iane_gb_rl_batch iane_gb_rl_batch;
#define IANE_GB_BATCH_AUTOTUNE 1u

int iane_gb_rl_batch_prepare(const iane_gb_view* psfs, int count, const int32_t* extents,
	unsigned flags, void* stream, iane_gb_rl_batch** batch);
size_t iane_gb_rl_batch_scratch_bytes(const iane_gb_rl_batch* batch);
/* Width of every image's work items: 64 x the tiles per item (their height is 64). */
int iane_gb_rl_batch_tiles(const iane_gb_rl_batch* batch, int32_t* tile_width);
/* The persistent launch's CTAs per SM, queue order (0: largest images first, 1: by PSF width)
 * and grouping level of the work items. */
int iane_gb_rl_batch_config(const iane_gb_rl_batch* batch, int32_t* blocks_per_sm, int32_t* order,
	int32_t* grouping);
/* Pin the launch configuration (for example one tuned offline): CTAs per SM from 1 to the
 * kernel's occupancy, order 0 or 1, grouping 0 to 3. The next run captures a new graph; results
 * are the same bits whatever the configuration. */
int iane_gb_rl_batch_configure(iane_gb_rl_batch* batch, int blocks_per_sm, int order, int grouping);
/* observed / estimates: `count` views each (observed f32 or u8, estimate f32 or u8). */
int iane_gb_rl_batch_run(iane_gb_rl_batch* batch, const iane_gb_view* observed,
	const iane_gb_view* estimates, int iterations, float epsilon, int init, void* scratch,
	size_t scratch_bytes, void* stream);
int iane_gb_rl_batch_destroy(iane_gb_rl_batch* batch);

/*
 * Learned warm start: kernels of a small 3-D encoder-decoder CNN (no counterpart in the
 * reference). Activations are BF16 (uint16_t bit patterns) in the C8 layout: channel octets,
 * each voxel-major with its 8 channels contiguous -- element (c, v) of a volume of V voxels
 * at ((c / 8) * V + v) * 8 + c % 8, ceil(C / 8) octets, voxels v = (z * h + y) * w + x.
 * FP32 outputs, residuals and targets are planar [c][v]. Weights are BF16 [co][ci][27]
 * with tap t = tx + 3 ty + 9 tz reading x(v + (tx-1, ty-1, tz-1)) (cross-correlation);
 * accumulation is FP32.
 */
/* y = act(bias + conv(concat(x0[c0], x1[c1]), weights) (+ residual, co == 1)), zero padding;
 * mask (co channels, optional): y *= (mask > 0). Writes y16 (bf16) and/or y32 (f32). co <= 64. */
int iane_gb_cnn_conv3(const uint16_t* x0, int c0, const uint16_t* x1, int c1, int d, int h, int w,
	const uint16_t* weights, const float* bias, int co, uint16_t* y16, float* y32,
	const float* residual, int act, const uint16_t* mask, void* stream);
/* dw[co][ci][t] += sum_v dy[co](v) x[ci](v + t - 1); db[co] += sum_v dy[co](v) (FP32,
 * deterministic split-K through `scratch`). c0 a multiple of 8 when c1 > 0; x0, x1 16-byte
 * aligned. */
size_t iane_gb_cnn_wgrad_scratch_bytes(int c0, int c1, int d, int h, int w, int co);
int iane_gb_cnn_conv3_wgrad(const uint16_t* x0, int c0, const uint16_t* x1, int c1, int d, int h, int w,
	const uint16_t* dy, int co, float* dw, float* db, void* scratch, size_t scratch_bytes, void* stream);
/* flipped[ci][co][26 - t] = weights[co][ci][t]: conv3 with these gives the input gradient. */
int iane_gb_cnn_flip(const uint16_t* weights, int co, int ci, uint16_t* flipped, void* stream);
int iane_gb_cnn_pool2(const uint16_t* x, int c, int d, int h, int w, uint16_t* y, void* stream);
int iane_gb_cnn_pool2_grad(const uint16_t* dy, int c, int d, int h, int w, uint16_t* dx,
	const uint16_t* mask, int accumulate, void* stream);
int iane_gb_cnn_up2(const uint16_t* x, int c, int d, int h, int w, uint16_t* y, void* stream);
int iane_gb_cnn_up2_grad(const uint16_t* dy, int c, int d, int h, int w, uint16_t* dx,
	const uint16_t* mask, void* stream);
/* *loss += mean((y - target)^2) (device double); dy = 2 (y - target) / n as bf16, a
 * one-channel C8 tensor (slot 0 of each voxel's octet). */
int iane_gb_cnn_mse(const float* y, const float* target, long long n, uint16_t* dy, double* loss,
	void* stream);
/* Tensor-core forward of conv3 (tcgen05, FP32 accumulation in TMEM) on C8 inputs with
 * weights packed by iane_gb_cnn_tc_pack. c0 is a multiple of 16 when c1 > 0; the BF16
 * output needs co a multiple of 8; buffers 16-byte aligned. No mask operand (forward only). */
size_t iane_gb_cnn_tc_packed_bytes(int co, int c0, int c1);
int iane_gb_cnn_tc_pack(const uint16_t* weights, int co, int c0, int c1, uint16_t* packed, void* stream);
int iane_gb_cnn_conv3_tc(const uint16_t* x0, int c0, const uint16_t* x1, int c1, int d, int h, int w,
	const uint16_t* packed, const float* bias, int co, uint16_t* y16, float* y32, const float* residual,
	int act, void* stream);
/* Adam step on FP32 parameters (grads scaled by grad_scale), refreshing their BF16 copy. */
int iane_gb_cnn_adam(float* params, uint16_t* params16, const float* grads, float* m, float* v,
	long long n, float lr, float beta1, float beta2, float eps, int step, float grad_scale,
	void* stream);

/*
 * Allocation-free Richardson-Lucy. No counterpart in the reference.
 *
 * For callers that must not allocate device memory: plugins inside a host application that
 * owns the device allocator or enforces a memory budget, and latency-bound loops that cannot
 * block in the allocator (cudaMalloc and cudaFree may synchronise the whole device). It runs
 * the same iteration as iane_gb_rl_prepare + iane_gb_rl_run, with
 * the same kernels and results, but calls no cudaMalloc, cudaFree or other allocating
 * routine: its scratch (ratio image, work estimate, edge-sensitivity table, reduction
 * partials) is one static device array of about 32.4 MiB that every GPU loading this
 * library keeps until the process exits. The caller passes the PSF (f32 device view, odd
 * extents, the image rank, used as given), the observed image (f32 or u8) and the estimate
 * (f32 or u8, as iane_gb_rl_run). Limits, rejected with IANE_GB_LENGTH_ERROR: at most
 * 4194304 voxels counting rows padded to a multiple of 4, nx + ny + nz <= 65536, PSF width
 * <= 31, height and depth <= 63, at most 32768 taps. No statistics are produced.
 *
 * The first call on a device looks up the array's device address with that device
 * current; make that first call before any stream capture. The mean start's reduction uses
 * at most 4096 blocks of partial sums. All calls share the one array:
 * calls whose GPU work overlaps (different streams, or different host threads, without
 * ordering between them) race on it and corrupt each other's results.
 */
int iane_gb_rl_run_noalloc(const iane_gb_view* psf, const iane_gb_view* observed,
	const iane_gb_view* estimate, int iterations, float epsilon, int init, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* IANE_GB_CAPI_H */
