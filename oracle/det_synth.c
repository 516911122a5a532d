/*
 * Deterministic synthetic RL inputs for the parity fixtures -- TEST INFRASTRUCTURE ONLY.
 *
 * The fixture of the full-size 3-D RL configuration is made where the reference builds (its
 * own RL run on this input) and checked on the GPU host, so both machines must produce the
 * same observed volume bit for bit. numpy's generators and exp() promise that only within
 * one version and platform, so this file generates the input itself:
 *
 *   - random numbers: splitmix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number
 *     generators", OOPSLA 2014), 53-bit uniforms in [0, 1);
 *   - ellipsoid phantom: background plus `count` ellipsoids with uniform centres, radii and
 *     intensities, membership tested in double with IEEE +, -, *, / only;
 *   - blur: the oracle's own convolution (FP64 fma in kernel raster order, zero border) into a
 *     double image;
 *   - Poisson noise: Knuth's product-of-uniforms method on chunks of mean <= 256, with exp()
 *     of the chunk mean computed here by range reduction to |r| <= ln2/2 and the Taylor series
 *     to degree 20, so no libm result enters.
 *
 * The library is built with -ffp-contract=off, so no a*b+c is fused differently on x86-64 and
 * aarch64; every operation above is then correctly rounded IEEE arithmetic on both.
 */
#include "../include/iane_gb/capi.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

int oracle_convolve(const iane_gb_view* src, const iane_gb_view* kernel, const iane_gb_view* dst, int border,
	int threads);

static uint64_t splitmix64(uint64_t* state)
{
	uint64_t z = (*state += 0x9E3779B97F4A7C15ULL);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return z ^ (z >> 31);
}

static double uniform01(uint64_t* state)
{
	return (double)(splitmix64(state) >> 11) * (1.0 / 9007199254740992.0);
}

static double uniform(uint64_t* state, double lo, double hi)
{
	return lo + (hi - lo) * uniform01(state);
}

/* e^x for x in [-1000, 0]: x = k ln2 + r with k the nearest integer to x / ln2, e^r by its
 * Taylor series (|r| <= 0.347, so the degree-20 remainder is below 1e-28), times 2^k. */
static double det_exp(double x)
{
	const double ln2 = 0.6931471805599453;
	const double k = floor(x / ln2 + 0.5);
	const double r = x - k * ln2;
	double term = 1.0, sum = 1.0;
	for (int n = 1; n <= 20; ++n) {
		term = term * r / (double)n;
		sum = sum + term;
	}
	return ldexp(sum, (int)k);
}

/* One Poisson(mean) sample: the mean is split into equal chunks of at most 256 and each
 * chunk sampled by Knuth's method (count uniforms until their product drops below e^-chunk). */
static uint32_t det_poisson(uint64_t* state, double mean)
{
	if (!(mean > 0.0)) {
		return 0;
	}
	const double chunks = ceil(mean / 256.0);
	const double part = mean / chunks;
	const double limit = det_exp(-part);
	uint32_t total = 0;
	for (int c = 0; c < (int)chunks; ++c) {
		double product = uniform01(state);
		while (product > limit) {
			++total;
			product = product * uniform01(state);
		}
	}
	return total;
}

/*
 * truth (f32, packed nx*ny*nz, axis 0 fastest): background plus `count` ellipsoids with
 * centres uniform in [0, n) per axis, radii uniform in [rmin, rmax] per axis and intensity
 * uniform in [imin, imax]; observed = Poisson(max(truth (*) psf, 0)) with a zero-border
 * convolution. psf: packed f32 of psf_extent (odd). Returns 0 or a negative status.
 */
int oracle_det_rl_volume(int nx, int ny, int nz, int count, double rmin, double rmax, double imin, double imax,
	double background, uint64_t seed, const float* psf, const int32_t* psf_extent, float* truth, float* observed,
	int threads)
{
	if (nx <= 0 || ny <= 0 || nz <= 0 || count < 0 || !psf || !psf_extent || !truth || !observed) {
		return IANE_GB_INVALID_ARGUMENT;
	}
	const int64_t n = (int64_t)nx * ny * nz;
	for (int64_t i = 0; i < n; ++i) {
		truth[i] = (float)background;
	}
	uint64_t state = seed;
	const int ext[3] = {nx, ny, nz};
	for (int e = 0; e < count; ++e) {
		double centre[3], radius[3];
		for (int a = 0; a < 3; ++a) centre[a] = uniform(&state, 0.0, (double)ext[a]);
		for (int a = 0; a < 3; ++a) radius[a] = uniform(&state, rmin, rmax);
		const float value = (float)uniform(&state, imin, imax);
		int lo[3], hi[3];
		for (int a = 0; a < 3; ++a) {
			const double l = floor(centre[a] - radius[a]);
			const double h = ceil(centre[a] + radius[a]);
			lo[a] = l < 0.0 ? 0 : (int)l;
			hi[a] = h > (double)(ext[a] - 1) ? ext[a] - 1 : (int)h;
		}
		for (int z = lo[2]; z <= hi[2]; ++z) {
			const double dz = ((double)z - centre[2]) / radius[2];
			for (int y = lo[1]; y <= hi[1]; ++y) {
				const double dy = ((double)y - centre[1]) / radius[1];
				for (int x = lo[0]; x <= hi[0]; ++x) {
					const double dx = ((double)x - centre[0]) / radius[0];
					if (dx * dx + dy * dy + dz * dz <= 1.0) {
						truth[((int64_t)z * ny + y) * nx + x] += value;
					}
				}
			}
		}
	}
	double* blurred = (double*)malloc((size_t)n * sizeof(double));
	if (!blurred) {
		return IANE_GB_OUT_OF_MEMORY;
	}
	iane_gb_view src, ker, dst;
	memset(&src, 0, sizeof src);
	memset(&ker, 0, sizeof ker);
	memset(&dst, 0, sizeof dst);
	src.ptr = truth;
	src.dtype = IANE_GB_F32;
	src.rank = 3;
	dst.ptr = blurred;
	dst.dtype = IANE_GB_F64;
	dst.rank = 3;
	ker.ptr = (void*)psf;
	ker.dtype = IANE_GB_F32;
	ker.rank = 3;
	int64_t s4 = 4, s8 = 8, k4 = 4;
	for (int a = 0; a < 3; ++a) {
		src.extent[a] = dst.extent[a] = ext[a];
		src.stride[a] = s4;
		dst.stride[a] = s8;
		s4 *= ext[a];
		s8 *= ext[a];
		ker.extent[a] = psf_extent[a];
		ker.stride[a] = k4;
		k4 *= psf_extent[a];
	}
	const int status = oracle_convolve(&src, &ker, &dst, IANE_GB_BORDER_ZERO, threads);
	if (status != 0) {
		free(blurred);
		return status;
	}
	for (int64_t i = 0; i < n; ++i) {
		/* one stream per voxel, so the result does not depend on the visiting order */
		uint64_t voxel_state = seed ^ ((uint64_t)(i + 1) * 0xD1B54A32D192ED03ULL);
		splitmix64(&voxel_state);
		observed[i] = (float)det_poisson(&voxel_state, blurred[i] > 0.0 ? blurred[i] : 0.0);
	}
	free(blurred);
	return 0;
}
