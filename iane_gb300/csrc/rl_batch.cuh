// Batched Richardson-Lucy over many images of uneven size, each with its own PSF.
//
// Each pass of an iteration is one persistent launch per tile shape and PSF width class (the
// groups): the grid is a few CTAs
// per SM and every CTA pulls work items -- (image, tile) pairs sorted by PSF width -- from
// a device queue (an atomic counter over the item list) and runs the tiled FP32 convolution
// body with that image's TMA map, kernel and fused epilogue. Items of one image wait for
// nothing: a pass's launch starts only after the previous pass's launch has finished (stream
// order inside the CUDA graph), which is the only dependency RL has. The whole schedule --
// start values, then for every iteration pass A and pass B for the four groups on four
// graph branches -- is captured once into a CUDA graph and replayed by later runs.
#pragma once

#include "rl.cuh"

#include <vector>

namespace iane_gb {

// Device-side description of one image of the batch (64-byte aligned for the maps).
struct alignas(64) BatchImage {
	CUtensorMap map_est;   // TMA map of the work estimate (pass A source)
	CUtensorMap map_ratio; // TMA map of the ratio image (pass B source)
	TileArgs pass_a;       // kernel = PSF
	TileArgs pass_b;       // kernel = adjoint
	EpiRatio epi_a;
	EpiUpdate epi_b;       // write_out is set only in the last iteration (write_out_final)
	int kx;
	int tiles_x;
	int write_out_final;
	int pad_;
};

// PSF width classes: narrow kernels (kx <= 15) take far fewer registers and less shared
// memory than wide ones (17..31), so each class has its own kernel and the narrow one fits
// more blocks per SM. Work items form four groups: (tile shape, width class).
inline bool batch_wide(int kx) { return kx > 15; }
constexpr int kBatchGroups = 4;
inline int batch_group(int wx, int kx) { return (wx - 1) + 2 * (batch_wide(kx) ? 1 : 0); }

struct BatchItem {
	int image;
	int tile;
};

// Persistent pass kernels (rl_batch_pass.cu). wx = wy = 1 (32x32 tiles) or 2 (64x64); wide:
// the items' PSFs are 17..31 wide (else 1..15).
int launch_batch_pass(int wx, bool wide, bool pass_b, const BatchImage* images, const BatchItem* items, int count,
	unsigned int* counter, int last, int grid, size_t smem, cudaStream_t stream);

// Largest dynamic shared memory a pass of this tile shape needs for PSF width kx, height ky.
size_t batch_tile_smem(int wx, int kx, int ky);

// The pass-B kernel of a tile shape and width class (the larger register footprint), for
// occupancy queries.
const void* batch_kernel_handle(int wx, bool wide);

// Fill the plan-dependent fields of one image's pass arguments and epilogues (rl.cu); the
// caller sets the buffer pointers, views and epsilon.
void rl_plan_fill_passes(const iane_gb_rl_plan* plan, TileArgs* pass_a, TileArgs* pass_b, EpiRatio* epi_a,
	EpiUpdate* epi_b, int* status);

// Choose the tile shape (wx = 1: 32x32, 2: 64x64) of every image by timing both shapes on a
// GPU-filling batch of copies of that image, once per (shape, PSF size, dtype, SM count);
// choices persist in the tuning cache file.
int batch_autotune(const std::vector<int>& nx, const std::vector<int>& ny, const std::vector<int>& kx,
	const std::vector<int>& ky, const std::vector<iane_gb_rl_plan*>& plans, std::vector<int>& wx, cudaStream_t stream);

}  // namespace iane_gb
