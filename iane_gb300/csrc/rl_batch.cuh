// Batched Richardson-Lucy over many images of uneven size, each with its own PSF.
//
// The whole run -- every pass of every iteration of every image -- is ONE persistent launch
// over a device work queue. The queue is the list of (image, run of 64x64 tiles) items of one pass,
// repeated once per phase (phase 2t = pass A of iteration t, 2t + 1 = pass B); item k is
// (phase k / T, entry k % T) for T items per pass. CTAs (a few per SM) take items from an
// atomic counter in queue order and run the tiled FP32 convolution body with that image's TMA
// map, PSF and fused epilogue. RL's only dependency is per image: a phase of an image reads
// (with a halo) what the image's previous phase wrote and overwrites what it read, so an item
// of phase p waits until all tiles of its image's phase p - 1 are done -- a per-image
// completion counter that reaches p * tiles -- instead of a grid-wide drain between passes.
// Images of the next phase start as soon as their own previous pass is complete.
//
// Progress: an item waits only for items earlier in the queue, which were handed to CTAs that
// are running, so the earliest unfinished item can always proceed. Every wait is bounded (two
// seconds of global time); a wait that gives up records IANE_GB_DEVICE_TIMEOUT in the status
// word and raises an abort flag that every other wait checks, so the launch ends promptly.
//
// The CUDA graph of a run holds the counter reset, the start values and that one launch; it is
// captured on the first run and replayed while the views, scratch and parameters are unchanged.
#pragma once

#include "rl.cuh"

#include <vector>

namespace iane_gb {

// Tile edge of every work item (64 x 64 outputs; the body is 2 x 2 warps of 32 x 32).
constexpr int kBatchTile = 64;

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
	int tiles;             // 64x64 tiles of this image (completions per phase)
	int write_out_final;
};

// `count` consecutive 64x64 tiles of one tile row of an image, from tile index `tile`: the
// item's shape is (64 count) x 64 (count is 1, 2 or 4, chosen per PSF size by the autotuner).
struct BatchItem {
	int image;
	int tile;
	int count;
	int image_tiles; // the image's 64x64 tiles (its completions per phase), read at hand-off
};

// Device words of a run, cleared before the launch: the queue counter, the abort flag and one
// completion counter per image.
struct BatchSync {
	unsigned int* queue;
	int* abort;
	unsigned int* done;
};

// The persistent launch (rl_batch_kernel.cu): `grid` CTAs of 128 threads, `smem` bytes of
// dynamic shared memory (batch_tile_smem over the batch), items * phases work items.
int launch_batch_persistent(const BatchImage* images, const BatchItem* items, int items_per_phase, int phases,
	BatchSync sync, int* status, int grid, size_t smem, cudaStream_t stream);

// Dynamic shared memory a tile of PSF width kx, height ky needs.
size_t batch_tile_smem(int kx, int ky);

// Resident CTAs per SM of the persistent kernel with `smem` bytes of dynamic shared memory.
int batch_blocks_per_sm(size_t smem);

// Fill the plan-dependent fields of one image's pass arguments and epilogues (rl.cu); the
// caller sets the buffer pointers, views and epsilon.
void rl_plan_fill_passes(const iane_gb_rl_plan* plan, TileArgs* pass_a, TileArgs* pass_b, EpiRatio* epi_a,
	EpiUpdate* epi_b, int* status);

}  // namespace iane_gb
