// pp_tiled.cuh -- tile configuration and launchers of the shared-memory tiled kernels.
#pragma once

#include "pp_kernels.cuh"

namespace pp {

// Tile of sample voxels handled by one CTA: 2^lx x 2^ly x 2^lz (32..512 voxels),
// and the shared-memory budget of its footprint box, in floats (multiple of 4).
struct TileCfg {
    int lx, ly, lz;
    int cap;
};

bool tiled_supported(const LaunchArgs& a, const TileCfg& t);
// warp-specialised pull family (8 x 8 x 30 tiles, pp_ws.cuh): geometry test and
// launch (cudaErrorNotSupported for ops or layouts it does not take)
bool ws_supported(const LaunchArgs& a);
cudaError_t launch_ws_pull(int op, const LaunchArgs& a, cudaStream_t s);
// the affine pull on the same kernels (positions A * (i, j, k, 1) in place of a deformation)
cudaError_t launch_ws_pull_affine(const LaunchArgs& a, const AffineMap& A, cudaStream_t s);
cudaError_t launch_pull_tiled(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s);
cudaError_t launch_push_tiled(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s);
// the affine push on the tiled push kernels (positions A * (i, j, k, 1))
cudaError_t launch_push_tiled_affine(const LaunchArgs& a, const TileCfg& t, const AffineMap& A, cudaStream_t s);

// Geometry of the tile grid, computed on the host once per launch.
struct TileGrid {
    int lx, ly, lz;     // log2 tile sides
    int ntx, nty, ntz;  // tiles per dimension
    int ntiles;         // ntx * nty * ntz * nb (tiles of all batches)
    // q = (u * m) >> s equals u / n{x,y,z} for every u < 2^31 (multiply-shift division)
    unsigned long long mx, my, mz;
    int sx, sy, sz;
    int cap;            // box budget in floats
    int pmod;           // box row pitch P is chosen with P % 32 == pmod
    int img_tma;        // pull: interior boxes may be loaded with one TMA copy (image tensor map valid)
};

// Fused forward + adjoint step over tiles: grid size for a launch, and the
// launch itself (one loss partial per CTA into a.partial[0 .. grid)).
int fused_tiled_grid(const LaunchArgs& a, const TileCfg& t);
cudaError_t launch_fused_tiled(const LaunchArgs& a, const TileCfg& t, cudaStream_t s, int grid);

// ---- batched uneven workload: one persistent launch over many volumes -------
// One entry per (image, deformation) pair.  Every tile of every item is pulled
// (f1 = pull(f0, phi), written) and the pulled values pushed back
// (out += push(f1, phi)) by the CTA that owns the tile.
struct BatchItem {
    LaunchArgs pull;     // phi, in = f0, out = f1
    LaunchArgs push;     // phi, in = f1, out = image-grid accumulator
    TileGrid t;          // 512-voxel tiles
    int tile_begin;      // first global tile index of this item
    int dp;              // isotropic degree + 1; 0: per-dimension degrees (per-voxel path)
};
TileGrid tile_grid(const LaunchArgs& a, const TileCfg& c);
// items in device memory; `counter` a zeroed device word for the work queue
cudaError_t launch_batch(const BatchItem* items, int nitems, int total_tiles, unsigned* counter, int cap,
                         cudaStream_t s);

// One warp, one CTA: a bounded wait on an mbarrier that never completes, with
// the given cycle limit (test of the timeout path; records the timeout bit).
cudaError_t launch_bounded_wait_probe(long long limit_cycles, cudaStream_t s);

// Read (and optionally clear) the device status word of the current device:
// bit 0 = a bounded device-side wait gave up.  0xffffffff if it cannot be read.
unsigned read_device_status(bool reset);

}  // namespace pp
