// pp_tiled_affine.cu -- affine push on the tiled push kernels: sample positions
// A * (i, j, k, 1) computed per voxel in place of a stored deformation, values
// streamed by the tile ring (kernels and helpers: pp_tiled_impl.cuh).
#include "pp_tiled_impl.cuh"

namespace pp {

cudaError_t launch_push_tiled_affine(const LaunchArgs& a, const TileCfg& t, const AffineMap& A, cudaStream_t s) {
    const bool small = a.g.n0 < (1LL << 31) - 1 && a.g.n1 < (1LL << 31) - 1;
    return small ? dispatch<kPush, int, true, true>(a, t, s, A) : dispatch<kPush, long long, true, true>(a, t, s, A);
}

unsigned status_push_affine(bool reset) { return unit_status(reset); }

}  // namespace pp
