// pp_ws_pull.cu -- warp-specialised pull family (pp_ws.cuh): pull, pull_grad and
// the affine pull here; pull_hess and the dot ops in their own translation units
// (pp_ws_hess.cu, pp_ws_grad_dot.cu, pp_ws_hess_dot.cu) so that they compile in
// parallel.
#include "pp_ws.cuh"

namespace pp {

cudaError_t launch_ws_hess(const LaunchArgs& a, const TileGrid& t, const CUtensorMap& phimap, cudaStream_t s);
cudaError_t launch_ws_grad_dot(const LaunchArgs& a, const TileGrid& t, const CUtensorMap& phimap, cudaStream_t s);
cudaError_t launch_ws_hess_dot(const LaunchArgs& a, const TileGrid& t, const CUtensorMap& phimap, cudaStream_t s);

bool ws_supported(const LaunchArgs& a) {
    const Geometry& g = a.g;
    if (!(g.dp[0] == g.dp[1] && g.dp[1] == g.dp[2])) return false;
    // most of a tile inside the sample grid (degenerate grids go per voxel)
    if (2 * g.d1[0] < 8 || 2 * g.d1[1] < 8 || 2 * g.d1[2] < kWsTz) return false;
    if (g.d1[0] > 0x7fffffffLL || g.d1[1] > 0x7fffffffLL || g.d1[2] > 0x7fffffffLL) return false;
    const long long ntx = (g.d1[0] + 7) >> 3, nty = (g.d1[1] + 7) >> 3, ntz = (g.d1[2] + kWsTz - 1) / kWsTz;
    return ntx * nty * ntz * g.nb < 0x7fffffffLL;
}

// Warp-specialised pull family; cudaErrorNotSupported when the deformation
// cannot be streamed by TMA (unaligned base or x extent), so the caller can
// fall back to the other kernels.
cudaError_t launch_ws_pull(int op, const LaunchArgs& a, cudaStream_t s) {
    const TileGrid t = ws_make_grid(a);
    CUtensorMap phimap;
    std::memset(&phimap, 0, sizeof phimap);
    if (!encode_ws_phi_map(&phimap, a.phi, a.g.d1, 3LL * a.g.nb)) return cudaErrorNotSupported;
    switch (op) {
        case kPull: return ws_dispatch_op<kPull>(a, t, phimap, s);
        case kPullGrad: return ws_dispatch_op<kPullGrad>(a, t, phimap, s);
        case kPullHess: return launch_ws_hess(a, t, phimap, s);
        case kPullGradDot: return launch_ws_grad_dot(a, t, phimap, s);
        case kPullHessDot: return launch_ws_hess_dot(a, t, phimap, s);
        default: return cudaErrorNotSupported;
    }
}

// Affine pull (pp_pull_affine) on the same kernels, positions computed in place.
cudaError_t launch_ws_pull_affine(const LaunchArgs& a, const AffineMap& A, cudaStream_t s) {
    const TileGrid t = ws_make_grid(a);
    CUtensorMap none;
    std::memset(&none, 0, sizeof none);
    const bool small = a.g.n0 < (1LL << 31) - 1 && a.g.n1 < (1LL << 31) - 1;
    return small ? ws_dispatch<kPull, int, true>(a, t, none, s, A) : ws_dispatch<kPull, long long, true>(a, t, none, s, A);
}

unsigned status_ws_pull(bool reset) { return unit_status(reset); }

}  // namespace pp
