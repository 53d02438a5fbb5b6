// pp_ws_pull.cu -- warp-specialised pull and pull_grad kernels (pp_ws.cuh).
#include "pp_ws.cuh"

namespace pp {

namespace {
template <int OP, typename IT, bool AFF = false>
cudaError_t ws_dispatch(const LaunchArgs& a, const TileGrid& t, const CUtensorMap& phimap, cudaStream_t s,
                        const AffineMap& aff = AffineMap{}) {
    switch (a.g.dp[0]) {
        case 1: return launch_ws_one<1, OP, IT, AFF>(a, t, phimap, aff, s);
        case 2: return launch_ws_one<2, OP, IT, AFF>(a, t, phimap, aff, s);
        case 3: return launch_ws_one<3, OP, IT, AFF>(a, t, phimap, aff, s);
        case 4: return launch_ws_one<4, OP, IT, AFF>(a, t, phimap, aff, s);
        default: return launch_ws_one<5, OP, IT, AFF>(a, t, phimap, aff, s);
    }
}
}  // namespace

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
    const bool small = a.g.n0 < (1LL << 31) - 1 && a.g.n1 < (1LL << 31) - 1;
    if (op == kPull) return small ? ws_dispatch<kPull, int>(a, t, phimap, s) : ws_dispatch<kPull, long long>(a, t, phimap, s);
    if (op == kPullGrad)
        return small ? ws_dispatch<kPullGrad, int>(a, t, phimap, s) : ws_dispatch<kPullGrad, long long>(a, t, phimap, s);
    return cudaErrorNotSupported;
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
