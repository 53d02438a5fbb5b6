// pp_tiled_fused.cu -- tiled fused forward + adjoint step kernels
// (kernels and helpers: pp_tiled_impl.cuh).
#include "pp_tiled_impl.cuh"

namespace pp {

cudaError_t launch_fused_tiled(const LaunchArgs& a, const TileCfg& t, cudaStream_t s, int grid) {
    const bool small = a.g.n0 < (1LL << 31) - 1 && a.g.n1 < (1LL << 31) - 1;
    switch (a.g.dp[0]) {
        case 1: return small ? launch_fused_dp<1, int>(a, t, s, grid) : launch_fused_dp<1, long long>(a, t, s, grid);
        case 2: return small ? launch_fused_dp<2, int>(a, t, s, grid) : launch_fused_dp<2, long long>(a, t, s, grid);
        case 3: return small ? launch_fused_dp<3, int>(a, t, s, grid) : launch_fused_dp<3, long long>(a, t, s, grid);
        case 4: return small ? launch_fused_dp<4, int>(a, t, s, grid) : launch_fused_dp<4, long long>(a, t, s, grid);
        default: return small ? launch_fused_dp<5, int>(a, t, s, grid) : launch_fused_dp<5, long long>(a, t, s, grid);
    }
}

unsigned status_fused(bool reset) { return unit_status(reset); }

}  // namespace pp
