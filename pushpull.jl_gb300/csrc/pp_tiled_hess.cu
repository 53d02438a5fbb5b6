// pp_tiled_hess.cu -- tiled pull_hess kernels
// (kernels and helpers: pp_tiled_impl.cuh).
#include "pp_tiled_impl.cuh"

namespace pp {

cudaError_t launch_tiled_pull_hess(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s) {
    (void)op;
    const bool small = a.g.n0 < (1LL << 31) - 1 && a.g.n1 < (1LL << 31) - 1;
    return small ? dispatch<kPullHess, int, false>(a, t, s) : dispatch<kPullHess, long long, false>(a, t, s);
}

unsigned status_pull_hess(bool reset) { return unit_status(reset); }

}  // namespace pp
