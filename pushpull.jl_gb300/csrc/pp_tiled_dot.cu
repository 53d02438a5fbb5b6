// pp_tiled_dot.cu -- tiled pull_grad / pull_hess contractions with an upstream (rrule kernels)
// (kernels and helpers: pp_tiled_impl.cuh).
#include "pp_tiled_impl.cuh"

namespace pp {

cudaError_t launch_tiled_pull_dot(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s) {
    const bool small = a.g.n0 < (1LL << 31) - 1 && a.g.n1 < (1LL << 31) - 1;
    if (op == kPullGradDot)
        return small ? dispatch<kPullGradDot, int, false>(a, t, s) : dispatch<kPullGradDot, long long, false>(a, t, s);
    return small ? dispatch<kPullHessDot, int, false>(a, t, s) : dispatch<kPullHessDot, long long, false>(a, t, s);
}

unsigned status_pull_dot(bool reset) { return unit_status(reset); }

}  // namespace pp
