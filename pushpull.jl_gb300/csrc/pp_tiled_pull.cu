// pp_tiled_pull.cu -- tiled pull and pull_grad kernels
// (kernels and helpers: pp_tiled_impl.cuh).
#include "pp_tiled_impl.cuh"

namespace pp {

cudaError_t launch_tiled_pull_basic(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s) {
    const bool small = a.g.n0 < (1LL << 31) - 1 && a.g.n1 < (1LL << 31) - 1;
    if (op == kPull) return small ? dispatch<kPull, int, false>(a, t, s) : dispatch<kPull, long long, false>(a, t, s);
    return small ? dispatch<kPullGrad, int, false>(a, t, s) : dispatch<kPullGrad, long long, false>(a, t, s);
}

unsigned status_pull_basic(bool reset) { return unit_status(reset); }

}  // namespace pp
