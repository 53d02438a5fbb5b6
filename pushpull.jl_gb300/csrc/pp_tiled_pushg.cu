// pp_tiled_pushg.cu -- tiled push_grad kernels
// (kernels and helpers: pp_tiled_impl.cuh).
#include "pp_tiled_impl.cuh"

namespace pp {

cudaError_t launch_tiled_push_grad(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s) {
    (void)op;
    const bool small = a.g.n0 < (1LL << 31) - 1 && a.g.n1 < (1LL << 31) - 1;
    return small ? dispatch<kPushGrad, int, true>(a, t, s) : dispatch<kPushGrad, long long, true>(a, t, s);
}

unsigned status_push_grad(bool reset) { return unit_status(reset); }

}  // namespace pp
