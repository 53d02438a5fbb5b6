// pp_tiled_push.cu -- tiled push kernels
// (kernels and helpers: pp_tiled_impl.cuh).
#include "pp_tiled_impl.cuh"

namespace pp {

cudaError_t launch_tiled_push(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s) {
    (void)op;
    const bool small = a.g.n0 < (1LL << 31) - 1 && a.g.n1 < (1LL << 31) - 1;
    return small ? dispatch<kPush, int, true>(a, t, s) : dispatch<kPush, long long, true>(a, t, s);
}

unsigned status_push(bool reset) { return unit_status(reset); }

}  // namespace pp
