// pp_ws_hess_dot.cu -- warp-specialised pull_hess_dot (pp_ws.cuh): the Hessian
// of every channel contracted with its upstream gradient, summed over channels.
#include "pp_ws.cuh"

namespace pp {

cudaError_t launch_ws_hess_dot(const LaunchArgs& a, const TileGrid& t, const CUtensorMap& phimap, cudaStream_t s) {
    return ws_dispatch_op<kPullHessDot>(a, t, phimap, s);
}

unsigned status_ws_hess_dot(bool reset) { return unit_status(reset); }

}  // namespace pp
