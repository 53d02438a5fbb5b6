// pp_ws_grad_dot.cu -- warp-specialised pull_grad_dot (pp_ws.cuh): the gradient
// of every channel contracted with its upstream value, summed over channels.
#include "pp_ws.cuh"

namespace pp {

cudaError_t launch_ws_grad_dot(const LaunchArgs& a, const TileGrid& t, const CUtensorMap& phimap, cudaStream_t s) {
    return ws_dispatch_op<kPullGradDot>(a, t, phimap, s);
}

unsigned status_ws_grad_dot(bool reset) { return unit_status(reset); }

}  // namespace pp
