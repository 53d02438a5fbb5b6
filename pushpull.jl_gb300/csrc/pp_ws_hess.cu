// pp_ws_hess.cu -- warp-specialised pull_hess (pp_ws.cuh): the Hessian of
// every channel.
#include "pp_ws.cuh"

namespace pp {

cudaError_t launch_ws_hess(const LaunchArgs& a, const TileGrid& t, const CUtensorMap& phimap, cudaStream_t s) {
    return ws_dispatch_op<kPullHess>(a, t, phimap, s);
}

unsigned status_ws_hess(bool reset) { return unit_status(reset); }

}  // namespace pp
