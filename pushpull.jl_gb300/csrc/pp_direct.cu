// pp_direct.cu -- pull / pull_grad / pull_hess / push / push_grad, one thread per
// sample voxel against global memory.
//
// The general path: any degree triple (including anisotropic ones), any sample
// grid shape (the host-pointer ABI passes only n1), any deformation.  Weights are
// derived once per voxel and reused for every channel (the reference relaunches
// per channel and recomputes them, ext/pushpull_gpu.jl:37-49); boundary signs are
// folded into the weights so each tap is one load (or one reduction) and one FMA.
//
// Reference kernels replaced: pull_element, pullg_element, pullh_element,
// push_element, pushg_element (artifacts/C/pushpull.cu:33-163).
#include "pp_voxel.cuh"

namespace pp {
namespace {

template <int DP, int OP, typename IT>
__global__ void __launch_bounds__(256) k_pull_direct(LaunchArgs a) {
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const int b = blockIdx.y;
    const float* phi = a.phi + (long long)b * 3 * n1;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n1;
         v += (long long)gridDim.x * blockDim.x) {
        float x0, x1, x2;
        if (!load_valid(__ldg(phi + v), __ldg(phi + v + n1), __ldg(phi + v + 2 * n1), g, x0, x1, x2))
            pull_voxel_nan<OP>(a, b, v);
        else
            pull_voxel_global<DP, OP, IT>(a, b, v, x0, x1, x2);
    }
}

template <int DP, int OP, typename IT>
__global__ void __launch_bounds__(256) k_push_direct(LaunchArgs a) {
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const int b = blockIdx.y;
    const float* phi = a.phi + (long long)b * 3 * n1;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n1;
         v += (long long)gridDim.x * blockDim.x) {
        float x0, x1, x2;
        if (load_valid(__ldg(phi + v), __ldg(phi + v + n1), __ldg(phi + v + 2 * n1), g, x0, x1, x2))
            push_voxel_global<DP, OP, IT>(a, b, v, x0, x1, x2);
    }
}

template <int DP, int OP, typename IT, bool PUSH>
void launch_one(const LaunchArgs& a, dim3 grid, cudaStream_t s) {
    if constexpr (PUSH) k_push_direct<DP, OP, IT><<<grid, 256, 0, s>>>(a);
    else k_pull_direct<DP, OP, IT><<<grid, 256, 0, s>>>(a);
}

template <int OP, typename IT, bool PUSH>
cudaError_t dispatch_dp(const LaunchArgs& a, dim3 grid, cudaStream_t s) {
    const int d = a.g.dp[0];
    const bool iso = a.g.dp[1] == d && a.g.dp[2] == d;
    switch (iso ? d : 0) {
        case 1: launch_one<1, OP, IT, PUSH>(a, grid, s); break;
        case 2: launch_one<2, OP, IT, PUSH>(a, grid, s); break;
        case 3: launch_one<3, OP, IT, PUSH>(a, grid, s); break;
        case 4: launch_one<4, OP, IT, PUSH>(a, grid, s); break;
        case 5: launch_one<5, OP, IT, PUSH>(a, grid, s); break;
        default: launch_one<0, OP, IT, PUSH>(a, grid, s); break;
    }
    return cudaGetLastError();
}

dim3 direct_grid(const LaunchArgs& a) {
    const long long blocks_needed = (a.g.n1 + 255) / 256;
    const long long cap = (long long)sm_count() * 8;
    return dim3((unsigned)(blocks_needed < cap ? blocks_needed : cap), (unsigned)a.g.nb);
}

}  // namespace

cudaError_t launch_pull_direct(int op, const LaunchArgs& a, cudaStream_t s) {
    const dim3 grid = direct_grid(a);
    const bool small = a.g.n0 < (1LL << 31) - 1;
    switch (op) {
        case kPull: return small ? dispatch_dp<kPull, int, false>(a, grid, s)
                                 : dispatch_dp<kPull, long long, false>(a, grid, s);
        case kPullGrad: return small ? dispatch_dp<kPullGrad, int, false>(a, grid, s)
                                     : dispatch_dp<kPullGrad, long long, false>(a, grid, s);
        case kPullHess: return small ? dispatch_dp<kPullHess, int, false>(a, grid, s)
                                     : dispatch_dp<kPullHess, long long, false>(a, grid, s);
        case kPullGradDot: return small ? dispatch_dp<kPullGradDot, int, false>(a, grid, s)
                                        : dispatch_dp<kPullGradDot, long long, false>(a, grid, s);
        default: return small ? dispatch_dp<kPullHessDot, int, false>(a, grid, s)
                              : dispatch_dp<kPullHessDot, long long, false>(a, grid, s);
    }
}

cudaError_t launch_push_direct(int op, const LaunchArgs& a, cudaStream_t s) {
    const dim3 grid = direct_grid(a);
    const bool small = a.g.n0 < (1LL << 31) - 1;
    if (op == kPush)
        return small ? dispatch_dp<kPush, int, true>(a, grid, s) : dispatch_dp<kPush, long long, true>(a, grid, s);
    return small ? dispatch_dp<kPushGrad, int, true>(a, grid, s) : dispatch_dp<kPushGrad, long long, true>(a, grid, s);
}

}  // namespace pp
