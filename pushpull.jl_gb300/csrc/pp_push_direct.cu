// pp_push_direct.cu -- push and push_grad as a direct scatter with global float atomics.
//
// One thread per sample voxel, weights computed once for all channels; each
// tap is one RED.ADD.F32 into the caller's output (which the caller zeroes, or
// which this library zeroes when accumulate == 0).  push_grad merges the three
// directional scatters of the reference (pushg1, artifacts/C/pushpull_dev.cu:332-354)
// into one reduction per tap.  This is the general path; the tiled kernels
// privatise the reductions in shared memory where the footprint allows.
//
// Reference kernels replaced: push_element, pushg_element (artifacts/C/pushpull.cu:111-163).
#include "pp_kernels.cuh"

namespace pp {
namespace {

template <int DP, int OP, typename IT>
__global__ void __launch_bounds__(256) k_push_direct(LaunchArgs a) {
    constexpr int ORD = OP == kPushGrad ? 1 : 0;
    constexpr int NCOMP = OP == kPushGrad ? 3 : 1;
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const int b = blockIdx.y;
    const float* phi = a.phi + (long long)b * 3 * n1;
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);

    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n1;
         v += (long long)gridDim.x * blockDim.x) {
        float x0, x1, x2;
        if (!load_valid(__ldg(phi + v), __ldg(phi + v + n1), __ldg(phi + v + 2 * n1), g, x0, x1, x2))
            continue;
        const float* inb = a.in + (long long)b * g.nc * NCOMP * n1 + v;
        Axis<DP, ORD, IT> ax, ay, az;
        int prev = -1;
        for (int c = 0; c < g.nc; ++c) {
            const float* in = inb + (long long)c * NCOMP * n1;
            float v0 = __ldg(in), v1 = 0.f, v2 = 0.f;
            if constexpr (OP == kPushGrad) {
                v1 = __ldg(in + n1);
                v2 = __ldg(in + 2 * n1);
                if (!(finitef(v0) && finitef(v1) && finitef(v2))) continue;
            } else {
                if (!finitef(v0)) continue;
            }
            const int bi = g.nbnd == 1 ? 0 : c;
            const int code = a.bnd.code[bi][0] | (a.bnd.code[bi][1] << 2) | (a.bnd.code[bi][2] << 4);
            if (code != prev) {
                ax.setup(x0, g.dp[0], a.bnd.code[bi][0], g.d0[0], (IT)1);
                ay.setup(x1, g.dp[1], a.bnd.code[bi][1], g.d0[1], sy);
                az.setup(x2, g.dp[2], a.bnd.code[bi][2], g.d0[2], sz);
                prev = code;
            }
            float* f0 = a.out + ((long long)b * g.nc + c) * g.n0;
            constexpr int N = Axis<DP, ORD, IT>::N;
#pragma unroll
            for (int k = 0; k < N; ++k) {
                if (DP == 0 && k >= az.n) break;
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    if (DP == 0 && j >= ay.n) break;
                    float* row = f0 + (az.off[k] + ay.off[j]);
                    float ca, cb;   // tap value = ca * dw_x + cb * w_x
                    if constexpr (OP == kPushGrad) {
                        ca = v0 * (ay.w[j] * az.w[k]);
                        cb = v1 * (ay.dw[j] * az.w[k]) + v2 * (ay.w[j] * az.dw[k]);
                    } else {
                        ca = 0.f;
                        cb = v0 * (ay.w[j] * az.w[k]);
                    }
#pragma unroll
                    for (int i = 0; i < N; ++i) {
                        if (DP == 0 && i >= ax.n) break;
                        float t;
                        if constexpr (OP == kPushGrad) t = fmaf(ca, ax.dw[i], cb * ax.w[i]);
                        else t = cb * ax.w[i];
                        atomicAdd(row + ax.off[i], t);
                    }
                }
            }
        }
    }
}

template <int OP, typename IT>
cudaError_t dispatch_dp(const LaunchArgs& a, dim3 grid, cudaStream_t s) {
    const int d = a.g.dp[0];
    const bool iso = a.g.dp[1] == d && a.g.dp[2] == d;
    if (iso) {
        switch (d) {
            case 1: k_push_direct<1, OP, IT><<<grid, 256, 0, s>>>(a); return cudaGetLastError();
            case 2: k_push_direct<2, OP, IT><<<grid, 256, 0, s>>>(a); return cudaGetLastError();
            case 3: k_push_direct<3, OP, IT><<<grid, 256, 0, s>>>(a); return cudaGetLastError();
            case 4: k_push_direct<4, OP, IT><<<grid, 256, 0, s>>>(a); return cudaGetLastError();
            case 5: k_push_direct<5, OP, IT><<<grid, 256, 0, s>>>(a); return cudaGetLastError();
            default: break;
        }
    }
    k_push_direct<0, OP, IT><<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_push_direct(int op, const LaunchArgs& a, cudaStream_t s) {
    const long long blocks_needed = (a.g.n1 + 255) / 256;
    const long long cap = (long long)sm_count() * 8;
    dim3 grid((unsigned)(blocks_needed < cap ? blocks_needed : cap), (unsigned)a.g.nb);
    const bool small = a.g.n0 < (1LL << 31) - 1;
    if (op == kPush)
        return small ? dispatch_dp<kPush, int>(a, grid, s) : dispatch_dp<kPush, long long>(a, grid, s);
    return small ? dispatch_dp<kPushGrad, int>(a, grid, s) : dispatch_dp<kPushGrad, long long>(a, grid, s);
}

}  // namespace pp
