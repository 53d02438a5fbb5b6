// pp_pull_direct.cu -- pull, pull_grad and pull_hess as a direct gather.
//
// One thread per sample voxel; the thread reads its deformation once, derives
// the B-spline weights once, and then evaluates every channel (the reference
// relaunches per channel and recomputes weights each time, ext/pushpull_gpu.jl:37-49).
// Boundary signs are folded into the weights, so each tap is one load and one FMA.
// Separable accumulation: a row of x taps, then y, then z.
//
// Reference kernels replaced: pull_element, pullg_element, pullh_element
// (artifacts/C/pushpull.cu:33-108), per-voxel math pull1 / pullg1 / pullh1
// (artifacts/C/pushpull_dev.cu:236-291).
#include "pp_kernels.cuh"

namespace pp {
namespace {

__device__ __forceinline__ float nanf_() { return __int_as_float(0x7fffffff); }

template <int DP, int OP, typename IT>
__global__ void __launch_bounds__(256) k_pull_direct(LaunchArgs a) {
    constexpr int ORD = OP;   // pull needs values, pull_grad first, pull_hess second derivatives
    constexpr int NCOMP = OP == kPull ? 1 : (OP == kPullGrad ? 3 : 9);
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const int b = blockIdx.y;
    const float* phi = a.phi + (long long)b * 3 * n1;
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);

    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n1;
         v += (long long)gridDim.x * blockDim.x) {
        float x0, x1, x2;
        const bool ok = load_valid(__ldg(phi + v), __ldg(phi + v + n1), __ldg(phi + v + 2 * n1), g,
                                   x0, x1, x2);
        float* outb = a.out + (long long)b * g.nc * NCOMP * n1 + v;
        if (!ok) {
            for (int c = 0; c < g.nc; ++c)
#pragma unroll
                for (int q = 0; q < NCOMP; ++q) outb[((long long)c * NCOMP + q) * n1] = nanf_();
            continue;
        }
        Axis<DP, ORD, IT> ax, ay, az;
        int prev = -1;
        for (int c = 0; c < g.nc; ++c) {
            const int bi = g.nbnd == 1 ? 0 : c;
            const int code = a.bnd.code[bi][0] | (a.bnd.code[bi][1] << 2) | (a.bnd.code[bi][2] << 4);
            if (code != prev) {
                ax.setup(x0, g.dp[0], a.bnd.code[bi][0], g.d0[0], (IT)1);
                ay.setup(x1, g.dp[1], a.bnd.code[bi][1], g.d0[1], sy);
                az.setup(x2, g.dp[2], a.bnd.code[bi][2], g.d0[2], sz);
                prev = code;
            }
            const float* f0 = a.in + ((long long)b * g.nc + c) * g.n0;
            constexpr int N = Axis<DP, ORD, IT>::N;
            // accumulators: see the per-OP comments below
            float r0k = 0.f, r1k = 0.f, r2k = 0.f, r3k = 0.f, r4k = 0.f, r5k = 0.f;
#pragma unroll
            for (int k = 0; k < N; ++k) {
                if (DP == 0 && k >= az.n) break;
                float j0 = 0.f, j1 = 0.f, j2 = 0.f, j3 = 0.f, j4 = 0.f, j5 = 0.f;
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    if (DP == 0 && j >= ay.n) break;
                    const float* row = f0 + (az.off[k] + ay.off[j]);
                    float i0 = 0.f, i1 = 0.f, i2 = 0.f;
#pragma unroll
                    for (int i = 0; i < N; ++i) {
                        if (DP == 0 && i >= ax.n) break;
                        const float f = __ldg(row + ax.off[i]);
                        i0 = fmaf(ax.w[i], f, i0);
                        if constexpr (ORD >= 1) i1 = fmaf(ax.dw[i], f, i1);
                        if constexpr (ORD >= 2) i2 = fmaf(ax.hw[i], f, i2);
                    }
                    if constexpr (OP == kPull) {
                        j0 = fmaf(ay.w[j], i0, j0);
                    } else if constexpr (OP == kPullGrad) {
                        j0 = fmaf(ay.w[j], i1, j0);    // -> d/dx
                        j1 = fmaf(ay.dw[j], i0, j1);   // -> d/dy
                        j2 = fmaf(ay.w[j], i0, j2);    // -> d/dz (z weight applied below)
                    } else {
                        j0 = fmaf(ay.w[j], i2, j0);    // xx
                        j1 = fmaf(ay.hw[j], i0, j1);   // yy
                        j2 = fmaf(ay.w[j], i0, j2);    // zz (needs hw_z)
                        j3 = fmaf(ay.dw[j], i1, j3);   // xy
                        j4 = fmaf(ay.w[j], i1, j4);    // xz (needs dw_z)
                        j5 = fmaf(ay.dw[j], i0, j5);   // yz (needs dw_z)
                    }
                }
                if constexpr (OP == kPull) {
                    r0k = fmaf(az.w[k], j0, r0k);
                } else if constexpr (OP == kPullGrad) {
                    r0k = fmaf(az.w[k], j0, r0k);
                    r1k = fmaf(az.w[k], j1, r1k);
                    r2k = fmaf(az.dw[k], j2, r2k);
                } else {
                    r0k = fmaf(az.w[k], j0, r0k);
                    r1k = fmaf(az.w[k], j1, r1k);
                    r2k = fmaf(az.hw[k], j2, r2k);
                    r3k = fmaf(az.w[k], j3, r3k);
                    r4k = fmaf(az.dw[k], j4, r4k);
                    r5k = fmaf(az.dw[k], j5, r5k);
                }
            }
            float* o = outb + (long long)c * NCOMP * n1;
            if constexpr (OP == kPull) {
                o[0] = r0k;
            } else if constexpr (OP == kPullGrad) {
                o[0] = r0k;
                o[n1] = r1k;
                o[2 * n1] = r2k;
            } else {
                // column-major 3x3, entry (p,q) at component p + 3q (artifacts/C/pushpull.c:129-134)
                o[0] = r0k;
                o[4 * n1] = r1k;
                o[8 * n1] = r2k;
                o[1 * n1] = r3k;
                o[3 * n1] = r3k;
                o[2 * n1] = r4k;
                o[6 * n1] = r4k;
                o[5 * n1] = r5k;
                o[7 * n1] = r5k;
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
            case 1: k_pull_direct<1, OP, IT><<<grid, 256, 0, s>>>(a); return cudaGetLastError();
            case 2: k_pull_direct<2, OP, IT><<<grid, 256, 0, s>>>(a); return cudaGetLastError();
            case 3: k_pull_direct<3, OP, IT><<<grid, 256, 0, s>>>(a); return cudaGetLastError();
            case 4: k_pull_direct<4, OP, IT><<<grid, 256, 0, s>>>(a); return cudaGetLastError();
            case 5: k_pull_direct<5, OP, IT><<<grid, 256, 0, s>>>(a); return cudaGetLastError();
            default: break;
        }
    }
    k_pull_direct<0, OP, IT><<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_pull_direct(int op, const LaunchArgs& a, cudaStream_t s) {
    const long long blocks_needed = (a.g.n1 + 255) / 256;
    const long long cap = (long long)sm_count() * 8;
    dim3 grid((unsigned)(blocks_needed < cap ? blocks_needed : cap), (unsigned)a.g.nb);
    const bool small = a.g.n0 < (1LL << 31) - 1;
    switch (op) {
        case kPull: return small ? dispatch_dp<kPull, int>(a, grid, s) : dispatch_dp<kPull, long long>(a, grid, s);
        case kPullGrad:
            return small ? dispatch_dp<kPullGrad, int>(a, grid, s) : dispatch_dp<kPullGrad, long long>(a, grid, s);
        default:
            return small ? dispatch_dp<kPullHess, int>(a, grid, s) : dispatch_dp<kPullHess, long long>(a, grid, s);
    }
}

}  // namespace pp
