// pp_fused.cu -- fused forward + adjoint step, per-voxel kernel, the loss
// reduction, and the host driver of both the tiled and per-voxel variants.
//
//   loss = sum_{b,c,v} (pull(f_c, phi)[v] - g_c[v])^2
//   df   = push(2 r, phi)                (the f cotangent of the pull rrule)
//   dphi = sum_c 2 r_c grad pull(f_c)    (the phi cotangent, src/pushpull_pb.jl:11-18)
//
// The reference evaluates this as pull, pull_grad, push and two broadcasts
// (config "differentiable step"); here one pass reads phi, f and g once.
#include "pp_tiled.cuh"
#include "pp_voxel.cuh"

namespace pp {
namespace {

template <int DP, typename IT>
__global__ void __launch_bounds__(256) k_fused_direct(const __grid_constant__ LaunchArgs a) {
    __shared__ double dred[8];
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const int b = blockIdx.y;
    const float* phi = a.phi + (long long)b * 3 * n1;
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);
    double loss = 0.0;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n1;
         v += (long long)gridDim.x * blockDim.x) {
        float x0, x1, x2;
        float* dp = a.out2 + (long long)b * 3 * n1 + v;
        if (!load_valid(__ldg(phi + v), __ldg(phi + v + n1), __ldg(phi + v + 2 * n1), g, x0, x1, x2)) {
            loss += (double)qnan();
            dp[0] = dp[n1] = dp[2 * n1] = qnan();
            continue;
        }
        Axis<DP, 1, IT> ax, ay, az;
        constexpr int N = Axis<DP, 1, IT>::N;
        float dphi[3] = {0.f, 0.f, 0.f};
        int prev = -1;
        for (int c = 0; c < g.nc; ++c) {
            int b0, b1, b2;
            const int code = bnd_code(a, c, b0, b1, b2);
            if (code != prev) {
                ax.setup(x0, g.dp[0], b0, g.d0[0], (IT)1);
                ay.setup(x1, g.dp[1], b1, g.d0[1], sy);
                az.setup(x2, g.dp[2], b2, g.d0[2], sz);
                prev = code;
            }
            const float* f0 = a.in + ((long long)b * g.nc + c) * g.n0;
            float r[6];
            contract<kPullValGrad, N>(ax, ay, az, ax.n, ay.n, az.n, DP == 0,
                                      [&](int k, int j, int i) { return __ldg(f0 + (az.off[k] + ay.off[j] + ax.off[i])); },
                                      r);
            const float res = r[3] - __ldg(a.up + ((long long)b * g.nc + c) * n1 + v);
            loss += (double)(res * res);
            const float d = 2.f * res;
            dphi[0] = fmaf(d, r[0], dphi[0]);
            dphi[1] = fmaf(d, r[1], dphi[1]);
            dphi[2] = fmaf(d, r[2], dphi[2]);
            if (!finitef(d)) continue;
            float* df = a.out + ((long long)b * g.nc + c) * g.n0;
#pragma unroll 1
            for (int k = 0; k < N; ++k) {
                if (DP == 0 && k >= az.n) break;
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    if (DP == 0 && j >= ay.n) break;
                    const float cb = d * (ay.w[j] * az.w[k]);
#pragma unroll
                    for (int i = 0; i < N; ++i) {
                        if (DP == 0 && i >= ax.n) break;
                        atomicAdd(df + (az.off[k] + ay.off[j] + ax.off[i]), cb * ax.w[i]);
                    }
                }
            }
        }
        dp[0] = dphi[0];
        dp[n1] = dphi[1];
        dp[2 * n1] = dphi[2];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
    if (lane == 0) dred[warp] = loss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < 8; ++w) s += dred[w];
        a.partial[blockIdx.x + (long long)gridDim.x * blockIdx.y] = s;
    }
}

// Deterministic sum of the per-CTA partials (fixed order, one block).
__global__ void __launch_bounds__(256) k_sum_partials(const double* p, int n, double* out) {
    __shared__ double red[256];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) s += p[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// max |f| per plane; non-negative floats order like their bit patterns, and a
// NaN (whose bits exceed +inf) propagates to the maximum.
__global__ void __launch_bounds__(256) k_absmax(const float* f, long long n, unsigned* out) {
    const float* p = f + (long long)blockIdx.y * n;
    unsigned m = 0;
    for (long long i = (long long)blockIdx.x * 256 + threadIdx.x; i < n; i += (long long)gridDim.x * 256)
        m = max(m, __float_as_uint(fabsf(__ldg(p + i))));
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0) atomicMax(out + blockIdx.y, m);
}

template <typename IT>
cudaError_t launch_direct_dp(const LaunchArgs& a, dim3 grid, cudaStream_t s) {
    const int d = a.g.dp[0];
    const bool iso = a.g.dp[1] == d && a.g.dp[2] == d;
    switch (iso ? d : 0) {
        case 1: k_fused_direct<1, IT><<<grid, 256, 0, s>>>(a); break;
        case 2: k_fused_direct<2, IT><<<grid, 256, 0, s>>>(a); break;
        case 3: k_fused_direct<3, IT><<<grid, 256, 0, s>>>(a); break;
        case 4: k_fused_direct<4, IT><<<grid, 256, 0, s>>>(a); break;
        case 5: k_fused_direct<5, IT><<<grid, 256, 0, s>>>(a); break;
        default: k_fused_direct<0, IT><<<grid, 256, 0, s>>>(a); break;
    }
    return cudaGetLastError();
}

}  // namespace

// Grid of the per-voxel fused kernel: (blocks, batches); partial slots = x * y.
dim3 fused_direct_grid(const LaunchArgs& a) {
    const long long blocks_needed = (a.g.n1 + 255) / 256;
    const long long cap = (long long)sm_count() * 8;
    return dim3((unsigned)(blocks_needed < cap ? blocks_needed : cap), (unsigned)a.g.nb);
}

cudaError_t launch_fused_direct(const LaunchArgs& a, cudaStream_t s) {
    const bool small = a.g.n0 < (1LL << 31) - 1;
    const dim3 grid = fused_direct_grid(a);
    return small ? launch_direct_dp<int>(a, grid, s) : launch_direct_dp<long long>(a, grid, s);
}

cudaError_t launch_absmax(const float* f, long long n, int planes, unsigned* out, cudaStream_t s) {
    if (planes > 65535) return cudaErrorInvalidConfiguration;
    const long long blocks = (n + 255) / 256;
    const long long cap = (long long)sm_count() * 4;
    k_absmax<<<dim3((unsigned)(blocks < cap ? blocks : cap), (unsigned)planes), 256, 0, s>>>(f, n, out);
    return cudaGetLastError();
}

cudaError_t launch_sum_partials(const double* partial, int n, double* out, cudaStream_t s) {
    k_sum_partials<<<1, 256, 0, s>>>(partial, n, out);
    return cudaGetLastError();
}

}  // namespace pp
