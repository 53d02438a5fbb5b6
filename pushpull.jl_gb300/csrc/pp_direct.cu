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

// Channel c of the pull family for one valid voxel into registers: the same
// arithmetic as pull_voxel_global for that channel.
template <int DP, int OP, typename IT>
__device__ __forceinline__ void pull_voxel_regs(const LaunchArgs& a, int b, int c, float x0, float x1, float x2,
                                                float (&r)[6]) {
    const Geometry& g = a.g;
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);
    Axis<DP, op_order(OP), IT> ax, ay, az;
    constexpr int N = Axis<DP, op_order(OP), IT>::N;
    int b0, b1, b2;
    bnd_code(a, c, b0, b1, b2);
    ax.setup(x0, g.dp[0], b0, g.d0[0], (IT)1);
    ay.setup(x1, g.dp[1], b1, g.d0[1], sy);
    az.setup(x2, g.dp[2], b2, g.d0[2], sz);
    const float* f0 = a.in + ((long long)b * g.nc + c) * g.n0;
    contract<OP, N>(ax, ay, az, ax.n, ay.n, az.n, DP == 0,
                    [&](int k, int j, int i) { return __ldg(f0 + (az.off[k] + ay.off[j] + ax.off[i])); }, r);
}

// One axis of a voxel whose taps all lie inside the image: weights only.
template <int DP, int ORD>
struct InAxis {
    float w[DP];
    float dw[ORD >= 1 ? DP : 1];
    float hw[ORD >= 2 ? DP : 1];
};

// Channel c of pull / pull_grad for a voxel whose taps all lie inside the image (no folding, 32-bit offsets): false, with
// nothing computed, otherwise.  The weights and the contraction are
// pull_voxel_global's, so the bits are the same.
template <int DP, int OP>
__device__ __forceinline__ bool pull_voxel_inside(const float* f0, const Geometry& g, int sy, int sz, float x0,
                                                  float x1, float x2, float (&r)[6]) {
    constexpr int ORD = op_order(OP);
    InAxis<DP, ORD> ax, ay, az;
    const int ox = spline_taps32<DP, ORD>(x0, ax.w, ax.dw, ax.hw);
    const int oy = spline_taps32<DP, ORD>(x1, ay.w, ay.dw, ay.hw);
    const int oz = spline_taps32<DP, ORD>(x2, az.w, az.dw, az.hw);
    if (ox < 0 || oy < 0 || oz < 0 || ox > (int)g.d0[0] - DP || oy > (int)g.d0[1] - DP || oz > (int)g.d0[2] - DP)
        return false;
    const float* p = f0 + (oz * sz + oy * sy + ox);
    contract<OP, DP>(ax, ay, az, DP, DP, DP, false, [&](int k, int j, int i) { return __ldg(p + (k * sz + j * sy + i)); },
                     r);
    return true;
}

struct Res6 {
    float v[6];
};

// Any other voxel: the general per-voxel path, out of line so that its 64-bit
// folding does not weigh on the registers of the common path.
template <int DP, int OP>
__device__ __noinline__ Res6 pull_voxel_folded(const LaunchArgs& a, int b, int c, float x0, float x1, float x2) {
    Res6 o;
    pull_voxel_regs<DP, OP, int>(a, b, c, x0, x1, x2, o.v);
    return o;
}

// pull and pull_grad at one tap per axis (degree 0, nearest neighbour): four
// consecutive sample voxels per thread and iteration.  The deformation arrives
// by 16-byte loads, the next group's while this group gathers, so each thread
// keeps 48 bytes of DRAM reads in flight (one voxel per thread leaves the
// kernel latency-bound far below HBM bandwidth: 192^3, GB300, 0.080 -> 0.048
// ms).  Channel by channel, the four voxels' results stay in registers up to
// 16-byte stores, so their gathers overlap.  Voxels whose tap is inside the
// image take a lean path; the rest the general one.  Same arithmetic as
// k_pull_direct.  Needs n1 % 4 == 0, 16-byte aligned phi and output, and an
// image of fewer than 2^31 elements.  (At two taps per axis the same scheme
// measured slower than the warp-specialised kernels.)
template <int OP>
__global__ void __launch_bounds__(256, 4) k_pull_nearest(LaunchArgs a) {
    constexpr int DP = 1;
    constexpr int NCOMP = OP == kPull ? 1 : 3;
    const Geometry& g = a.g;
    const long long n1 = g.n1, n4 = n1 >> 2;
    const int b = blockIdx.y;
    const int sy = (int)g.d0[0], sz = (int)(g.d0[0] * g.d0[1]);
    const float* phi = a.phi + (long long)b * 3 * n1;
    const float4* p0 = reinterpret_cast<const float4*>(phi);
    const float4* p1 = reinterpret_cast<const float4*>(phi + n1);
    const float4* p2 = reinterpret_cast<const float4*>(phi + 2 * n1);
    const long long step = (long long)gridDim.x * blockDim.x;
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float4 c0 = make_float4(0.f, 0.f, 0.f, 0.f), c1 = c0, c2 = c0;
    if (q < n4) {
        c0 = __ldg(p0 + q);
        c1 = __ldg(p1 + q);
        c2 = __ldg(p2 + q);
    }
    for (; q < n4; q += step) {
        const float X[4] = {c0.x, c0.y, c0.z, c0.w};
        const float Y[4] = {c1.x, c1.y, c1.z, c1.w};
        const float Z[4] = {c2.x, c2.y, c2.z, c2.w};
        if (q + step < n4) {
            c0 = __ldg(p0 + q + step);
            c1 = __ldg(p1 + q + step);
            c2 = __ldg(p2 + q + step);
        }
        const long long v0 = 4 * q;
#pragma unroll 1
        for (int c = 0; c < g.nc; ++c) {
            const float* f0 = a.in + ((long long)b * g.nc + c) * g.n0;
            float r[4][6];
            bool ok[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                float x0, x1, x2;
                ok[u] = load_valid(X[u], Y[u], Z[u], g, x0, x1, x2);
                if (ok[u] && !pull_voxel_inside<DP, OP>(f0, g, sy, sz, x0, x1, x2, r[u])) {
                    const Res6 o = pull_voxel_folded<DP, OP>(a, b, c, x0, x1, x2);
#pragma unroll
                    for (int p = 0; p < 6; ++p) r[u][p] = o.v[p];
                }
            }
            float* o = pull_out<OP>(a, b, c, v0);
#pragma unroll
            for (int p = 0; p < NCOMP; ++p)
                *reinterpret_cast<float4*>(o + p * n1) =
                    make_float4(ok[0] ? r[0][p] : qnan(), ok[1] ? r[1][p] : qnan(), ok[2] ? r[2][p] : qnan(),
                                ok[3] ? r[3][p] : qnan());
        }
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

// k_pull_nearest for pull and pull_grad at degree 0 when the sample count is a
// multiple of 4, phi and the output are 16-byte aligned and the image has fewer
// than 2^31 elements.
cudaError_t launch_pull_nearest(int op, const LaunchArgs& a, cudaStream_t s) {
    const Geometry& g = a.g;
    if ((op != kPull && op != kPullGrad) || g.dp[0] != 1 || g.dp[1] != 1 || g.dp[2] != 1) return cudaErrorNotSupported;
    if ((g.n1 & 3) || (reinterpret_cast<uintptr_t>(a.phi) & 15) || (reinterpret_cast<uintptr_t>(a.out) & 15) ||
        g.n0 >= (1LL << 31) - 1)
        return cudaErrorNotSupported;
    const long long blocks_needed = ((g.n1 >> 2) + 255) / 256;
    const long long cap = (long long)sm_count() * 4;
    const dim3 grid((unsigned)(blocks_needed < cap ? blocks_needed : cap), (unsigned)g.nb);
    if (op == kPull) k_pull_nearest<kPull><<<grid, 256, 0, s>>>(a);
    else k_pull_nearest<kPullGrad><<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_pull_direct(int op, const LaunchArgs& a, cudaStream_t s) {
    const cudaError_t en = launch_pull_nearest(op, a, s);
    if (en != cudaErrorNotSupported) return en;
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
