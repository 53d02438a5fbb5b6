// pp_voxel.cuh -- one sample voxel, all channels, against global memory.
//
// Used by the direct kernels and as the per-tile fallback of the tiled kernels
// (a tile whose image footprint does not fit its shared-memory box).
#pragma once

#include "pp_kernels.cuh"

namespace pp {

__device__ __forceinline__ float qnan() { return __int_as_float(0x7fffffff); }

__device__ __forceinline__ int bnd_code(const LaunchArgs& a, int c, int& b0, int& b1, int& b2) {
    const int bi = a.g.nbnd == 1 ? 0 : c;
    b0 = a.bnd.code[bi][0];
    b1 = a.bnd.code[bi][1];
    b2 = a.bnd.code[bi][2];
    return b0 | (b1 << 2) | (b2 << 4);
}

// output components per channel (dot ops: 3 for the whole voxel, see pull_out)
template <int OP>
__device__ __forceinline__ constexpr int pull_ncomp() {
    return OP == kPull ? 1 : (OP == kPullHess ? 9 : 3);
}
template <int OP>
__device__ __forceinline__ constexpr bool pull_is_dot() {
    return OP == kPullGradDot || OP == kPullHessDot;
}
// the contraction a pull-family op evaluates per channel
template <int OP>
__device__ __forceinline__ constexpr int pull_base_op() {
    return OP == kPullGradDot ? kPullGrad : (OP == kPullHessDot ? kPullHess : OP);
}
// first output element of (batch b, channel c) for voxel v
template <int OP>
__device__ __forceinline__ float* pull_out(const LaunchArgs& a, int b, int c, long long v) {
    constexpr int NCOMP = pull_ncomp<OP>();
    if constexpr (pull_is_dot<OP>()) return a.out + (long long)b * 3 * a.g.n1 + v;
    return a.out + ((long long)b * a.g.nc + c) * NCOMP * a.g.n1 + v;
}

// Write every output component of voxel v as NaN (invalid sample).
template <int OP>
__device__ __forceinline__ void pull_voxel_nan(const LaunchArgs& a, int b, long long v) {
    constexpr int NCOMP = pull_ncomp<OP>();
    const long long n1 = a.g.n1;
    const int nch = pull_is_dot<OP>() ? 1 : a.g.nc;
    for (int c = 0; c < nch; ++c) {
        float* o = pull_out<OP>(a, b, c, v);
#pragma unroll
        for (int q = 0; q < NCOMP; ++q) o[(long long)q * n1] = qnan();
    }
}

// Accumulate one channel's gradient (r[0..2]) or Hessian (r[0..5] = xx, yy, zz,
// xy, xz, yz) contracted with the upstream of (b, c, v) into acc[0..2].
template <int OP>
__device__ __forceinline__ void dot_accumulate(const LaunchArgs& a, int b, int c, long long v, const float (&r)[6],
                                               float (&acc)[3]) {
    const long long n1 = a.g.n1;
    if constexpr (OP == kPullGradDot) {
        const float u = __ldg(a.up + ((long long)b * a.g.nc + c) * n1 + v);
        acc[0] = fmaf(u, r[0], acc[0]);
        acc[1] = fmaf(u, r[1], acc[1]);
        acc[2] = fmaf(u, r[2], acc[2]);
    } else if constexpr (OP == kPullHessDot) {
        const float* up = a.up + ((long long)b * a.g.nc + c) * 3 * n1 + v;
        const float u0 = __ldg(up), u1 = __ldg(up + n1), u2 = __ldg(up + 2 * n1);
        acc[0] += r[0] * u0 + r[3] * u1 + r[4] * u2;
        acc[1] += r[3] * u0 + r[1] * u1 + r[5] * u2;
        acc[2] += r[4] * u0 + r[5] * u1 + r[2] * u2;
    }
}

// Store the per-op results of one channel (pull 1, grad 3, Hessian 9 planar comps).
template <int OP>
__device__ __forceinline__ void pull_store(float* o, long long n1, const float (&r)[6]) {
    if constexpr (OP == kPull) {
        o[0] = r[0];
    } else if constexpr (OP == kPullGrad) {
        o[0] = r[0];
        o[n1] = r[1];
        o[2 * n1] = r[2];
    } else {
        // column-major 3x3, entry (p,q) at component p + 3q (artifacts/C/pushpull.c:88-93)
        o[0] = r[0];
        o[4 * n1] = r[1];
        o[8 * n1] = r[2];
        o[1 * n1] = r[3];
        o[3 * n1] = r[3];
        o[2 * n1] = r[4];
        o[6 * n1] = r[4];
        o[5 * n1] = r[5];
        o[7 * n1] = r[5];
    }
}

// Separable patch contraction.  `tap(k, j, i)` returns the (signed) image value of
// tap (i, j, k); weights come from the three axes.  Results in r[] as pull_store
// expects; kPullValGrad returns the gradient in r[0..2] and the value in r[3].
template <int OP, int N, class AX, class AY, class AZ, class TAP>
__device__ __forceinline__ void contract(const AX& ax, const AY& ay, const AZ& az, int nx, int ny, int nz,
                                         bool runtime_n, TAP tap, float (&r)[6]) {
#pragma unroll
    for (int q = 0; q < 6; ++q) r[q] = 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (runtime_n && k >= nz) break;
        float j0 = 0.f, j1 = 0.f, j2 = 0.f, j3 = 0.f, j4 = 0.f, j5 = 0.f;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            if (runtime_n && j >= ny) break;
            float i0 = 0.f, i1 = 0.f, i2 = 0.f;
#pragma unroll
            for (int i = 0; i < N; ++i) {
                if (runtime_n && i >= nx) break;
                const float f = tap(k, j, i);
                i0 = fmaf(ax.w[i], f, i0);
                if constexpr (op_order(OP) >= 1) i1 = fmaf(ax.dw[i], f, i1);
                if constexpr (op_order(OP) >= 2) i2 = fmaf(ax.hw[i], f, i2);
            }
            if constexpr (OP == kPull) {
                j0 = fmaf(ay.w[j], i0, j0);
            } else if constexpr (OP == kPullGrad || OP == kPullValGrad) {
                j0 = fmaf(ay.w[j], i1, j0);    // d/dx
                j1 = fmaf(ay.dw[j], i0, j1);   // d/dy
                j2 = fmaf(ay.w[j], i0, j2);    // d/dz once the z derivative weight is applied
            } else {
                j0 = fmaf(ay.w[j], i2, j0);    // xx
                j1 = fmaf(ay.hw[j], i0, j1);   // yy
                j2 = fmaf(ay.w[j], i0, j2);    // zz
                j3 = fmaf(ay.dw[j], i1, j3);   // xy
                j4 = fmaf(ay.w[j], i1, j4);    // xz
                j5 = fmaf(ay.dw[j], i0, j5);   // yz
            }
        }
        if constexpr (OP == kPull) {
            r[0] = fmaf(az.w[k], j0, r[0]);
        } else if constexpr (OP == kPullGrad || OP == kPullValGrad) {
            r[0] = fmaf(az.w[k], j0, r[0]);
            r[1] = fmaf(az.w[k], j1, r[1]);
            r[2] = fmaf(az.dw[k], j2, r[2]);
            if constexpr (OP == kPullValGrad) r[3] = fmaf(az.w[k], j2, r[3]);   // the value itself
        } else {
            r[0] = fmaf(az.w[k], j0, r[0]);
            r[1] = fmaf(az.w[k], j1, r[1]);
            r[2] = fmaf(az.hw[k], j2, r[2]);
            r[3] = fmaf(az.w[k], j3, r[3]);
            r[4] = fmaf(az.dw[k], j4, r[4]);
            r[5] = fmaf(az.dw[k], j5, r[5]);
        }
    }
}

// pull family for one valid voxel, every channel, gathering from global memory.
template <int DP, int OP_, typename IT>
__device__ __forceinline__ void pull_voxel_global(const LaunchArgs& a, int b, long long v, float x0, float x1,
                                                  float x2) {
    constexpr int OP = pull_base_op<OP_>();
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);
    float acc[3] = {0.f, 0.f, 0.f};
    Axis<DP, op_order(OP), IT> ax, ay, az;
    constexpr int N = Axis<DP, op_order(OP), IT>::N;
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
        contract<OP, N>(ax, ay, az, ax.n, ay.n, az.n, DP == 0,
                        [&](int k, int j, int i) { return __ldg(f0 + (az.off[k] + ay.off[j] + ax.off[i])); }, r);
        if constexpr (pull_is_dot<OP_>()) dot_accumulate<OP_>(a, b, c, v, r, acc);
        else pull_store<OP>(pull_out<OP_>(a, b, c, v), n1, r);
    }
    if constexpr (pull_is_dot<OP_>()) {
        float* o = pull_out<OP_>(a, b, 0, v);
        o[0] = acc[0];
        o[n1] = acc[1];
        o[2 * n1] = acc[2];
    }
}

// push family for one valid voxel, every channel, scattering with global float atomics.
template <int DP, int OP, typename IT>
__device__ __forceinline__ void push_voxel_global(const LaunchArgs& a, int b, long long v, float x0, float x1,
                                                  float x2) {
    constexpr int ORD = OP == kPushGrad ? 1 : 0;
    constexpr int NCOMP = OP == kPushGrad ? 3 : 1;
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);
    const float* inb = a.in + (long long)b * g.nc * NCOMP * n1 + v;
    Axis<DP, ORD, IT> ax, ay, az;
    constexpr int N = Axis<DP, ORD, IT>::N;
    int prev = -1;
    for (int c = 0; c < g.nc; ++c) {
        const float* in = inb + (long long)c * NCOMP * n1;
        const float v0 = __ldg(in);
        float v1 = 0.f, v2 = 0.f;
        if constexpr (OP == kPushGrad) {
            v1 = __ldg(in + n1);
            v2 = __ldg(in + 2 * n1);
            if (!(finitef(v0) && finitef(v1) && finitef(v2))) continue;
        } else {
            if (!finitef(v0)) continue;
        }
        int b0, b1, b2;
        const int code = bnd_code(a, c, b0, b1, b2);
        if (code != prev) {
            ax.setup(x0, g.dp[0], b0, g.d0[0], (IT)1);
            ay.setup(x1, g.dp[1], b1, g.d0[1], sy);
            az.setup(x2, g.dp[2], b2, g.d0[2], sz);
            prev = code;
        }
        float* f0 = a.out + ((long long)b * g.nc + c) * g.n0;
        // push with a count image (pushc): the weights alone go to out2 as well
        float* c0 = OP == kPush && a.out2 ? a.out2 + ((long long)b * g.nc + c) * g.n0 : nullptr;
#pragma unroll
        for (int k = 0; k < N; ++k) {
            if (DP == 0 && k >= az.n) break;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                if (DP == 0 && j >= ay.n) break;
                float* row = f0 + (az.off[k] + ay.off[j]);
                if constexpr (OP == kPush) {
                    if (c0) {
                        const float wyz = ay.w[j] * az.w[k];
                        float* crow = c0 + (az.off[k] + ay.off[j]);
#pragma unroll
                        for (int i = 0; i < N; ++i) {
                            if (DP == 0 && i >= ax.n) break;
                            atomicAdd(crow + ax.off[i], wyz * ax.w[i]);
                        }
                    }
                }
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

}  // namespace pp
