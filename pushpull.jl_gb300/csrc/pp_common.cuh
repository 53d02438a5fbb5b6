// pp_common.cuh -- device-side arithmetic shared by every pull / push kernel.
//
// Semantics follow PushPull.jl's reference (paths within that project):
//   x      = phi - 1.0f in float32                        artifacts/C/pushpull.c:24-26
//   valid  = x finite and, when ext == 0,
//            -0.01f <= x <= (float)d - 0.99f               artifacts/C/pushpull.c:6-9
//   tap 0  = (int64) ceilf(x - 0.5f * dp)                 artifacts/C/bspline.cu:66
//   fold   = circulant / DCT-II mirror / DST-II mirror     artifacts/C/patch.cu:5-59
//   weights: centred B-spline of degree dp-1 and its first and second derivatives,
//            with the reference's degree-0/1 conventions     artifacts/C/bspline.cu:63-244
// The float operations that decide which voxels are valid and which taps are
// read are issued with explicit round-to-nearest intrinsics so the compiler
// cannot contract them; the weight polynomials are free to use FMA.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pp {

constexpr int kMaxDP = 5;        // degree 4 + 1
constexpr int kMaxBnd = 64;      // per-channel boundary codes carried in the launch

// Boundary codes per channel, 3 per channel, packed into the launch parameters.
struct BndTable {
    unsigned char code[kMaxBnd][3];
};

// Geometry and settings of one launch (all channels and batches of one op).
struct Geometry {
    long long d0[3];     // image (source) dimensions
    long long d1[3];     // sample-grid (deformation) dimensions
    long long n0, n1;    // voxel counts
    int nc, nb;          // channels, batch
    int dp[3];           // degree + 1 per dimension
    int ext;             // extrapolate flag
    int nbnd;            // 1 or nc
    float hi[3];         // (float)d0[k] - 0.99f: upper end of the ext == 0 band (float arithmetic)
};

__device__ __forceinline__ bool finitef(float v) { return fabsf(v) <= 3.402823466e38f; }

// Explicit shared-memory accesses through 32-bit shared-window addresses, so
// box reads and reductions are always issued as shared-space instructions.
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ float lds_f32(unsigned a) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}
__device__ __forceinline__ void red_shared_s32(unsigned a, int v) {
    asm volatile("red.shared.add.s32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void red_shared_f32(unsigned a, float v) {
    asm volatile("red.shared.add.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}

// The validity test (VOXOK) of a 0-based position.
__device__ __forceinline__ bool position_valid(float x0, float x1, float x2, const Geometry& g) {
    if (!(finitef(x0) && finitef(x1) && finitef(x2))) return false;
    if (g.ext) return true;
    return x0 >= -0.01f && x0 <= g.hi[0] && x1 >= -0.01f && x1 <= g.hi[1] && x2 >= -0.01f && x2 <= g.hi[2];
}

// x = phi - 1 and the validity test, exactly as the reference evaluates them.
__device__ __forceinline__ bool load_valid(float p0, float p1, float p2, const Geometry& g,
                                           float& x0, float& x1, float& x2) {
    x0 = __fsub_rn(p0, 1.0f);
    x1 = __fsub_rn(p1, 1.0f);
    x2 = __fsub_rn(p2, 1.0f);
    return position_valid(x0, x1, x2, g);
}

// A 3x4 affine map (column-major, 0-based) in place of a stored deformation.
struct AffineMap {
    float m[12];
};

// Position of sample voxel (i, j, k) under A, rounded as the reference CPU code
// (artifacts/C/pushpull.c:190-200): xj = A[3+c] j + A[6+c] k + A[9+c], then
// x = xj + A[c] i, every operation rounded separately.
__device__ __forceinline__ void affine_position(const AffineMap& A, float fi, float fj, float fk, float& x0,
                                                float& x1, float& x2) {
    float x[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float xj = __fadd_rn(__fadd_rn(__fmul_rn(A.m[3 + c], fj), __fmul_rn(A.m[6 + c], fk)), A.m[9 + c]);
        x[c] = __fadd_rn(xj, __fmul_rn(A.m[c], fi));
    }
    x0 = x[0];
    x1 = x[1];
    x2 = x[2];
}

// Map an unbounded tap index into [0, d) and return the sign the boundary rule
// attaches to it.  In-range taps (the common case) skip the 64-bit modulo.
__device__ __forceinline__ long long fold_tap(int bnd, long long i, long long d, float& sign) {
    sign = 1.0f;
    if (i >= 0 && i < d) return i;
    if (bnd == 0) {
        if (i < 0 && i >= -d) return i + d;   // one period either side: no 64-bit modulo
        if (i >= d && i < 2 * d) return i - d;
        long long r = i % d;
        return r < 0 ? r + d : r;
    }
    const long long n2 = 2 * d;
    long long r;
    if (i < 0 && i >= -d) {
        r = i + n2;                       // fast path one period to the left
    } else if (i >= d && i < n2) {
        r = i;
    } else {
        r = i % n2;
        if (r < 0) r += n2;
    }
    if (r < d) return r;
    if (bnd == 2) sign = -1.0f;
    return n2 - 1 - r;
}

// B-spline weights for the DP taps that start at the returned first tap (as a
// float holding an integer).  ORD 0: values; 1: values and first derivative;
// 2: also the second derivative.
template <int DP, int ORD>
__device__ __forceinline__ float spline_weights(float x, float* w, float* dw, float* hw) {
    const float fo = ceilf(__fsub_rn(x, 0.5f * (float)DP));
    if constexpr (DP == 1) {
        w[0] = 1.0f;
        if constexpr (ORD >= 1) dw[0] = 0.0f;
        if constexpr (ORD >= 2) hw[0] = 0.0f;
    } else if constexpr (DP == 2) {             // t in (0, 1]
        const float t = __fsub_rn(x, fo);
        w[0] = 1.0f - t;
        w[1] = t;
        if constexpr (ORD >= 1) { dw[0] = -1.0f; dw[1] = 1.0f; }
        if constexpr (ORD >= 2) { hw[0] = 0.0f; hw[1] = 0.0f; }
    } else if constexpr (DP == 3) {             // s = t - 1 in (-1/2, 1/2]
        const float s = __fsub_rn(x, fo + 1.0f);
        const float a = 0.5f - s, b = 0.5f + s;
        w[0] = 0.5f * a * a;
        w[1] = 0.75f - s * s;
        w[2] = 0.5f * b * b;
        if constexpr (ORD >= 1) { dw[0] = -a; dw[1] = -2.0f * s; dw[2] = b; }
        if constexpr (ORD >= 2) { hw[0] = 1.0f; hw[1] = -2.0f; hw[2] = 1.0f; }
    } else if constexpr (DP == 4) {             // s = t - 1 in (0, 1]
        const float s = __fsub_rn(x, fo + 1.0f);
        const float a = 1.0f - s;
        w[0] = a * a * a * (1.0f / 6.0f);
        w[1] = (2.0f / 3.0f) - s * s * (1.0f - 0.5f * s);
        w[2] = (2.0f / 3.0f) - a * a * (1.0f - 0.5f * a);
        w[3] = s * s * s * (1.0f / 6.0f);
        if constexpr (ORD >= 1) {
            dw[0] = -0.5f * a * a;
            dw[1] = s * (1.5f * s - 2.0f);
            dw[2] = -a * (1.5f * a - 2.0f);
            dw[3] = 0.5f * s * s;
        }
        if constexpr (ORD >= 2) {
            hw[0] = a;
            hw[1] = 3.0f * s - 2.0f;
            hw[2] = 3.0f * a - 2.0f;
            hw[3] = s;
        }
    } else {                                    // DP == 5, s = t - 2 in (-1/2, 1/2]
        const float s = __fsub_rn(x, fo + 2.0f);
        const float a = 0.5f - s, b = 0.5f + s, p = 1.0f + s, q = 1.0f - s;
        w[0] = a * a * a * a * (1.0f / 24.0f);
        w[4] = b * b * b * b * (1.0f / 24.0f);
        w[2] = (115.0f / 192.0f) + s * s * (s * s * 0.25f - 0.625f);
        w[1] = (55.0f / 96.0f) + p * ((5.0f / 24.0f) + p * (-1.25f + p * ((5.0f / 6.0f) - p * (1.0f / 6.0f))));
        w[3] = (55.0f / 96.0f) + q * ((5.0f / 24.0f) + q * (-1.25f + q * ((5.0f / 6.0f) - q * (1.0f / 6.0f))));
        if constexpr (ORD >= 1) {
            dw[0] = -a * a * a * (1.0f / 6.0f);
            dw[4] = b * b * b * (1.0f / 6.0f);
            dw[2] = s * (s * s - 1.25f);
            dw[1] = (5.0f / 24.0f) + p * (-2.5f + p * (2.5f - p * (2.0f / 3.0f)));
            dw[3] = -((5.0f / 24.0f) + q * (-2.5f + q * (2.5f - q * (2.0f / 3.0f))));
        }
        if constexpr (ORD >= 2) {
            hw[0] = 0.5f * a * a;
            hw[4] = 0.5f * b * b;
            hw[2] = 3.0f * s * s - 1.25f;
            hw[1] = -2.5f + p * (5.0f - 2.0f * p);
            hw[3] = -2.5f + q * (5.0f - 2.0f * q);
        }
    }
    return fo;
}

template <int DP, int ORD>
__device__ __forceinline__ long long spline_taps(float x, float* w, float* dw, float* hw) {
    return (long long)spline_weights<DP, ORD>(x, w, dw, hw);
}

// 32-bit first tap (saturating), for callers that know it is in range.
template <int DP, int ORD>
__device__ __forceinline__ int spline_taps32(float x, float* w, float* dw, float* hw) {
    return __float2int_rz(spline_weights<DP, ORD>(x, w, dw, hw));
}

// First tap as a saturating 32-bit integer: ceil(x - dp/2) with the reference's
// float rounding; equals (int64) ceilf(...) whenever that fits in 32 bits.
__device__ __forceinline__ int first_tap32(float x, int DP) { return __float2int_ru(__fsub_rn(x, 0.5f * (float)DP)); }

// Runtime-degree variant (dp in 1..5) writing kMaxDP slots; unused slots get 0.
template <int ORD>
__device__ __forceinline__ long long spline_taps_rt(int dp, float x, float* w, float* dw, float* hw) {
#pragma unroll
    for (int i = 0; i < kMaxDP; ++i) {
        w[i] = 0.0f;
        if constexpr (ORD >= 1) dw[i] = 0.0f;
        if constexpr (ORD >= 2) hw[i] = 0.0f;
    }
    switch (dp) {
        case 1: return spline_taps<1, ORD>(x, w, dw, hw);
        case 2: return spline_taps<2, ORD>(x, w, dw, hw);
        case 3: return spline_taps<3, ORD>(x, w, dw, hw);
        case 4: return spline_taps<4, ORD>(x, w, dw, hw);
        default: return spline_taps<5, ORD>(x, w, dw, hw);
    }
}

// One axis of a patch: signed weights and folded element offsets (index * stride).
// DP > 0: compile-time width.  DP == 0: runtime width up to kMaxDP.
template <int DP, int ORD, typename IT>
struct Axis {
    static constexpr int N = DP > 0 ? DP : kMaxDP;
    float w[N];
    float dw[ORD >= 1 ? N : 1];
    float hw[ORD >= 2 ? N : 1];
    IT off[N];
    int n;   // live taps

    __device__ __forceinline__ void setup(float x, int dp, int bnd, long long d, IT stride) {
        long long o;
        if constexpr (DP > 0) {
            o = spline_taps<DP, ORD>(x, w, dw, hw);
            n = DP;
        } else {
            o = spline_taps_rt<ORD>(dp, x, w, dw, hw);
            n = dp;
        }
#pragma unroll
        for (int i = 0; i < N; ++i) {
            float s;
            const long long b = fold_tap(bnd, o + i, d, s);
            off[i] = (IT)b * stride;
            w[i] *= s;
            if constexpr (ORD >= 1) dw[i] *= s;
            if constexpr (ORD >= 2) hw[i] *= s;
        }
    }
};

}  // namespace pp
