// pp_affine.cu -- pull and push under a 3x4 affine map instead of a stored
// deformation: the sample position of output voxel (i, j, k) is A * (i, j, k, 1)
// (0-based, the matrix already adjusted from the 1-based convention), so the
// kernels read only the image (pull) or the values (push): 8 bytes per voxel.
//
// Reference: affine_pull_element / affine_push_element (artifacts/C/pushpull.cu:
// 187-231) and the CPU pull_affine / push_affine (artifacts/C/pushpull.c:176-243),
// whose rounding of the position this follows: xj = A[3]*j + A[6]*k + A[9],
// then x = xj + A[0]*i, every operation rounded separately.
#include "pp_voxel.cuh"
#include "pushpull_gb300.h"

namespace pp {
namespace {

struct Affine {
    float m[12];   // column-major 3x4, 0-based
};

// 0-based position of voxel v of the d1 grid, rounded as the reference CPU code
template <typename IT>
__device__ __forceinline__ void affine_position(const Affine& A, IT v, IT d1x, IT d1y, float& x0, float& x1,
                                                float& x2) {
    const IT jk = v / d1x;
    const IT i = v - jk * d1x;
    const IT k = jk / d1y;
    const IT j = jk - k * d1y;
    const float fi = (float)i, fj = (float)j, fk = (float)k;
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

// the reference's VOXOK on a 0-based position (artifacts/C/pushpull.c:6-9)
__device__ __forceinline__ bool position_valid(float x0, float x1, float x2, const Geometry& g) {
    if (!(finitef(x0) && finitef(x1) && finitef(x2))) return false;
    if (g.ext) return true;
    return x0 >= -0.01f && x0 <= g.hi[0] && x1 >= -0.01f && x1 <= g.hi[1] && x2 >= -0.01f && x2 <= g.hi[2];
}

template <int DP, typename IT>
__global__ void __launch_bounds__(256) k_affine_pull(LaunchArgs a, Affine A) {
    const Geometry& g = a.g;
    const IT n1 = (IT)g.n1, d1x = (IT)g.d1[0], d1y = (IT)g.d1[1];
    const int b = blockIdx.y;
    for (IT v = (IT)blockIdx.x * blockDim.x + threadIdx.x; v < n1; v += (IT)gridDim.x * blockDim.x) {
        float x0, x1, x2;
        affine_position<IT>(A, v, d1x, d1y, x0, x1, x2);
        if (!position_valid(x0, x1, x2, g)) pull_voxel_nan<kPull>(a, b, (long long)v);
        else pull_voxel_global<DP, kPull, IT>(a, b, (long long)v, x0, x1, x2);
    }
}

template <int DP, typename IT>
__global__ void __launch_bounds__(256) k_affine_push(LaunchArgs a, Affine A) {
    const Geometry& g = a.g;
    const IT n1 = (IT)g.n1, d1x = (IT)g.d1[0], d1y = (IT)g.d1[1];
    const int b = blockIdx.y;
    for (IT v = (IT)blockIdx.x * blockDim.x + threadIdx.x; v < n1; v += (IT)gridDim.x * blockDim.x) {
        float x0, x1, x2;
        affine_position<IT>(A, v, d1x, d1y, x0, x1, x2);
        if (position_valid(x0, x1, x2, g)) push_voxel_global<DP, kPush, IT>(a, b, (long long)v, x0, x1, x2);
    }
}

template <typename IT>
cudaError_t launch_affine_it(bool push, const LaunchArgs& a, const Affine& A, dim3 grid, cudaStream_t s) {
    const int d = a.g.dp[0];
    const bool iso = a.g.dp[1] == d && a.g.dp[2] == d;
#define PP_AFF_CASE(DPV)                                                           \
    case DPV:                                                                      \
        if (push) k_affine_push<DPV, IT><<<grid, 256, 0, s>>>(a, A);               \
        else k_affine_pull<DPV, IT><<<grid, 256, 0, s>>>(a, A);                    \
        break;
    switch (iso ? d : 0) {
        PP_AFF_CASE(1)
        PP_AFF_CASE(2)
        PP_AFF_CASE(3)
        PP_AFF_CASE(4)
        PP_AFF_CASE(5)
        PP_AFF_CASE(0)
        default: break;
    }
#undef PP_AFF_CASE
    return cudaGetLastError();
}

}  // namespace

int fail_status(int code, const char* fmt, ...);
int prepare_args(LaunchArgs& a, float* out, const float* phi, const float* in, const pp_usize d0[3],
                 const pp_usize d1[3], int nc, int nb, const int* bnd, int nbnd, const int deg[3], int ext);

int run_affine(bool push, float* out, const float* in, const float* Aff, const pp_usize d0[3], const pp_usize d1[3],
               int nc, int nb, const int* bnd, int nbnd, const int deg[3], int ext, int accumulate, void* stream) {
    LaunchArgs a{};
    // the affine ops read no deformation: the input stands in for it in the shared checks
    int rc = prepare_args(a, out, in, in, d0, d1, nc, nb, bnd, nbnd, deg, ext);
    if (rc != PP_OK) return rc;
    if (!Aff) return fail_status(PP_ERR_NULL, "Aff must not be NULL");
    a.phi = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    if (push && !accumulate && a.g.n0 > 0) {
        e = cudaMemsetAsync(out, 0, (size_t)a.g.n0 * a.g.nc * a.g.nb * sizeof(float), s);
        if (e != cudaSuccess) return fail_status(PP_ERR_CUDA, "zero output: %s", cudaGetErrorString(e));
    }
    if (a.g.n1 == 0) return PP_OK;
    Affine A;
    for (int q = 0; q < 12; ++q) A.m[q] = Aff[q];
    const long long blocks_needed = (a.g.n1 + 255) / 256;
    const long long cap = (long long)sm_count() * 8;
    const dim3 grid((unsigned)(blocks_needed < cap ? blocks_needed : cap), (unsigned)a.g.nb);
    const bool small = a.g.n0 < (1LL << 31) - 1 && a.g.n1 < (1LL << 31) - 1;
    e = small ? launch_affine_it<int>(push, a, A, grid, s) : launch_affine_it<long long>(push, a, A, grid, s);
    if (e != cudaSuccess) return fail_status(PP_ERR_CUDA, "affine launch: %s", cudaGetErrorString(e));
    return PP_OK;
}

}  // namespace pp

extern "C" {

int pp_pull_affine(float* f1, const float* f0, const float* Aff, const pp_usize d0[3], const pp_usize d1[3], int nc,
                   int nb, const int* bnd, int nbnd, const int deg[3], int ext, void* stream) {
    return pp::run_affine(false, f1, f0, Aff, d0, d1, nc, nb, bnd, nbnd, deg, ext, 0, stream);
}

int pp_push_affine(float* f0, const float* f1, const float* Aff, const pp_usize d0[3], const pp_usize d1[3], int nc,
                   int nb, const int* bnd, int nbnd, const int deg[3], int ext, int accumulate, void* stream) {
    return pp::run_affine(true, f0, f1, Aff, d0, d1, nc, nb, bnd, nbnd, deg, ext, accumulate, stream);
}

}  // extern "C"
