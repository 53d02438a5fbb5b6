// pp_affine.cu -- pull and push under a 3x4 affine map instead of a stored
// deformation: the sample position of output voxel (i, j, k) is A * (i, j, k, 1)
// (0-based, the matrix already adjusted from the 1-based convention), so the
// kernels read only the image (pull) or the values (push): 8 bytes per voxel.
//
// Isotropic degrees 1..4 run on the tiled kernels with the positions computed
// in place: the warp-specialised pull (pp_ws.cuh) and the tiled push
// (pp_tiled_impl.cuh, pp_tiled_affine.cu), whose footprint boxes an affine map
// keeps regular.  The per-voxel kernels below take everything else
// (anisotropic degrees, degenerate grids, or the direct path).
//
// Reference: affine_pull_element / affine_push_element (artifacts/C/pushpull.cu:
// 187-231) and the CPU pull_affine / push_affine (artifacts/C/pushpull.c:176-243),
// whose rounding of the position this follows: xj = A[3]*j + A[6]*k + A[9],
// then x = xj + A[0]*i, every operation rounded separately.
#include "pp_tiled.cuh"
#include "pp_voxel.cuh"
#include "pushpull_gb300.h"

namespace pp {
namespace {

// 0-based position of voxel v of the d1 grid
template <typename IT>
__device__ __forceinline__ void voxel_position(const AffineMap& A, IT v, IT d1x, IT d1y, float& x0, float& x1,
                                               float& x2) {
    const IT jk = v / d1x;
    const IT i = v - jk * d1x;
    const IT k = jk / d1y;
    const IT j = jk - k * d1y;
    affine_position(A, (float)i, (float)j, (float)k, x0, x1, x2);
}

template <int DP, typename IT>
__global__ void __launch_bounds__(256) k_affine_pull(LaunchArgs a, AffineMap A) {
    const Geometry& g = a.g;
    const IT n1 = (IT)g.n1, d1x = (IT)g.d1[0], d1y = (IT)g.d1[1];
    const int b = blockIdx.y;
    for (IT v = (IT)blockIdx.x * blockDim.x + threadIdx.x; v < n1; v += (IT)gridDim.x * blockDim.x) {
        float x0, x1, x2;
        voxel_position<IT>(A, v, d1x, d1y, x0, x1, x2);
        if (!position_valid(x0, x1, x2, g)) pull_voxel_nan<kPull>(a, b, (long long)v);
        else pull_voxel_global<DP, kPull, IT>(a, b, (long long)v, x0, x1, x2);
    }
}

template <int DP, typename IT>
__global__ void __launch_bounds__(256) k_affine_push(LaunchArgs a, AffineMap A) {
    const Geometry& g = a.g;
    const IT n1 = (IT)g.n1, d1x = (IT)g.d1[0], d1y = (IT)g.d1[1];
    const int b = blockIdx.y;
    for (IT v = (IT)blockIdx.x * blockDim.x + threadIdx.x; v < n1; v += (IT)gridDim.x * blockDim.x) {
        float x0, x1, x2;
        voxel_position<IT>(A, v, d1x, d1y, x0, x1, x2);
        if (position_valid(x0, x1, x2, g)) push_voxel_global<DP, kPush, IT>(a, b, (long long)v, x0, x1, x2);
    }
}

template <typename IT>
cudaError_t launch_affine_it(bool push, const LaunchArgs& a, const AffineMap& A, dim3 grid, cudaStream_t s) {
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
TileCfg tile_for(int op_index, int deg);
int current_path();
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
    AffineMap A;
    for (int q = 0; q < 12; ++q) A.m[q] = Aff[q];
    e = cudaErrorNotSupported;
    if (current_path() != PP_PATH_DIRECT) {
        // the registry's pull (op 0) and push (op 3) entries decide, as for the
        // deformation ops: a zero budget means the per-voxel kernels
        if (!push) {
            if (tile_for(0, deg[0]).cap > 0 && ws_supported(a)) e = launch_ws_pull_affine(a, A, s);
        } else {
            const TileCfg t = tile_for(3, deg[0]);
            if (t.cap > 0 && tiled_supported(a, t)) e = launch_push_tiled_affine(a, t, A, s);
        }
        if (e == cudaErrorNotSupported) (void)cudaGetLastError();
        else if (e != cudaSuccess) return fail_status(PP_ERR_CUDA, "affine launch: %s", cudaGetErrorString(e));
        else return PP_OK;
    }
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
