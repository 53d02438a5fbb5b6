// pp_noalloc.cu -- the fused step for callers that must not allocate device memory.
//
// pp_fused_step needs a little scratch memory (one loss partial per thread
// block and the largest |f0| of every (channel, batch) plane), which it takes
// from a stream-ordered pool owned by this library.  Some callers cannot let a
// library allocate: programs whose own caching allocator has already reserved
// (almost) all device memory, so any further allocation fails or fragments
// their pool, and services with a fixed memory budget that forbid allocation on
// their request path.  pp_fused_step_noalloc does the same work with its scratch
// in a fixed array compiled into the library instead, so it calls no allocator.
#include <mutex>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "pp_kernels.cuh"
#include "pp_tiled.cuh"
#include "pushpull_gb300.h"

namespace pp {
int fail_status(int code, const char* fmt, ...);
int prepare_args(LaunchArgs& a, float* out, const float* phi, const float* in, const pp_usize d0[3],
                 const pp_usize d1[3], int nc, int nb, const int* bnd, int nbnd, const int deg[3], int ext);
TileCfg tile_for(int op_index, int deg);
int current_path();
}  // namespace pp

namespace {

// Scratch layout: PP_NOALLOC_MAX_PARTIALS doubles, then PP_NOALLOC_MAX_PLANES
// unsigned words.  80 KiB in all, held by every device that loads the library
// until the process exits.
constexpr size_t kPartialBytes = (size_t)PP_NOALLOC_MAX_PARTIALS * sizeof(double);
constexpr size_t kScratchBytes = kPartialBytes + (size_t)PP_NOALLOC_MAX_PLANES * sizeof(unsigned);
static_assert(kPartialBytes % 256 == 0, "plane maxima must start 256-byte aligned");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// In host code g_noalloc_scratch names a host-side shadow, not device memory:
// the device address comes from cudaGetSymbolAddress, once per device and
// context, with that device current.  The address is cached together with the
// unique id of the context it was taken in; a call under a different context
// (after cudaDeviceReset re-created the primary context, which reloads this
// module) queries it again instead of using a stale address.
constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
void* g_addr[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};

// Unique id of the current context (0 when the driver cannot say).
unsigned long long current_context_id() {
    static std::once_flag once;
    static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

int scratch_address(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return pp::fail_status(PP_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return pp::fail_status(PP_ERR_UNSUPPORTED, "device %d out of range", dev);
    // the runtime makes the device's primary context current with cudaGetSymbolAddress
    // below on a first call; query the id after that, and compare on later calls
    std::lock_guard<std::mutex> lk(g_addr_mu);
    const unsigned long long ctx = g_addr[dev] ? current_context_id() : 0;
    if (!g_addr[dev] || ctx == 0 || ctx != g_ctx_id[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return pp::fail_status(PP_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        g_addr[dev] = p;
        g_ctx_id[dev] = current_context_id();
    }
    *out = g_addr[dev];
    return PP_OK;
}

}  // namespace

extern "C" int pp_fused_step_noalloc(double* loss, float* df, float* dphi, const float* f0, const float* phi,
                                     const float* g, const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
                                     const int* bnd, int nbnd, const int deg[3], int ext, int accumulate,
                                     void* stream) {
    using namespace pp;
    LaunchArgs a{};
    int rc = prepare_args(a, df, phi, f0, d0, d1, nc, nb, bnd, nbnd, deg, ext);
    if (rc != PP_OK) return rc;
    if (!loss) return fail_status(PP_ERR_NULL, "loss pointer must not be NULL");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    // sizes are checked against the fixed scratch before anything is written
    const TileCfg t = tile_for(PP_OP_FUSED, deg[0]);
    bool tiled = false;
    long long slots = 0;
    int grid = 0;
    if (a.g.n1 > 0) {
        if (!g || !dphi) return fail_status(PP_ERR_NULL, "g and dphi must not be NULL");
        if ((reinterpret_cast<uintptr_t>(g) & 3u) || (reinterpret_cast<uintptr_t>(dphi) & 3u))
            return fail_status(PP_ERR_ALIGN, "float pointers must be 4-byte aligned");
        a.up = g;
        a.out2 = dphi;
        tiled = current_path() != PP_PATH_DIRECT && tiled_supported(a, t);
        if (tiled) {
            grid = fused_tiled_grid(a, t);
            slots = grid;
        } else {
            const dim3 gd = fused_direct_grid(a);
            slots = (long long)gd.x * gd.y;
        }
        const long long planes = (long long)a.g.nc * a.g.nb;
        if (slots > PP_NOALLOC_MAX_PARTIALS)
            return fail_status(PP_ERR_TOO_LARGE,
                               "pp_fused_step_noalloc: %lld loss partials needed, the fixed scratch holds %d "
                               "(reduce nb or use pp_fused_step)", slots, PP_NOALLOC_MAX_PARTIALS);
        if (planes > PP_NOALLOC_MAX_PLANES)
            return fail_status(PP_ERR_TOO_LARGE,
                               "pp_fused_step_noalloc: nc*nb = %lld planes, the fixed scratch holds %d "
                               "(use pp_fused_step)", planes, PP_NOALLOC_MAX_PLANES);
    }
    if (!accumulate && a.g.n0 > 0 && df) {
        e = cudaMemsetAsync(df, 0, (size_t)a.g.n0 * a.g.nc * a.g.nb * sizeof(float), s);
        if (e != cudaSuccess) return fail_status(PP_ERR_CUDA, "zero df: %s", cudaGetErrorString(e));
    }
    if (a.g.n1 == 0) {
        e = cudaMemsetAsync(loss, 0, sizeof(double), s);
        return e == cudaSuccess ? PP_OK : fail_status(PP_ERR_CUDA, "zero loss: %s", cudaGetErrorString(e));
    }
    const long long planes = (long long)a.g.nc * a.g.nb;
    void* base = nullptr;
    if ((rc = scratch_address(&base)) != PP_OK) return rc;
    double* partial = static_cast<double*>(base);
    unsigned* fmax = reinterpret_cast<unsigned*>(static_cast<unsigned char*>(base) + kPartialBytes);
    a.partial = partial;
    a.fmax = fmax;
    // the array keeps the previous call's contents: every partial is rewritten by
    // its block, the plane maxima are accumulated and so start from zero
    e = cudaSuccess;
    if (tiled) {
        e = cudaMemsetAsync(fmax, 0, (size_t)planes * sizeof(unsigned), s);
        if (e == cudaSuccess) e = launch_absmax(f0, a.g.n0, (int)planes, fmax, s);
    }
    if (e == cudaSuccess) e = tiled ? launch_fused_tiled(a, t, s, grid) : launch_fused_direct(a, s);
    if (e == cudaSuccess) e = launch_sum_partials(partial, (int)slots, loss, s);
    if (e != cudaSuccess) return fail_status(PP_ERR_CUDA, "fused step launch: %s", cudaGetErrorString(e));
    return PP_OK;
}
