// pp_abi.cu -- the C ABI: argument validation, dispatch, errors, and the
// host-pointer compatibility layer with the reference's CPU signatures.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "pp_kernels.cuh"
#include "pp_tiled.cuh"
#include "pushpull_gb300.h"

namespace pp {

namespace {
thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(PP_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

bool aligned4(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 3u) == 0; }

bool mul_ok(long long a, long long b, long long& r) {
    if (a < 0 || b < 0) return false;
    if (a != 0 && b > (1LL << 62) / a) return false;
    r = a * b;
    return true;
}
}  // namespace

int sm_count() {
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (cache[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        cache[dev] = n;
    }
    return cache[dev];
}

void set_error_message(const char* msg) { g_err = msg ? msg : ""; }

// Stream-ordered scratch comes from a memory pool owned by this library, one per
// device, that keeps its memory between calls (the device's default pool returns
// memory to the system at every synchronisation, which would re-map it per call).
static cudaError_t scratch_pool(cudaMemPool_t* out) {
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(mu);
    if (!pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p;
        if ((e = cudaMemPoolCreate(&p, &props)) != cudaSuccess) return e;
        unsigned long long keep = ~0ULL;
        if ((e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess) return e;
        pools[dev] = p;
    }
    *out = pools[dev];
    return cudaSuccess;
}

cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t s) {
    cudaMemPool_t pool;
    cudaError_t e = scratch_pool(&pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

// ---- tile configuration registry (per op, per isotropic degree) and path choice
namespace {
std::mutex g_cfg_mu;
TileCfg g_tiles[6][5];   // ops: pull, pull_grad, pull_hess, push, push_grad, fused step
bool g_tiles_init = false;
int g_path = PP_PATH_AUTO;

// The tile code (lx, ly, lz) = (3, 3, 4) selects the warp-specialised pull
// kernels (pp_ws.cuh, 8 x 8 x 30 tiles); every other shape the
// block-synchronous ones.
bool is_ws_tile(const TileCfg& t) { return t.lx == 3 && t.ly == 3 && t.lz == 4 && t.cap > 0; }

void init_tiles_locked() {
    if (g_tiles_init) return;
    // 8x8x8 tiles; the push family keeps two words per accumulator element; the
    // fused step's 2560-float budget at degree 2 leaves room for three CTAs per SM.
    // Degrees 0 and 1 (one or two taps per axis) default to the per-voxel
    // kernels (cap 0; the pull family at degree 1 is set below): with so few
    // taps, gathering through L2 is faster than a block-synchronous staging of
    // a footprint box (192^3, GB300: pull 0.10 vs 0.16 ms, push 0.13 vs
    // 0.24 ms, fused step 0.29 vs 0.40 ms at degree 1).
    for (int op = 0; op < 6; ++op)
        for (int d = 0; d < 5; ++d)
            g_tiles[op][d] = TileCfg{3, 3, 3, d <= 1 ? 0 : (op < 3 ? 8192 : (op < 5 ? 16384 : (d == 2 ? 2560 : 4096)))};
    // pull, pull_grad and pull_hess (with the dot ops, which share their
    // entries) at degrees 1..4: the warp-specialised kernels (192^3, GB300,
    // against the next best family: cubic pull 0.179 vs 0.254 ms, pull_grad
    // 0.198 vs 0.262 ms, pull_hess 0.222 vs 0.285 ms, pull_grad_dot 0.201 vs
    // 0.271 ms, pull_hess_dot 0.236 vs 0.298 ms; linear pull 0.084 vs 0.095 ms,
    // pull_grad 0.095 vs 0.144 ms, pull_hess 0.117 vs 0.177 ms)
    for (int op = 0; op < 3; ++op)
        for (int d = 1; d < 5; ++d) g_tiles[op][d] = TileCfg{3, 3, 4, 15360};
    g_tiles_init = true;
}
}  // namespace

TileCfg tile_for(int op_index, int deg) {
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    init_tiles_locked();
    return g_tiles[op_index][deg < 0 ? 0 : (deg > 4 ? 4 : deg)];
}

int current_path() {
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    return g_path;
}

// Validate the common arguments and fill the launch descriptor.
// comps_in / comps_out: planar components per channel of the input / output.
static int prepare(LaunchArgs& a, float* out, const float* phi, const float* in,
                   const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
                   const int* bnd, int nbnd, const int deg[3], int ext) {
    g_err.clear();
    if (!d0 || !d1 || !deg) return fail(PP_ERR_NULL, "d0, d1 and deg must not be NULL");
    if (nc < 1 || nb < 1) return fail(PP_ERR_CHANNELS, "nc (%d) and nb (%d) must be >= 1", nc, nb);
    if (nb > 65535) return fail(PP_ERR_TOO_LARGE, "nb (%d) exceeds 65535", nb);
    if (!(nbnd == 1 || nbnd == nc))
        return fail(PP_ERR_CHANNELS, "nbnd (%d) must be 1 or nc (%d)", nbnd, nc);
    if (!bnd) return fail(PP_ERR_NULL, "bnd must not be NULL");
    if (nbnd > kMaxBnd)
        return fail(PP_ERR_TOO_LARGE, "per-channel boundaries support at most %d channels per call", kMaxBnd);
    for (int k = 0; k < 3; ++k) {
        if (deg[k] < 0 || deg[k] > 4) return fail(PP_ERR_DEGREE, "deg[%d] = %d outside 0..4", k, deg[k]);
        if (d0[k] > (pp_usize)(1ULL << 40) || d1[k] > (pp_usize)(1ULL << 40))
            return fail(PP_ERR_DIMS, "dimension too large");
    }
    for (int c = 0; c < nbnd; ++c)
        for (int k = 0; k < 3; ++k) {
            const int b = bnd[3 * c + k];
            if (b < 0 || b > 2) return fail(PP_ERR_BOUND, "bnd[%d] = %d outside {0,1,2}", 3 * c + k, b);
            a.bnd.code[c][k] = (unsigned char)b;
        }
    Geometry& g = a.g;
    long long t;
    for (int k = 0; k < 3; ++k) {
        g.d0[k] = (long long)d0[k];
        g.d1[k] = (long long)d1[k];
        g.dp[k] = deg[k] + 1;
    }
    if (!mul_ok(g.d0[0], g.d0[1], t) || !mul_ok(t, g.d0[2], g.n0)) return fail(PP_ERR_DIMS, "d0 overflows");
    if (!mul_ok(g.d1[0], g.d1[1], t) || !mul_ok(t, g.d1[2], g.n1)) return fail(PP_ERR_DIMS, "d1 overflows");
    for (int k = 0; k < 3; ++k) {
        volatile float dk = (float)g.d0[k];   // float arithmetic, as artifacts/C/pushpull.c:7-9
        g.hi[k] = dk - 0.99f;
    }
    g.nc = nc;
    g.nb = nb;
    g.ext = ext ? 1 : 0;
    g.nbnd = nbnd;
    if (g.n1 == 0) return PP_OK;   // nothing to sample: the call is a no-op
    if (g.n0 == 0) return fail(PP_ERR_DIMS, "image has zero voxels but %lld samples were requested", g.n1);
    if (!out || !phi || !in) return fail(PP_ERR_NULL, "data pointers must not be NULL");
    if (!aligned4(out) || !aligned4(phi) || !aligned4(in))
        return fail(PP_ERR_ALIGN, "float pointers must be 4-byte aligned");
    a.phi = phi;
    a.in = in;
    a.out = out;
    return PP_OK;
}

int fail_status(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

int prepare_args(LaunchArgs& a, float* out, const float* phi, const float* in, const pp_usize d0[3],
                 const pp_usize d1[3], int nc, int nb, const int* bnd, int nbnd, const int deg[3], int ext) {
    return prepare(a, out, phi, in, d0, d1, nc, nb, bnd, nbnd, deg, ext);
}

static int run_pull(int op, float* out, const float* phi, const float* f0, const pp_usize d0[3],
                    const pp_usize d1[3], int nc, int nb, const int* bnd, int nbnd, const int deg[3],
                    int ext, void* stream, const float* up = nullptr) {
    LaunchArgs a{};
    int rc = prepare(a, out, phi, f0, d0, d1, nc, nb, bnd, nbnd, deg, ext);
    if (rc != PP_OK || a.g.n1 == 0) return rc;
    if (op == kPullGradDot || op == kPullHessDot) {
        if (!up) return fail(PP_ERR_NULL, "upstream pointer must not be NULL");
        if (!aligned4(up)) return fail(PP_ERR_ALIGN, "float pointers must be 4-byte aligned");
        a.up = up;
    }
    TileCfg t = tile_for(op < 3 ? op : op - 2, deg[0]);
    cudaError_t e = cudaErrorNotSupported;
    const bool auto_path = current_path() != PP_PATH_DIRECT;
    if (auto_path && is_ws_tile(t)) {
        if (ws_supported(a)) e = launch_ws_pull(op, a, (cudaStream_t)stream);
        if (e == cudaErrorNotSupported) {
            (void)cudaGetLastError();
            // ops or geometries the warp-specialised kernels do not take: the
            // block-synchronous kernels, or the per-voxel ones at one or two taps per axis
            t = TileCfg{3, 3, 3, deg[0] <= 1 ? 0 : 8192};
        }
    }
    if (e == cudaErrorNotSupported) {
        if (auto_path && t.cap > 0 && tiled_supported(a, t))
            e = launch_pull_tiled(op, a, t, (cudaStream_t)stream);
        else
            e = launch_pull_direct(op, a, (cudaStream_t)stream);
    }
    if (e != cudaSuccess) return cuda_fail(e, "pull launch");
    return PP_OK;
}

static int run_push(int op, float* out, const float* phi, const float* in, const pp_usize d0[3],
                    const pp_usize d1[3], int nc, int nb, const int* bnd, int nbnd, const int deg[3],
                    int ext, int accumulate, void* stream) {
    LaunchArgs a{};
    int rc = prepare(a, out, phi, in, d0, d1, nc, nb, bnd, nbnd, deg, ext);
    if (rc != PP_OK) return rc;
    const Geometry& g = a.g;
    if (!accumulate && g.n0 > 0) {
        if (!out) return fail(PP_ERR_NULL, "output pointer must not be NULL");
        cudaError_t e = cudaMemsetAsync(out, 0, (size_t)g.n0 * g.nc * g.nb * sizeof(float), (cudaStream_t)stream);
        if (e != cudaSuccess) return cuda_fail(e, "zero output");
    }
    if (g.n1 == 0) return PP_OK;
    const TileCfg t = tile_for(3 + op, deg[0]);
    cudaError_t e;
    if (current_path() != PP_PATH_DIRECT && tiled_supported(a, t))
        e = launch_push_tiled(op, a, t, (cudaStream_t)stream);
    else
        e = launch_push_direct(op, a, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "push launch");
    return PP_OK;
}

// Fused step: loss (double, written), df (accumulated or zeroed first), dphi (written).
static int run_fused(double* loss, float* df, float* dphi, const float* f0, const float* phi, const float* g,
                     const pp_usize d0[3], const pp_usize d1[3], int nc, int nb, const int* bnd, int nbnd,
                     const int deg[3], int ext, int accumulate, void* stream) {
    LaunchArgs a{};
    int rc = prepare(a, df, phi, f0, d0, d1, nc, nb, bnd, nbnd, deg, ext);
    if (rc != PP_OK) return rc;
    if (!loss) return fail(PP_ERR_NULL, "loss pointer must not be NULL");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    if (!accumulate && a.g.n0 > 0 && df) {
        e = cudaMemsetAsync(df, 0, (size_t)a.g.n0 * a.g.nc * a.g.nb * sizeof(float), s);
        if (e != cudaSuccess) return cuda_fail(e, "zero df");
    }
    if (a.g.n1 == 0) {
        e = cudaMemsetAsync(loss, 0, sizeof(double), s);
        return e == cudaSuccess ? PP_OK : cuda_fail(e, "zero loss");
    }
    if (!g || !dphi) return fail(PP_ERR_NULL, "g and dphi must not be NULL");
    if (!aligned4(g) || !aligned4(dphi)) return fail(PP_ERR_ALIGN, "float pointers must be 4-byte aligned");
    a.up = g;
    a.out2 = dphi;
    const TileCfg t = tile_for(PP_OP_FUSED, deg[0]);
    const bool tiled = current_path() != PP_PATH_DIRECT && tiled_supported(a, t);
    long long slots;
    int grid = 0;
    if (tiled) {
        grid = fused_tiled_grid(a, t);
        slots = grid;
    } else {
        const dim3 gd = fused_direct_grid(a);
        slots = (long long)gd.x * gd.y;
    }
    // scratch, stream ordered: per-CTA loss partials and max |f0| per (channel, batch)
    const int planes = a.g.nc * a.g.nb;
    const size_t part_bytes = ((size_t)slots * sizeof(double) + 255) & ~(size_t)255;
    double* partial = nullptr;
    e = scratch_alloc(reinterpret_cast<void**>(&partial), part_bytes + (size_t)planes * sizeof(unsigned), s);
    if (e != cudaSuccess) return cuda_fail(e, "allocate scratch");
    unsigned* fmax = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(partial) + part_bytes);
    a.partial = partial;
    a.fmax = fmax;
    if (tiled) {
        e = cudaMemsetAsync(fmax, 0, (size_t)planes * sizeof(unsigned), s);
        if (e == cudaSuccess) e = launch_absmax(f0, a.g.n0, planes, fmax, s);
    }
    if (e == cudaSuccess) e = tiled ? launch_fused_tiled(a, t, s, grid) : launch_fused_direct(a, s);
    if (e == cudaSuccess) e = launch_sum_partials(partial, (int)slots, loss, s);
    const cudaError_t ef = cudaFreeAsync(partial, s);
    if (e != cudaSuccess) return cuda_fail(e, "fused step launch");
    if (ef != cudaSuccess) return cuda_fail(ef, "free loss partials");
    return PP_OK;
}

}  // namespace pp

using pp::run_fused;
using pp::run_pull;
using pp::run_push;

extern "C" {

int pp_pull(float* f1, const float* phi, const float* f0, const pp_usize d0[3], const pp_usize d1[3], int nc,
            int nb, const int* bnd, int nbnd, const int deg[3], int ext, void* stream) {
    return run_pull(pp::kPull, f1, phi, f0, d0, d1, nc, nb, bnd, nbnd, deg, ext, stream);
}

int pp_pull_grad(float* g1, const float* phi, const float* f0, const pp_usize d0[3], const pp_usize d1[3], int nc,
                 int nb, const int* bnd, int nbnd, const int deg[3], int ext, void* stream) {
    return run_pull(pp::kPullGrad, g1, phi, f0, d0, d1, nc, nb, bnd, nbnd, deg, ext, stream);
}

int pp_pull_hess(float* h1, const float* phi, const float* f0, const pp_usize d0[3], const pp_usize d1[3], int nc,
                 int nb, const int* bnd, int nbnd, const int deg[3], int ext, void* stream) {
    return run_pull(pp::kPullHess, h1, phi, f0, d0, d1, nc, nb, bnd, nbnd, deg, ext, stream);
}

int pp_pull_grad_dot(float* dphi, const float* phi, const float* f0, const float* up, const pp_usize d0[3],
                     const pp_usize d1[3], int nc, int nb, const int* bnd, int nbnd, const int deg[3], int ext,
                     void* stream) {
    return run_pull(pp::kPullGradDot, dphi, phi, f0, d0, d1, nc, nb, bnd, nbnd, deg, ext, stream, up);
}

int pp_pull_hess_dot(float* dphi, const float* phi, const float* f0, const float* up, const pp_usize d0[3],
                     const pp_usize d1[3], int nc, int nb, const int* bnd, int nbnd, const int deg[3], int ext,
                     void* stream) {
    return run_pull(pp::kPullHessDot, dphi, phi, f0, d0, d1, nc, nb, bnd, nbnd, deg, ext, stream, up);
}

int pp_push(float* f0, const float* phi, const float* f1, const pp_usize d0[3], const pp_usize d1[3], int nc,
            int nb, const int* bnd, int nbnd, const int deg[3], int ext, int accumulate, void* stream) {
    return run_push(pp::kPush, f0, phi, f1, d0, d1, nc, nb, bnd, nbnd, deg, ext, accumulate, stream);
}

int pp_push_grad(float* g0, const float* phi, const float* g1, const pp_usize d0[3], const pp_usize d1[3], int nc,
                 int nb, const int* bnd, int nbnd, const int deg[3], int ext, int accumulate, void* stream) {
    return run_push(pp::kPushGrad, g0, phi, g1, d0, d1, nc, nb, bnd, nbnd, deg, ext, accumulate, stream);
}

int pp_push_count(float* f0, float* c0, const float* phi, const float* f1, const pp_usize d0[3], const pp_usize d1[3],
                  int nc, int nb, const int* bnd, int nbnd, const int deg[3], int ext, int accumulate, void* stream) {
    using namespace pp;
    LaunchArgs a{};
    int rc = prepare(a, f0, phi, f1, d0, d1, nc, nb, bnd, nbnd, deg, ext);
    if (rc != PP_OK) return rc;
    if (!c0) return fail(PP_ERR_NULL, "count image pointer must not be NULL");
    if (!aligned4(c0)) return fail(PP_ERR_ALIGN, "float pointers must be 4-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    if (!accumulate && a.g.n0 > 0) {
        const size_t bytes = (size_t)a.g.n0 * a.g.nc * a.g.nb * sizeof(float);
        cudaError_t e = cudaMemsetAsync(f0, 0, bytes, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(c0, 0, bytes, s);
        if (e != cudaSuccess) return cuda_fail(e, "zero outputs");
    }
    if (a.g.n1 == 0) return PP_OK;
    a.out2 = c0;
    const cudaError_t e = launch_push_direct(kPush, a, s);
    return e == cudaSuccess ? PP_OK : cuda_fail(e, "push_count launch");
}

int pp_fused_step(double* loss, float* df, float* dphi, const float* f0, const float* phi, const float* g,
                  const pp_usize d0[3], const pp_usize d1[3], int nc, int nb, const int* bnd, int nbnd,
                  const int deg[3], int ext, int accumulate, void* stream) {
    return run_fused(loss, df, dphi, f0, phi, g, d0, d1, nc, nb, bnd, nbnd, deg, ext, accumulate, stream);
}

const char* pp_last_error(void) { return pp::g_err.c_str(); }

int pp_set_tile(int op, int deg, int lx, int ly, int lz, int cap_floats) {
    pp::g_err.clear();
    if (op < -1 || op > 5) return pp::fail(PP_ERR_UNSUPPORTED, "op %d outside -1..5", op);
    if (deg < -1 || deg > 4) return pp::fail(PP_ERR_DEGREE, "deg %d outside -1..4", deg);
    const bool ws = lx == 3 && ly == 3 && lz == 4;   // the warp-specialised pull tile
    if (!ws && (lx < 0 || ly < 0 || lz < 0 || lx + ly + lz < 5 || lx + ly + lz > 9))
        return pp::fail(PP_ERR_UNSUPPORTED, "tile 2^%d x 2^%d x 2^%d must hold 32..512 voxels (or be the code 3,3,4)", lx,
                        ly, lz);
    if (ws && cap_floats != 0 && (op < 0 || op > 2))
        return pp::fail(PP_ERR_UNSUPPORTED, "the tile code 3,3,4 (warp-specialised kernels) serves pull and pull_grad only");
    if (cap_floats != 0 && (cap_floats < 64 || (cap_floats & 3) || cap_floats > (227 * 1024) / 4))
        return pp::fail(PP_ERR_UNSUPPORTED, "cap %d floats must be 0 or a multiple of 4 in [64, 58112]",
                        cap_floats);
    std::lock_guard<std::mutex> lk(pp::g_cfg_mu);
    pp::init_tiles_locked();
    for (int o = 0; o < 6; ++o)
        for (int d = 0; d < 5; ++d)
            if ((op < 0 || o == op) && (deg < 0 || d == deg)) pp::g_tiles[o][d] = pp::TileCfg{lx, ly, lz, cap_floats};
    return PP_OK;
}

int pp_get_tile(int op, int deg, int* lx, int* ly, int* lz, int* cap_floats) {
    if (op < 0 || op > 5 || deg < 0 || deg > 4) return pp::fail(PP_ERR_UNSUPPORTED, "op/deg out of range");
    if (!lx || !ly || !lz || !cap_floats) return pp::fail(PP_ERR_NULL, "outputs must not be NULL");
    const pp::TileCfg t = pp::tile_for(op, deg);
    *lx = t.lx;
    *ly = t.ly;
    *lz = t.lz;
    *cap_floats = t.cap;
    return PP_OK;
}

int pp_set_path(int path) {
    if (path != PP_PATH_AUTO && path != PP_PATH_DIRECT) return pp::fail(PP_ERR_UNSUPPORTED, "path %d", path);
    std::lock_guard<std::mutex> lk(pp::g_cfg_mu);
    pp::g_path = path;
    return PP_OK;
}

int pp_version(void) { return 100; }

int pp_autotune(int op, float* out, const float* phi, const float* in, const pp_usize d0[3], const pp_usize d1[3],
                int nc, int nb, const int* bnd, int nbnd, const int deg[3], int ext, int reps, void* stream,
                int* best, float* best_ms) {
    using namespace pp;
    if (op < 0 || op > 4) return fail(PP_ERR_UNSUPPORTED, "autotune supports ops 0..4 (got %d)", op);
    if (!deg || !best || !best_ms) return fail(PP_ERR_NULL, "deg, best and best_ms must not be NULL");
    if (deg[0] < 0 || deg[0] > 4) return fail(PP_ERR_DEGREE, "deg[0] = %d outside 0..4", deg[0]);
    if (reps < 1) reps = 3;
    cudaStream_t s = (cudaStream_t)stream;
    const bool is_push = op >= 3;
    auto run = [&]() -> int {
        switch (op) {
            case 0: return pp_pull(out, phi, in, d0, d1, nc, nb, bnd, nbnd, deg, ext, stream);
            case 1: return pp_pull_grad(out, phi, in, d0, d1, nc, nb, bnd, nbnd, deg, ext, stream);
            case 2: return pp_pull_hess(out, phi, in, d0, d1, nc, nb, bnd, nbnd, deg, ext, stream);
            case 3: return pp_push(out, phi, in, d0, d1, nc, nb, bnd, nbnd, deg, ext, 0, stream);
            default: return pp_push_grad(out, phi, in, d0, d1, nc, nb, bnd, nbnd, deg, ext, 0, stream);
        }
    };
    const int tiles[][3] = {{3, 3, 3}, {4, 3, 2}, {4, 2, 3}, {5, 2, 2}, {3, 4, 2}, {3, 3, 2}, {4, 2, 2}, {3, 3, 4}};
    const int caps_pull[] = {6144, 8192, 12288};
    const int caps_push[] = {12288, 16384, 20480};
    const TileCfg saved = tile_for(op, deg[0]);
    const int saved_path = current_path();
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return fail(PP_ERR_CUDA, "event create");
    float bestv = 3.0e38f;
    int bcfg[5] = {saved.lx, saved.ly, saved.lz, saved.cap, PP_PATH_AUTO};
    auto measure = [&](float& ms) -> int {
        int rc = run();                                   // warm-up (and one-time set-up)
        if (rc != PP_OK) return rc;
        float tot = 0.f;
        for (int r = 0; r < reps; ++r) {
            cudaEventRecord(e0, s);
            rc = run();
            cudaEventRecord(e1, s);
            if (rc != PP_OK) return rc;
            if (cudaEventSynchronize(e1) != cudaSuccess) return fail(PP_ERR_CUDA, "event sync");
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            tot += t;
        }
        ms = tot / reps;
        return PP_OK;
    };
    int rc = PP_OK;
    // the per-voxel kernels
    pp_set_path(PP_PATH_DIRECT);
    float ms = 0.f;
    if ((rc = measure(ms)) == PP_OK && ms < bestv) {
        bestv = ms;
        bcfg[4] = PP_PATH_DIRECT;
    }
    pp_set_path(PP_PATH_AUTO);
    for (const auto& t : tiles) {
        const bool ws = t[0] == 3 && t[1] == 3 && t[2] == 4;
        if (ws && is_push) continue;
        for (int ci = 0; ci < (ws ? 1 : 3) && rc == PP_OK; ++ci) {
            const int cap = ws ? 15360 : (is_push ? caps_push[ci] : caps_pull[ci]);
            if (pp_set_tile(op, deg[0], t[0], t[1], t[2], cap) != PP_OK) continue;
            if ((rc = measure(ms)) != PP_OK) break;
            if (ms < bestv) {
                bestv = ms;
                bcfg[0] = t[0];
                bcfg[1] = t[1];
                bcfg[2] = t[2];
                bcfg[3] = cap;
                bcfg[4] = PP_PATH_AUTO;
            }
        }
        if (rc != PP_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    pp_set_path(saved_path);
    if (rc != PP_OK) {
        pp_set_tile(op, deg[0], saved.lx, saved.ly, saved.lz, saved.cap);
        return rc;
    }
    // install the winner: a tile configuration, or cap 0 for the per-voxel kernels
    if (bcfg[4] == PP_PATH_AUTO) pp_set_tile(op, deg[0], bcfg[0], bcfg[1], bcfg[2], bcfg[3]);
    else {
        pp_set_tile(op, deg[0], saved.lx, saved.ly, saved.lz, 0);
        bcfg[0] = saved.lx;
        bcfg[1] = saved.ly;
        bcfg[2] = saved.lz;
        bcfg[3] = 0;
    }
    for (int k = 0; k < 5; ++k) best[k] = bcfg[k];
    *best_ms = bestv;
    return PP_OK;
}

unsigned pp_device_status(int reset) { return pp::read_device_status(reset != 0); }

int pp_test_bounded_wait(long long limit_cycles, void* stream) {
    pp::g_err.clear();
    if (limit_cycles < 1 || limit_cycles > (1LL << 31))
        return pp::fail(PP_ERR_UNSUPPORTED, "limit_cycles %lld outside [1, 2^31]", limit_cycles);
    const cudaError_t e = pp::launch_bounded_wait_probe(limit_cycles, (cudaStream_t)stream);
    return e == cudaSuccess ? PP_OK : pp::cuda_fail(e, "bounded-wait probe launch");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Compatibility layer (host pointers, reference CPU signatures)
// ---------------------------------------------------------------------------
namespace {

// Per-thread device workspace of the host-pointer layer: a grow-only buffer and
// three streams (host-to-device copies, kernels, device-to-host copies) with
// per-slab events, so the copies of one slab overlap the kernels of another.
constexpr int kSlabs = 8;
struct HostWorkspace {
    int device = -1;
    cudaStream_t stream = nullptr;   // kernels
    cudaStream_t h2d = nullptr;
    cudaStream_t d2h = nullptr;
    cudaEvent_t in_ready = nullptr;          // inputs shared by every slab are on the device
    cudaEvent_t slab_in[kSlabs] = {};        // slab inputs copied
    cudaEvent_t slab_out[kSlabs] = {};       // slab computed
    void* buf = nullptr;
    size_t cap = 0;
    void release() {
        if (buf) cudaFree(buf);
        for (cudaStream_t* st : {&stream, &h2d, &d2h})
            if (*st) cudaStreamDestroy(*st);
        if (in_ready) cudaEventDestroy(in_ready);
        for (int k = 0; k < kSlabs; ++k) {
            if (slab_in[k]) cudaEventDestroy(slab_in[k]);
            if (slab_out[k]) cudaEventDestroy(slab_out[k]);
            slab_in[k] = slab_out[k] = nullptr;
        }
        buf = nullptr;
        cap = 0;
        stream = h2d = d2h = nullptr;
        in_ready = nullptr;
    }
    ~HostWorkspace() { release(); }
    int reserve(size_t bytes) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return pp::cuda_fail(e, "cudaGetDevice");
        if (dev != device) {
            release();
            device = dev;
            for (cudaStream_t* st : {&stream, &h2d, &d2h})
                if ((e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking)) != cudaSuccess)
                    return pp::cuda_fail(e, "cudaStreamCreate");
            if ((e = cudaEventCreateWithFlags(&in_ready, cudaEventDisableTiming)) != cudaSuccess)
                return pp::cuda_fail(e, "cudaEventCreate");
            for (int k = 0; k < kSlabs; ++k)
                if ((e = cudaEventCreateWithFlags(&slab_in[k], cudaEventDisableTiming)) != cudaSuccess ||
                    (e = cudaEventCreateWithFlags(&slab_out[k], cudaEventDisableTiming)) != cudaSuccess)
                    return pp::cuda_fail(e, "cudaEventCreate");
        }
        if (bytes > cap) {
            if (buf) cudaFree(buf);
            buf = nullptr;
            cap = 0;
            e = cudaMalloc(&buf, bytes);
            if (e != cudaSuccess) return pp::cuda_fail(e, "cudaMalloc workspace");
            cap = bytes;
        }
        return PP_OK;
    }
};
thread_local HostWorkspace g_ws;

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

void report(const char* fn, int rc) {
    if (rc != PP_OK) std::fprintf(stderr, "pushpull_gb300: %s failed (%d): %s\n", fn, rc, pp_last_error());
}

// The host ABI passes the samples as a flat list of n1 voxels.  Each voxel is
// computed independently, so any grid shape with n1 voxels gives the same
// result; the shape only decides how voxels are grouped into tiles.  Samples on
// the image grid (the usual case) are given that grid's shape so the tiled
// kernels apply; otherwise the largest image-like factorisation is used.
void infer_sample_grid(const pp_usize* d0, pp_usize n1, pp_usize d1[3]) {
    const pp_usize plane = d0[0] * d0[1];
    if (plane > 0 && n1 % plane == 0) {
        d1[0] = d0[0];
        d1[1] = d0[1];
        d1[2] = n1 / plane;
    } else if (d0[0] > 0 && n1 % d0[0] == 0) {
        d1[0] = d0[0];
        d1[1] = n1 / d0[0];
        d1[2] = 1;
    } else {
        d1[0] = n1;
        d1[1] = d1[2] = 1;
    }
}

// z-slab boundaries zb[0..n] of a sample grid of `planes` z-planes of `plane`
// voxels; returns n <= kSlabs.  Large slabs hold at least 1 Mi voxels; the last
// ones halve down to about an eighth of a large slab, because computing a plane
// takes less time than copying its inputs in, so only the last (small) slab's
// kernels, and for the pull family its copy back, remain after the last input
// has arrived.  Grids under 2 Mi voxels are one slab.
int slab_bounds(pp_usize planes, pp_usize plane, pp_usize* zb) {
    zb[0] = 0;
    const pp_usize min_planes = plane ? ((1u << 20) + plane - 1) / plane : planes;
    if (planes < 2 || planes * plane < (2u << 20)) {
        zb[1] = planes;
        return 1;
    }
    pp_usize big = (planes + kSlabs - 4) / (kSlabs - 3);
    if (big < min_planes) big = min_planes;
    pp_usize size[kSlabs];
    int n = 0;
    pp_usize sum = 0, t = big / 8 ? big / 8 : 1;
    while (sum < planes && n < kSlabs) {   // from the back: t, 2t, 4t, ... up to big
        pp_usize sz = t < big ? t : big;
        if (n == kSlabs - 1 || sz > planes - sum) sz = planes - sum;
        size[n++] = sz;
        sum += sz;
        t *= 2;
    }
    for (int k = 0; k < n; ++k) zb[k + 1] = zb[k] + size[n - 1 - k];
    return n;
}

// kind: 0 pull, 1 pullg, 2 pullh, 3 push, 4 pushg.  The sample grid is cut into
// up to kSlabs z-slabs: slab k's inputs are copied (h2d stream) while slab k-1
// is computed (kernel stream) and slab k-2's results are copied back (d2h
// stream).  Every copy is one cudaMemcpyAsync of a contiguous range.
int compat_call(int kind, float* out, const float* phi, const float* in, const pp_usize* d0, pp_usize n1,
                const int* bnd, const pp_usize* dp, int ext) {
    if (!d0 || !bnd || !dp) return pp::fail(PP_ERR_NULL, "d0, bnd and dp must not be NULL");
    int deg[3], b[3];
    for (int k = 0; k < 3; ++k) {
        if (dp[k] < 1 || dp[k] > 5) return pp::fail(PP_ERR_DEGREE, "dp[%d] = %llu outside 1..5", k, dp[k]);
        deg[k] = (int)dp[k] - 1;
        b[k] = (bnd[k] >= 0 && bnd[k] <= 2) ? bnd[k] : 1;   // other codes act as reflect (patch.cu:55-57)
    }
    if (n1 == 0) return PP_OK;
    if (!out || !phi || !in) return pp::fail(PP_ERR_NULL, "data pointers must not be NULL");
    const pp_usize n0 = d0[0] * d0[1] * d0[2];
    pp_usize d1[3];
    infer_sample_grid(d0, n1, d1);
    const bool is_push = kind >= 3;
    const size_t comps_in = kind == 4 ? 3 : 1;
    const size_t comps_out = kind == 1 ? 3 : (kind == 2 ? 9 : 1);
    const size_t phi_b = (size_t)n1 * 3 * sizeof(float);
    const size_t in_b = (is_push ? (size_t)n1 * comps_in : (size_t)n0) * sizeof(float);
    const size_t out_b = (is_push ? (size_t)n0 : (size_t)n1 * comps_out) * sizeof(float);
    int rc = g_ws.reserve(round256(phi_b) + round256(in_b) + round256(out_b));
    if (rc != PP_OK) return rc;
    char* base = (char*)g_ws.buf;
    float* dphi = (float*)base;
    float* din = (float*)(base + round256(phi_b));
    float* dout = (float*)(base + round256(phi_b) + round256(in_b));
    HostWorkspace& w = g_ws;
    cudaError_t e;
    // inputs every slab needs: the image (pull family) or the accumulator (push family)
    if (is_push) e = cudaMemcpyAsync(dout, out, out_b, cudaMemcpyHostToDevice, w.h2d);
    else e = cudaMemcpyAsync(din, in, in_b, cudaMemcpyHostToDevice, w.h2d);
    if (e != cudaSuccess) return pp::cuda_fail(e, "copy shared input");
    if ((e = cudaEventRecord(w.in_ready, w.h2d)) != cudaSuccess) return pp::cuda_fail(e, "event");
    if ((e = cudaStreamWaitEvent(w.stream, w.in_ready, 0)) != cudaSuccess) return pp::cuda_fail(e, "wait");
    // slabs of whole z-planes
    const pp_usize plane = d1[0] * d1[1];
    pp_usize zb[kSlabs + 1];
    const int nslab = slab_bounds(d1[2], plane, zb);
    for (int k = 0; k < nslab; ++k) {
        const pp_usize z0 = zb[k], z1 = zb[k + 1];
        const pp_usize off = z0 * plane, ns = (z1 - z0) * plane;
        if (ns == 0) continue;
        // slab inputs, compact: phi (ns, 3) at dphi + 3 off; push values (ns, comps) at din + comps off
        float* sphi = dphi + 3 * off;
        for (int c = 0; c < 3; ++c)
            if ((e = cudaMemcpyAsync(sphi + c * ns, phi + c * n1 + off, ns * sizeof(float), cudaMemcpyHostToDevice,
                                     w.h2d)) != cudaSuccess)
                return pp::cuda_fail(e, "copy phi slab");
        float* sin = is_push ? din + comps_in * off : din;
        if (is_push)
            for (size_t c = 0; c < comps_in; ++c)
                if ((e = cudaMemcpyAsync(sin + c * ns, in + c * n1 + off, ns * sizeof(float),
                                         cudaMemcpyHostToDevice, w.h2d)) != cudaSuccess)
                    return pp::cuda_fail(e, "copy value slab");
        if ((e = cudaEventRecord(w.slab_in[k], w.h2d)) != cudaSuccess) return pp::cuda_fail(e, "event");
        if ((e = cudaStreamWaitEvent(w.stream, w.slab_in[k], 0)) != cudaSuccess) return pp::cuda_fail(e, "wait");
        const pp_usize sd1[3] = {d1[0], d1[1], z1 - z0};
        float* sout = is_push ? dout : dout + comps_out * off;
        switch (kind) {
            case 0: rc = pp_pull(sout, sphi, din, d0, sd1, 1, 1, b, 1, deg, ext, w.stream); break;
            case 1: rc = pp_pull_grad(sout, sphi, din, d0, sd1, 1, 1, b, 1, deg, ext, w.stream); break;
            case 2: rc = pp_pull_hess(sout, sphi, din, d0, sd1, 1, 1, b, 1, deg, ext, w.stream); break;
            case 3: rc = pp_push(sout, sphi, sin, d0, sd1, 1, 1, b, 1, deg, ext, 1, w.stream); break;
            default: rc = pp_push_grad(sout, sphi, sin, d0, sd1, 1, 1, b, 1, deg, ext, 1, w.stream); break;
        }
        if (rc != PP_OK) {
            for (cudaStream_t st : {w.h2d, w.stream, w.d2h}) cudaStreamSynchronize(st);
            return rc;
        }
        if (!is_push) {
            if ((e = cudaEventRecord(w.slab_out[k], w.stream)) != cudaSuccess) return pp::cuda_fail(e, "event");
            if ((e = cudaStreamWaitEvent(w.d2h, w.slab_out[k], 0)) != cudaSuccess) return pp::cuda_fail(e, "wait");
            for (size_t c = 0; c < comps_out; ++c)
                if ((e = cudaMemcpyAsync(out + c * n1 + off, sout + c * ns, ns * sizeof(float),
                                         cudaMemcpyDeviceToHost, w.d2h)) != cudaSuccess)
                    return pp::cuda_fail(e, "copy result slab");
        }
    }
    if (is_push) {
        if ((e = cudaEventRecord(w.slab_out[0], w.stream)) != cudaSuccess) return pp::cuda_fail(e, "event");
        if ((e = cudaStreamWaitEvent(w.d2h, w.slab_out[0], 0)) != cudaSuccess) return pp::cuda_fail(e, "wait");
        if ((e = cudaMemcpyAsync(out, dout, out_b, cudaMemcpyDeviceToHost, w.d2h)) != cudaSuccess)
            return pp::cuda_fail(e, "copy result");
    }
    for (cudaStream_t st : {w.h2d, w.stream, w.d2h})
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return pp::cuda_fail(e, "synchronize");
    return PP_OK;
}

// pull_affine / push_affine on host pointers: one (channel, batch) slice, Aff
// already 0-based (artifacts/C/pushpull.c:176-243)
int compat_affine(bool push, float* out, const float* in, const pp_usize* d0, pp_usize n1, const pp_usize* d1,
                  const float* Aff, const int* bnd, const pp_usize* dp, int ext) {
    if (!d0 || !d1 || !bnd || !dp || !Aff) return pp::fail(PP_ERR_NULL, "d0, d1, Aff, bnd and dp must not be NULL");
    int deg[3], b[3];
    for (int k = 0; k < 3; ++k) {
        if (dp[k] < 1 || dp[k] > 5) return pp::fail(PP_ERR_DEGREE, "dp[%d] = %llu outside 1..5", k, dp[k]);
        deg[k] = (int)dp[k] - 1;
        b[k] = (bnd[k] >= 0 && bnd[k] <= 2) ? bnd[k] : 1;
    }
    if (n1 != d1[0] * d1[1] * d1[2]) return pp::fail(PP_ERR_DIMS, "n1 must equal d1[0]*d1[1]*d1[2]");
    if (n1 == 0) return PP_OK;
    const pp_usize n0 = d0[0] * d0[1] * d0[2];
    const size_t in_b = (push ? (size_t)n1 : (size_t)n0) * sizeof(float);
    const size_t out_b = (push ? (size_t)n0 : (size_t)n1) * sizeof(float);
    int rc = g_ws.reserve(round256(in_b) + round256(out_b));
    if (rc != PP_OK) return rc;
    float* din = (float*)g_ws.buf;
    float* dout = (float*)((char*)g_ws.buf + round256(in_b));
    cudaStream_t s = g_ws.stream;   // the affine calls run on the kernel stream alone
    cudaError_t e;
    if ((e = cudaMemcpyAsync(din, in, in_b, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return pp::cuda_fail(e, "copy input");
    if (push && (e = cudaMemcpyAsync(dout, out, out_b, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return pp::cuda_fail(e, "copy accumulator");
    rc = push ? pp_push_affine(dout, din, Aff, d0, d1, 1, 1, b, 1, deg, ext, 1, s)
              : pp_pull_affine(dout, din, Aff, d0, d1, 1, 1, b, 1, deg, ext, s);
    if (rc != PP_OK) {
        cudaStreamSynchronize(s);
        return rc;
    }
    if ((e = cudaMemcpyAsync(out, dout, out_b, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return pp::cuda_fail(e, "copy result");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return pp::cuda_fail(e, "synchronize");
    return PP_OK;
}

}  // namespace

extern "C" {

void pull(float* f1, const float* phi, const float* f0, const pp_usize* d0, const pp_usize n1, const int* bnd,
          const pp_usize* dp, const int ext) {
    report("pull", compat_call(0, f1, phi, f0, d0, n1, bnd, dp, ext));
}

void pullg(float* g1, const float* phi, const float* f0, const pp_usize* d0, const pp_usize n1, const int* bnd,
           const pp_usize* dp, const int ext) {
    report("pullg", compat_call(1, g1, phi, f0, d0, n1, bnd, dp, ext));
}

void pullh(float* h1, const float* phi, const float* f0, const pp_usize* d0, const pp_usize n1, const int* bnd,
           const pp_usize* dp, const int ext) {
    report("pullh", compat_call(2, h1, phi, f0, d0, n1, bnd, dp, ext));
}

void push(float* f0, const float* phi, const float* f1, const pp_usize* d0, const pp_usize n1, const int* bnd,
          const pp_usize* dp, const int ext) {
    report("push", compat_call(3, f0, phi, f1, d0, n1, bnd, dp, ext));
}

void pushg(float* g0, const float* phi, const float* g1, const pp_usize* d0, const pp_usize n1, const int* bnd,
           const pp_usize* dp, const int ext) {
    report("pushg", compat_call(4, g0, phi, g1, d0, n1, bnd, dp, ext));
}

void pull_affine(float* f1, const float* f0, const pp_usize* d0, const pp_usize n1, const pp_usize* d1,
                 const float* Aff, const int* bnd, const pp_usize* dp, const int ext) {
    report("pull_affine", compat_affine(false, f1, f0, d0, n1, d1, Aff, bnd, dp, ext));
}

void push_affine(float* f0, const float* f1, const pp_usize* d0, const pp_usize n1, const pp_usize* d1,
                 const float* Aff, const int* bnd, const pp_usize* dp, const int ext) {
    report("push_affine", compat_affine(true, f0, f1, d0, n1, d1, Aff, bnd, dp, ext));
}

}  // extern "C"
