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

// ---- tile configuration registry (per op, per isotropic degree) and path choice
namespace {
std::mutex g_cfg_mu;
TileCfg g_tiles[5][5];
bool g_tiles_init = false;
int g_path = PP_PATH_AUTO;

void init_tiles_locked() {
    if (g_tiles_init) return;
    // 8x8x8 tiles; the push family keeps two words per accumulator element
    for (int op = 0; op < 5; ++op)
        for (int d = 0; d < 5; ++d) g_tiles[op][d] = TileCfg{3, 3, 3, op < 3 ? 8192 : 12288};
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
        volatile float dk = (float)g.d0[k];   // float arithmetic, as artifacts/C/pushpull.c:8-10
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

static int run_pull(int op, float* out, const float* phi, const float* f0, const pp_usize d0[3],
                    const pp_usize d1[3], int nc, int nb, const int* bnd, int nbnd, const int deg[3],
                    int ext, void* stream) {
    LaunchArgs a{};
    int rc = prepare(a, out, phi, f0, d0, d1, nc, nb, bnd, nbnd, deg, ext);
    if (rc != PP_OK || a.g.n1 == 0) return rc;
    const TileCfg t = tile_for(op, deg[0]);
    cudaError_t e;
    if (current_path() != PP_PATH_DIRECT && tiled_supported(a, t))
        e = launch_pull_tiled(op, a, t, (cudaStream_t)stream);
    else
        e = launch_pull_direct(op, a, (cudaStream_t)stream);
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

}  // namespace pp

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

int pp_push(float* f0, const float* phi, const float* f1, const pp_usize d0[3], const pp_usize d1[3], int nc,
            int nb, const int* bnd, int nbnd, const int deg[3], int ext, int accumulate, void* stream) {
    return run_push(pp::kPush, f0, phi, f1, d0, d1, nc, nb, bnd, nbnd, deg, ext, accumulate, stream);
}

int pp_push_grad(float* g0, const float* phi, const float* g1, const pp_usize d0[3], const pp_usize d1[3], int nc,
                 int nb, const int* bnd, int nbnd, const int deg[3], int ext, int accumulate, void* stream) {
    return run_push(pp::kPushGrad, g0, phi, g1, d0, d1, nc, nb, bnd, nbnd, deg, ext, accumulate, stream);
}

const char* pp_last_error(void) { return pp::g_err.c_str(); }

int pp_set_tile(int op, int deg, int lx, int ly, int lz, int cap_floats) {
    pp::g_err.clear();
    if (op < -1 || op > 4) return pp::fail(PP_ERR_UNSUPPORTED, "op %d outside -1..4", op);
    if (deg < -1 || deg > 4) return pp::fail(PP_ERR_DEGREE, "deg %d outside -1..4", deg);
    if (lx < 0 || ly < 0 || lz < 0 || lx + ly + lz < 5 || lx + ly + lz > 9)
        return pp::fail(PP_ERR_UNSUPPORTED, "tile 2^%d x 2^%d x 2^%d must hold 32..512 voxels", lx, ly, lz);
    if (cap_floats < 64 || (cap_floats & 3) || cap_floats > (227 * 1024) / 4)
        return pp::fail(PP_ERR_UNSUPPORTED, "cap %d floats must be a multiple of 4 in [64, 58112]", cap_floats);
    std::lock_guard<std::mutex> lk(pp::g_cfg_mu);
    pp::init_tiles_locked();
    for (int o = 0; o < 5; ++o)
        for (int d = 0; d < 5; ++d)
            if ((op < 0 || o == op) && (deg < 0 || d == deg)) pp::g_tiles[o][d] = pp::TileCfg{lx, ly, lz, cap_floats};
    return PP_OK;
}

int pp_get_tile(int op, int deg, int* lx, int* ly, int* lz, int* cap_floats) {
    if (op < 0 || op > 4 || deg < 0 || deg > 4) return pp::fail(PP_ERR_UNSUPPORTED, "op/deg out of range");
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

unsigned pp_device_status(int reset) { return pp::read_device_status(reset != 0); }

}  // extern "C"

// ---------------------------------------------------------------------------
// Compatibility layer (host pointers, reference CPU signatures)
// ---------------------------------------------------------------------------
namespace {

struct HostWorkspace {
    int device = -1;
    cudaStream_t stream = nullptr;
    void* buf = nullptr;
    size_t cap = 0;
    ~HostWorkspace() {
        if (buf) cudaFree(buf);
        if (stream) cudaStreamDestroy(stream);
    }
    int reserve(size_t bytes) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return pp::cuda_fail(e, "cudaGetDevice");
        if (dev != device) {
            if (buf) cudaFree(buf);
            if (stream) cudaStreamDestroy(stream);
            buf = nullptr;
            cap = 0;
            stream = nullptr;
            device = dev;
            e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
            if (e != cudaSuccess) return pp::cuda_fail(e, "cudaStreamCreate");
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

// kind: 0 pull, 1 pullg, 2 pullh, 3 push, 4 pushg
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
    const pp_usize n0 = d0[0] * d0[1] * d0[2];
    const pp_usize d1[3] = {n1, 1, 1};
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
    cudaStream_t s = g_ws.stream;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(dphi, phi, phi_b, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return pp::cuda_fail(e, "copy phi");
    if ((e = cudaMemcpyAsync(din, in, in_b, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return pp::cuda_fail(e, "copy input");
    if (is_push && (e = cudaMemcpyAsync(dout, out, out_b, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return pp::cuda_fail(e, "copy accumulator");
    switch (kind) {
        case 0: rc = pp_pull(dout, dphi, din, d0, d1, 1, 1, b, 1, deg, ext, s); break;
        case 1: rc = pp_pull_grad(dout, dphi, din, d0, d1, 1, 1, b, 1, deg, ext, s); break;
        case 2: rc = pp_pull_hess(dout, dphi, din, d0, d1, 1, 1, b, 1, deg, ext, s); break;
        case 3: rc = pp_push(dout, dphi, din, d0, d1, 1, 1, b, 1, deg, ext, 1, s); break;
        default: rc = pp_push_grad(dout, dphi, din, d0, d1, 1, 1, b, 1, deg, ext, 1, s); break;
    }
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

}  // extern "C"
