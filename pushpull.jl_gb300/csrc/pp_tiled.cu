// pp_tiled.cu -- host side of the tiled kernels: support test, grid shape, dispatch to the
// per-group translation units and the combined device status
// (kernels and helpers: pp_tiled_impl.cuh).
#include "pp_tiled_impl.cuh"

namespace pp {

cudaError_t launch_tiled_pull_basic(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s);
cudaError_t launch_tiled_pull_hess(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s);
cudaError_t launch_tiled_pull_dot(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s);
cudaError_t launch_tiled_push(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s);
cudaError_t launch_tiled_push_grad(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s);
unsigned status_pull_basic(bool reset);
unsigned status_pull_hess(bool reset);
unsigned status_pull_dot(bool reset);
unsigned status_push(bool reset);
unsigned status_push_grad(bool reset);
unsigned status_fused(bool reset);
unsigned status_batch(bool reset);
unsigned status_ws_pull(bool reset);
unsigned status_ws_hess(bool reset);
unsigned status_ws_grad_dot(bool reset);
unsigned status_ws_hess_dot(bool reset);
unsigned status_push_affine(bool reset);

bool tiled_supported(const LaunchArgs& a, const TileCfg& t) {
    const Geometry& g = a.g;
    const int vox = 1 << (t.lx + t.ly + t.lz);
    if (!(g.dp[0] == g.dp[1] && g.dp[1] == g.dp[2])) return false;
    // whole tiles of 256 or 512 voxels: every thread owns one voxel slot per V
    if (!(vox == kThreads || vox == 2 * kThreads) || t.cap < 64 || (t.cap & 3) || t.cap > 24 * 1024) return false;
    // a tile must be mostly inside the sample grid: degenerate grids (e.g. a
    // flat list of n1 samples) are better served by the per-voxel kernels
    for (int k = 0; k < 3; ++k) {
        const int l = k == 0 ? t.lx : (k == 1 ? t.ly : t.lz);
        if (2 * g.d1[k] < (1LL << l)) return false;
    }
    const long long ntx = (g.d1[0] + (1 << t.lx) - 1) >> t.lx;
    const long long nty = (g.d1[1] + (1 << t.ly) - 1) >> t.ly;
    const long long ntz = (g.d1[2] + (1 << t.lz) - 1) >> t.lz;
    return ntx * nty * ntz * g.nb < 0x7fffffffLL;
}

cudaError_t launch_pull_tiled(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s) {
    switch (op) {
        case kPull:
        case kPullGrad: return launch_tiled_pull_basic(op, a, t, s);
        case kPullHess: return launch_tiled_pull_hess(op, a, t, s);
        default: return launch_tiled_pull_dot(op, a, t, s);
    }
}

cudaError_t launch_push_tiled(int op, const LaunchArgs& a, const TileCfg& t, cudaStream_t s) {
    return op == kPush ? launch_tiled_push(op, a, t, s) : launch_tiled_push_grad(op, a, t, s);
}

int fused_tiled_grid(const LaunchArgs& a, const TileCfg& c) {
    const TileGrid t = make_grid(a, c);
    // every CTA resident at once: as many per SM as the shared memory (ring,
    // two box buffers, two-word accumulator) admits, at most what the kernel's
    // register budget allows (three up to degree 2, two above)
    const int nv = (1 << (c.lx + c.ly + c.lz)) > kThreads ? 2 * kThreads : kThreads;
    const long long smem = (long long)kStages * 4 * nv * 4 + 4LL * c.cap * 4 + 8 * kStages + 1024;
    const long long reg_cap = a.g.dp[0] <= 3 ? 3 : 2;
    long long per_sm = (228LL * 1024) / smem;
    per_sm = per_sm < 1 ? 1 : (per_sm > reg_cap ? reg_cap : per_sm);
    const long long want = per_sm * sm_count();
    return (int)(t.ntiles < want ? t.ntiles : want);
}

TileGrid tile_grid(const LaunchArgs& a, const TileCfg& c) { return make_grid(a, c); }

namespace {
// One warp waits on an mbarrier that no copy or thread will ever complete, with
// a caller-given cycle limit: the bounded wait gives up, records the timeout in
// this unit's status word and the kernel returns normally.
__global__ void k_bounded_wait_probe(long long limit) {
    __shared__ __align__(8) unsigned long long bar;
    const unsigned a = smem_addr(&bar);
    if (threadIdx.x == 0) {
        mbar_init(a, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    mbar_wait_limit(a, 0u, limit);
    __syncwarp();
    if (threadIdx.x == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(a) : "memory");
}
}  // namespace

cudaError_t launch_bounded_wait_probe(long long limit_cycles, cudaStream_t s) {
    k_bounded_wait_probe<<<1, 32, 0, s>>>(limit_cycles);
    return cudaGetLastError();
}

unsigned read_device_status(bool reset) {
    unsigned v = status_pull_basic(reset);
    v |= status_pull_hess(reset);
    v |= status_pull_dot(reset);
    v |= status_push(reset);
    v |= status_push_grad(reset);
    v |= status_fused(reset);
    v |= status_batch(reset);
    v |= status_ws_pull(reset);
    v |= status_ws_hess(reset);
    v |= status_ws_grad_dot(reset);
    v |= status_ws_hess_dot(reset);
    v |= status_push_affine(reset);
    v |= unit_status(reset);   // the bounded-wait probe of this unit
    return v;
}

}  // namespace pp
