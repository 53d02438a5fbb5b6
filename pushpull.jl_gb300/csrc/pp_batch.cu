// pp_batch.cu -- plans for the batched uneven workload: many (image, deformation)
// pairs of different sizes, channel counts and degrees -- e.g. registration
// pairs together with their multigrid pyramid levels -- pulled and pushed back
// in one persistent launch, optionally replayed from a CUDA graph.
//
// The reference processes each array with its own host loop and one launch
// per (channel, batch) (ext/pushpull_gpu.jl:37-49); the multigrid code calls
// pull/push once per level (src/multigrid.jl:21-55).
#include <cstring>
#include <new>
#include <vector>

#include "pp_tiled.cuh"
#include "pushpull_gb300.h"

namespace pp {
int fail_status(int code, const char* fmt, ...);
int prepare_args(LaunchArgs& a, float* out, const float* phi, const float* in, const pp_usize d0[3],
                 const pp_usize d1[3], int nc, int nb, const int* bnd, int nbnd, const int deg[3], int ext);
TileCfg tile_for(int op_index, int deg);
}  // namespace pp

// Shared-memory budget of the batched kernel, in floats: three words per box
// element (two accumulator words, one image word).
constexpr int kBatchCap = 24576;

struct pp_batch {
    int device = -1;
    std::vector<pp::BatchItem> items;
    pp::BatchItem* dev_items = nullptr;
    unsigned* counter = nullptr;
    int total = 0;
    int cap = kBatchCap;
    bool zero_outputs = false;
    std::vector<std::pair<float*, size_t>> outputs;   // (pointer, bytes) zeroed before each run
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// a 512-voxel tile shape that fits the sample grid (first fit, cubic first)
pp::TileCfg batch_tile_for(const pp_usize d1[3], int deg) {
    const pp::TileCfg pref = pp::tile_for(PP_OP_PULL, deg);
    const int shapes[][3] = {{pref.lx, pref.ly, pref.lz}, {3, 3, 3}, {4, 3, 2}, {4, 2, 3}, {5, 2, 2}, {3, 4, 2},
                             {4, 4, 1}, {5, 3, 1}, {5, 4, 0}, {4, 5, 0}};
    for (const auto& sh : shapes) {
        if (sh[0] + sh[1] + sh[2] != 9) continue;
        bool ok = true;
        for (int k = 0; k < 3; ++k) ok = ok && 2 * (long long)d1[k] >= (1LL << sh[k]);
        if (ok) return pp::TileCfg{sh[0], sh[1], sh[2], 0};
    }
    return pp::TileCfg{5, 4, 0, 0};
}

int run_plan(pp_batch* p, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(p->counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return pp::fail_status(PP_ERR_CUDA, "reset work counter: %s", cudaGetErrorString(e));
    if (p->zero_outputs)
        for (const auto& o : p->outputs)
            if ((e = cudaMemsetAsync(o.first, 0, o.second, s)) != cudaSuccess)
                return pp::fail_status(PP_ERR_CUDA, "zero outputs: %s", cudaGetErrorString(e));
    e = pp::launch_batch(p->dev_items, (int)p->items.size(), p->total, p->counter, p->cap, s);
    if (e != cudaSuccess) return pp::fail_status(PP_ERR_CUDA, "batch launch: %s", cudaGetErrorString(e));
    return PP_OK;
}

}  // namespace

extern "C" {

int pp_batch_create(pp_batch** plan, const pp_batch_item* items, int n, int zero_outputs) {
    if (!plan || (!items && n > 0)) return pp::fail_status(PP_ERR_NULL, "plan and items must not be NULL");
    if (n < 0) return pp::fail_status(PP_ERR_DIMS, "negative item count");
    *plan = nullptr;
    pp_batch* p = new (std::nothrow) pp_batch;
    if (!p) return pp::fail_status(PP_ERR_TOO_LARGE, "out of host memory");
    p->zero_outputs = zero_outputs != 0;
    cudaGetDevice(&p->device);
    long long total = 0;
    for (int i = 0; i < n; ++i) {
        const pp_batch_item& it = items[i];
        const bool per_dim = it.deg == -1;
        const int deg[3] = {per_dim ? it.deg3[0] : it.deg, per_dim ? it.deg3[1] : it.deg,
                            per_dim ? it.deg3[2] : it.deg};
        const bool per_chan = it.nbnd > 1;
        if (per_chan && !it.bnds) {
            delete p;
            return pp::fail_status(PP_ERR_NULL, "batch item %d: nbnd > 1 needs bnds", i);
        }
        const int* bnd = per_chan ? it.bnds : it.bnd;
        const int nbnd = per_chan ? it.nbnd : 1;
        pp::BatchItem bi;
        std::memset(&bi, 0, sizeof bi);
        int rc = pp::prepare_args(bi.pull, it.f1, it.phi, it.f0, it.d0, it.d1, it.nc, 1, bnd, nbnd, deg, it.ext);
        if (rc == PP_OK)
            rc = pp::prepare_args(bi.push, it.out, it.phi, it.f1, it.d0, it.d1, it.nc, 1, bnd, nbnd, deg, it.ext);
        if (rc != PP_OK) {
            delete p;
            return rc;
        }
        if (bi.pull.g.n1 == 0) continue;
        if (bi.pull.g.n0 >= (1LL << 31) - 1 || bi.pull.g.n1 >= (1LL << 31) - 1) {
            delete p;
            return pp::fail_status(PP_ERR_TOO_LARGE, "batch item %d exceeds 2^31 voxels", i);
        }
        const bool iso = deg[0] == deg[1] && deg[1] == deg[2];
        const pp::TileCfg tc = batch_tile_for(it.d1, deg[0]);
        bi.t = pp::tile_grid(bi.pull, tc);
        // the push registry entry of the degree sets the box budget (two words per
        // element there, three here), within the kernel's fixed budget
        const pp::TileCfg pc = pp::tile_for(PP_OP_PUSH, deg[0]);
        const long long want = pc.cap > 0 ? (3LL * pc.cap / 2) & ~3LL : p->cap;
        bi.t.cap = (int)(want < 64 ? 64 : (want > p->cap ? p->cap : want));
        // anisotropic degrees: the per-voxel path of the batched kernel (dp 0)
        bi.dp = iso ? deg[0] + 1 : 0;
        bi.tile_begin = (int)total;
        total += (long long)bi.t.ntiles;
        if (total >= (1LL << 31) - 1) {
            delete p;
            return pp::fail_status(PP_ERR_TOO_LARGE, "batch exceeds 2^31 tiles");
        }
        p->items.push_back(bi);
        p->outputs.emplace_back(it.out, (size_t)bi.pull.g.n0 * it.nc * sizeof(float));
    }
    p->total = (int)total;
    cudaError_t e = cudaSuccess;
    if (!p->items.empty()) {
        e = cudaMalloc(&p->dev_items, p->items.size() * sizeof(pp::BatchItem));
        if (e == cudaSuccess)
            e = cudaMemcpy(p->dev_items, p->items.data(), p->items.size() * sizeof(pp::BatchItem),
                           cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMalloc(&p->counter, sizeof(unsigned));
    if (e != cudaSuccess) {
        pp_batch_destroy(p);
        return pp::fail_status(PP_ERR_CUDA, "batch plan upload: %s", cudaGetErrorString(e));
    }
    *plan = p;
    return PP_OK;
}

int pp_batch_tiles(const pp_batch* plan) { return plan ? plan->total : -1; }

int pp_batch_run(pp_batch* plan, void* stream) {
    if (!plan) return pp::fail_status(PP_ERR_NULL, "plan must not be NULL");
    return run_plan(plan, (cudaStream_t)stream);
}

int pp_batch_capture(pp_batch* plan, void* stream) {
    if (!plan) return pp::fail_status(PP_ERR_NULL, "plan must not be NULL");
    cudaStream_t s = (cudaStream_t)stream;
    if (!s) return pp::fail_status(PP_ERR_UNSUPPORTED, "graph capture needs a non-default stream");
    // one eager run so every one-time setup (kernel attributes) happens outside the capture
    int rc = run_plan(plan, s);
    if (rc != PP_OK) return rc;
    if (plan->exec) {
        cudaGraphExecDestroy(plan->exec);
        plan->exec = nullptr;
    }
    if (plan->graph) {
        cudaGraphDestroy(plan->graph);
        plan->graph = nullptr;
    }
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return pp::fail_status(PP_ERR_CUDA, "begin capture: %s", cudaGetErrorString(e));
    rc = run_plan(plan, s);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(s, &g);
    if (rc != PP_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return pp::fail_status(PP_ERR_CUDA, "end capture: %s", cudaGetErrorString(e));
    plan->graph = g;
    e = cudaGraphInstantiate(&plan->exec, g, 0);
    if (e != cudaSuccess) return pp::fail_status(PP_ERR_CUDA, "instantiate graph: %s", cudaGetErrorString(e));
    return PP_OK;
}

int pp_batch_launch(pp_batch* plan, void* stream) {
    if (!plan) return pp::fail_status(PP_ERR_NULL, "plan must not be NULL");
    if (!plan->exec) return pp::fail_status(PP_ERR_UNSUPPORTED, "no captured graph (call pp_batch_capture)");
    cudaError_t e = cudaGraphLaunch(plan->exec, (cudaStream_t)stream);
    if (e != cudaSuccess) return pp::fail_status(PP_ERR_CUDA, "graph launch: %s", cudaGetErrorString(e));
    return PP_OK;
}

void pp_batch_destroy(pp_batch* plan) {
    if (!plan) return;
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    if (plan->dev_items) cudaFree(plan->dev_items);
    if (plan->counter) cudaFree(plan->counter);
    delete plan;
}

}  // extern "C"
