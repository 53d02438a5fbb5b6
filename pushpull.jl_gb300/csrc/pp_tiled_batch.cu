// pp_tiled_batch.cu -- persistent batched pull + push kernel
// (kernels and helpers: pp_tiled_impl.cuh).
#define PP_TILED_BATCH
#include "pp_tiled_impl.cuh"

namespace pp {

cudaError_t launch_batch(const BatchItem* items, int nitems, int total_tiles, unsigned* counter, int cap,
                         cudaStream_t s) {
    const size_t smem = (size_t)cap * sizeof(float);
    cudaError_t e = opt_in(k_batch, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, kThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long want = (long long)sm_count() * per_sm;
    const int grid = (int)(total_tiles < want ? total_tiles : want);
    if (grid < 1) return cudaSuccess;
    k_batch<<<grid, kThreads, smem, s>>>(items, nitems, total_tiles, counter, cap);
    return cudaGetLastError();
}

unsigned status_batch(bool reset) { return unit_status(reset); }

}  // namespace pp
