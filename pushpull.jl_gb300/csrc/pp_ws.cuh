// pp_ws.cuh -- warp-specialised persistent pull family.
//
// Included after pp_tiled_impl.cuh (whose helpers it uses) by pp_ws_pull.cu.
//
// One CTA per SM: 16 consumer warps and one producer warp.  The CTA walks
// tiles of 8 x 8 x 16 sample voxels (two per consumer thread).  The producer
// warp does all per-tile bookkeeping one unit ahead of the consumers:
//   * streams each tile's deformation into a ring of shared-memory slots with
//     one TMA copy per tile (mbarrier complete_tx),
//   * reduces the tile's first taps to its footprint box in the image,
//   * stages the box of every (tile, channel) unit into one of two buffers:
//     boxes inside the image that fit a fixed 24 x 16 x 24 window arrive by one
//     TMA copy; all other boxes (boundary folding, DST-II signs) are gathered by
//     the producer warp itself, 16-byte chunks where a row is in range,
//   * publishes the box record and signals the buffer full.
// The consumers only evaluate voxels against the staged box and release the
// buffer; there is no CTA-wide barrier in the steady state, so the per-tile
// work (bounds, staging, folding) overlaps the contraction of the previous unit.
// Boxes larger than a buffer take the per-voxel global path for that tile.
//
// Reference kernels replaced: pull_element / pullg_element / pullh_element
// (artifacts/C/pushpull.cu:33-108); per-voxel math pull1 / pullg1 / pullh1
// (artifacts/C/pushpull_dev.cu:61-116).
#pragma once

#include "pp_tiled_impl.cuh"

namespace pp {
namespace {

constexpr int kWsCons = 512;                   // consumer threads (16 warps)
constexpr int kWsThreads = kWsCons + 32;       // plus the producer warp
constexpr int kWsV = 2;                        // sample voxels per consumer thread
constexpr int kWsNV = kWsCons * kWsV;          // voxels per tile: 8 x 8 x 16
constexpr int kWsLx = 3, kWsLy = 3, kWsLz = 4;
constexpr int kWsStages = 4;                   // deformation ring slots
constexpr int kWsBufs = 2;                     // box buffers
constexpr int kWsWinX = 24, kWsWinY = 16, kWsWinZ = 24;   // TMA image window (row pitch 24)
constexpr int kWsCap = kWsWinX * kWsWinY * kWsWinZ;         // floats per box buffer
constexpr size_t kWsSmem = (size_t)(kWsStages * 3 * kWsNV + kWsBufs * kWsCap) * sizeof(float);

__device__ __forceinline__ void mbar_arrive(unsigned bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Tile-local voxel lin (x fastest, 8 x 8 x 16) -> linear sample index, or -1.
template <typename IT>
__device__ __forceinline__ IT ws_index(const TileOrigin& o, int lin, int D0, int D1, int D2) {
    const int gx = o.x0 + (lin & 7), gy = o.y0 + ((lin >> 3) & 7), gz = o.z0 + (lin >> 6);
    if (gx >= D0 || gy >= D1 || gz >= D2) return (IT)-1;
    return (IT)gx + (IT)D0 * ((IT)gy + (IT)D1 * (IT)gz);
}

// Footprint box of the tile in `slot`, computed by the producer warp (every
// lane ends with the same record).  win_ok: interior boxes may use the TMA window.
template <int DP, typename IT>
__device__ __forceinline__ Box ws_tile_box(const Geometry& g, const TileOrigin& o, const float* slot, int D0, int D1,
                                           int D2, bool win_ok, int lane) {
    int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
#pragma unroll 4
    for (int i = lane; i < kWsNV; i += 32) {
        if (ws_index<IT>(o, i, D0, D1, D2) < 0) continue;
        float x[3];
        if (!load_valid(slot[i], slot[kWsNV + i], slot[2 * kWsNV + i], g, x[0], x[1], x[2])) continue;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int f = first_tap32(x[k], DP);
            const int c = f < -kClamp ? -kClamp : (f > kClamp ? kClamp : f);
            mn[k] = min(mn[k], c);
            mx[k] = max(mx[k], c);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        mn[k] = __reduce_min_sync(0xffffffffu, mn[k]);
        mx[k] = __reduce_max_sync(0xffffffffu, mx[k]);
    }
    Box box;
    box.S = 0.f;
    box.E = 0;
    box.tma = 0;
    if (mn[0] > mx[0]) {   // no valid voxel in the tile
        box.mode = 0;
        box.interior = 0;
        box.xo = box.lo[0] = box.lo[1] = box.lo[2] = 0;
        box.ext[0] = box.ext[1] = box.ext[2] = 0;
        box.P = box.Q = box.size = 0;
        return box;
    }
    const int xo = mn[0] & ~3;
    const long long e0 = (long long)mx[0] + DP - xo;
    const long long e1 = (long long)mx[1] + DP - mn[1];
    const long long e2 = (long long)mx[2] + DP - mn[2];
    int interior = 0;
    if (xo >= 0 && (long long)mx[0] + DP <= g.d0[0]) interior |= 1;
    if (mn[1] >= 0 && (long long)mx[1] + DP <= g.d0[1]) interior |= 2;
    if (mn[2] >= 0 && (long long)mx[2] + DP <= g.d0[2]) interior |= 4;
    box.interior = interior;
    box.xo = xo;
    box.lo[0] = mn[0];
    box.lo[1] = mn[1];
    box.lo[2] = mn[2];
    if (win_ok && interior == 7 && e0 <= kWsWinX && e1 <= kWsWinY && e2 <= kWsWinZ) {
        box.mode = 1;
        box.tma = 1;
        box.P = kWsWinX;
        box.Q = kWsWinX * kWsWinY;
        box.size = kWsCap;
        box.ext[0] = (int)e0;
        box.ext[1] = (int)e1;
        box.ext[2] = (int)e2;
        return box;
    }
    // gathered box: row pitch P % 32 == 8 keeps an 8 x 4 warp tile's rows in
    // disjoint banks; pack tightly when the padding does not fit
    long long P = (e0 + 3) & ~3LL;
    const long long Pp = P + (((8 - (int)(P & 31)) + 32) & 31);
    long long Q = (Pp * e1 + 31) & ~31LL;
    if (Q * e2 <= kWsCap) {
        P = Pp;
    } else {
        Q = (P * e1 + 3) & ~3LL;
    }
    const bool fits = e0 <= 4096 && e1 <= 4096 && e2 <= 4096 && Q * e2 <= kWsCap;
    box.mode = fits ? 1 : 2;
    box.ext[0] = fits ? (int)e0 : 0;
    box.ext[1] = fits ? (int)e1 : 0;
    box.ext[2] = fits ? (int)e2 : 0;
    box.P = fits ? (int)P : 0;
    box.Q = fits ? (int)Q : 0;
    box.size = fits ? (int)(Q * e2) : 0;
    return box;
}

// Gather one channel of a box into shared memory with the producer warp,
// folding (and signing) out-of-range taps; in-range 16-byte row chunks are one
// vector load each.  Lanes split over (row, chunk) pairs.
template <typename IT>
__device__ __forceinline__ void ws_stage_gather(const Box& box, const Geometry& g, int b0, int b1, int b2,
                                                const float* f0, float* sm, int lane) {
    const int ex = box.ext[0], ey = box.ext[1], ez = box.ext[2];
    const int n4 = (ex + 3) >> 2;
    const int nn = n4 < 1 ? 1 : (n4 > 32 ? 32 : n4);
    const int lg = 32 - __clz(nn - 1);          // lanes per row = 1 << lg
    const int lpr = 1 << lg;
    const int sub = lane >> lg, e4 = lane & (lpr - 1), step = 32 >> lg;
    const bool vec = (g.d0[0] & 3) == 0 && (reinterpret_cast<uintptr_t>(f0) & 15) == 0;
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);
    const long long dx = g.d0[0];
    const int nrows = ey * ez;
    for (int r = sub; r < nrows; r += step) {
        const int rz = r / ey, ry = r - rz * ey;
        float sgy = 1.f, sgz = 1.f;
        const IT gy = (box.interior & 2) ? (IT)(box.lo[1] + ry)
                                         : (IT)fold_tap(b1, (long long)box.lo[1] + ry, g.d0[1], sgy);
        const IT gz = (box.interior & 4) ? (IT)(box.lo[2] + rz)
                                         : (IT)fold_tap(b2, (long long)box.lo[2] + rz, g.d0[2], sgz);
        const float s = sgy * sgz;
        const float* grow = f0 + (gz * sz + gy * sy);
        float* srow = sm + (rz * box.Q + ry * box.P);
        for (int ch = e4; ch < n4; ch += lpr) {
            const long long x = (long long)box.xo + 4 * ch;
            if (vec && x >= 0 && x + 4 <= dx) {
                float4 v = __ldg(reinterpret_cast<const float4*>(grow + (IT)x));
                v.x *= s;
                v.y *= s;
                v.z *= s;
                v.w *= s;
                *reinterpret_cast<float4*>(srow + 4 * ch) = v;
            } else {
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    float sgx;
                    const IT gx = (IT)fold_tap(b0, x + u, dx, sgx);
                    srow[4 * ch + u] = s * sgx * __ldg(grow + gx);
                }
            }
        }
    }
}

// One consumer thread, one (tile, channel) unit of the pull family: its two
// voxels against the staged box (dot ops accumulate into acc and store after
// the last channel).
template <int DP, int OP_, typename IT>
__device__ __forceinline__ void ws_pull_unit(const LaunchArgs& a, const TileOrigin& o, int ctid, const float* slot,
                                             int c, const Box& box, const float* sm, float (&acc)[kWsV][3], int D0,
                                             int D1, int D2) {
    constexpr int OP = pull_base_op<OP_>();
    constexpr int NCOMP = pull_ncomp<OP_>();
    constexpr int ORD = op_order(OP);
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const bool last = c == g.nc - 1;
    auto voxel = [&](int q) {
        const int lin = ctid + q * kWsCons;
        const IT v = ws_index<IT>(o, lin, D0, D1, D2);
        if (v < 0) return;
        float x0, x1, x2;
        if (!load_valid(slot[lin], slot[kWsNV + lin], slot[2 * kWsNV + lin], g, x0, x1, x2)) {
            if (!pull_is_dot<OP_>() || last) {
                float* out = pull_out<OP_>(a, o.b, c, (long long)v);
#pragma unroll
                for (int p = 0; p < NCOMP; ++p) out[(long long)p * n1] = qnan();
            }
            return;
        }
        if (box.mode == 2) {   // box larger than a buffer: every channel from global memory, once
            if (c == 0) pull_voxel_lean<DP, OP_, IT>(a, o.b, (long long)v, x0, x1, x2);
            return;
        }
        if (box.mode != 1) return;
        W3<DP, ORD> wx, wy, wz;
        const int ox = spline_taps32<DP, ORD>(x0, wx.w, wx.dw, wx.hw) - box.xo;
        const int oy = spline_taps32<DP, ORD>(x1, wy.w, wy.dw, wy.hw) - box.lo[1];
        const int oz = spline_taps32<DP, ORD>(x2, wz.w, wz.dw, wz.hw) - box.lo[2];
        const unsigned P4 = 4u * box.P, Q4 = 4u * box.Q;
        const unsigned p = smem_addr(sm) + 4u * (unsigned)(oz * box.Q + oy * box.P + ox);
        float r[6];
        contract_smem<OP, DP>(wx, wy, wz, p, P4, Q4, r);
        if constexpr (pull_is_dot<OP_>()) {
            dot_accumulate<OP_>(a, o.b, c, (long long)v, r, acc[q]);
            if (last) {
                float* out = pull_out<OP_>(a, o.b, 0, (long long)v);
                out[0] = acc[q][0];
                out[n1] = acc[q][1];
                out[2 * n1] = acc[q][2];
            }
        } else {
            pull_store<OP>(pull_out<OP_>(a, o.b, c, (long long)v), n1, r);
        }
    };
    if constexpr (pull_is_dot<OP_>()) {
#pragma unroll
        for (int q = 0; q < kWsV; ++q) voxel(q);
    } else {
#pragma unroll 1
        for (int q = 0; q < kWsV; ++q) voxel(q);
    }
}

template <int DP, int OP, typename IT>
__global__ void __maxnreg__(120) k_pull_ws(const __grid_constant__ LaunchArgs a,
                                                           const __grid_constant__ TileGrid t,
                                                           const __grid_constant__ CUtensorMap phimap,
                                                           const __grid_constant__ CUtensorMap imgmap) {
    extern __shared__ __align__(128) float4 smem4[];
    __shared__ __align__(8) unsigned long long bars[kWsStages + 2 * kWsBufs];
    __shared__ Box rec[kWsBufs];
    __shared__ volatile int s_abort;
    const Geometry& g = a.g;
    const int G = gridDim.x;
    const int T0 = blockIdx.x;
    if (T0 >= t.ntiles) return;
    const int ntl = (t.ntiles - T0 + G - 1) / G;
    const int nc = g.nc;
    const int D0 = (int)g.d1[0], D1 = (int)g.d1[1], D2 = (int)g.d1[2];
    float* ring = reinterpret_cast<float*>(smem4);
    float* bufs = ring + kWsStages * 3 * kWsNV;
    const unsigned phi_full = smem_addr(&bars[0]);
    const unsigned box_full = smem_addr(&bars[kWsStages]);
    const unsigned box_empty = smem_addr(&bars[kWsStages + kWsBufs]);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int k = 0; k < kWsStages; ++k) mbar_init(phi_full + 8u * k, 1);
        for (int k = 0; k < kWsBufs; ++k) {
            mbar_init(box_full + 8u * k, 1);
            mbar_init(box_empty + 8u * k, kWsCons / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == kWsCons / 32) {
        // ---------------- producer warp ----------------
        auto load_phi = [&](int j) {   // lane 0: tile j's deformation into slot j % kWsStages
            if (lane == 0) {
                const TileOrigin o = tile_origin(t, T0 + j * G);
                const unsigned bar = phi_full + 8u * (j % kWsStages);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_expect_tx(bar, (unsigned)(3 * kWsNV * sizeof(float)));
                tma_load_4d(smem_addr(ring + (j % kWsStages) * 3 * kWsNV), &phimap, bar, o.x0, o.y0, o.z0, 3 * o.b);
            }
        };
        for (int j = 0; j < kWsStages && j < ntl; ++j) load_phi(j);
        for (int j = 0; j < ntl && !s_abort; ++j) {
            const TileOrigin o = tile_origin(t, T0 + j * G);
            const float* slot = ring + (j % kWsStages) * 3 * kWsNV;
            if (!mbar_wait(phi_full + 8u * (j % kWsStages), (unsigned)((j / kWsStages) & 1))) {
                s_abort = 1;
                break;
            }
            const Box box = ws_tile_box<DP, IT>(g, o, slot, D0, D1, D2, t.img_tma != 0, lane);
            for (int c = 0; c < nc; ++c) {
                const int q = j * nc + c, b = q % kWsBufs, k = q / kWsBufs;
                if (k >= 1 && !mbar_wait(box_empty + 8u * b, (unsigned)((k - 1) & 1))) {
                    s_abort = 1;
                    break;
                }
                // the consumers have finished unit q - 2, so every unit of tile
                // j - 2 (at most 2 units per channel set): its ring slot is free
                if (c == 0 && j >= 2 && j - 2 + kWsStages < ntl) load_phi(j - 2 + kWsStages);
                if (lane == 0) rec[b] = box;
                float* buf = bufs + b * kWsCap;
                const unsigned fb = box_full + 8u * b;
                if (box.mode == 1 && box.tma) {
                    __syncwarp();
                    if (lane == 0) {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        mbar_expect_tx(fb, (unsigned)(kWsCap * sizeof(float)));
                        tma_load_4d(smem_addr(buf), &imgmap, fb, box.xo, box.lo[1], box.lo[2], o.b * nc + c);
                    }
                } else {
                    if (box.mode == 1) {
                        int b0, b1, b2;
                        bnd_code(a, c, b0, b1, b2);
                        ws_stage_gather<IT>(box, g, b0, b1, b2, a.in + ((long long)o.b * nc + c) * g.n0, buf, lane);
                    }
                    __syncwarp();
                    if (lane == 0) mbar_arrive(fb);
                }
            }
        }
        return;
    }

    // ---------------- consumer warps ----------------
    const int ctid = threadIdx.x;
    for (int j = 0; j < ntl; ++j) {
        const TileOrigin o = tile_origin(t, T0 + j * G);
        const float* slot = ring + (j % kWsStages) * 3 * kWsNV;
        if (!mbar_wait(phi_full + 8u * (j % kWsStages), (unsigned)((j / kWsStages) & 1))) s_abort = 1;
        if (s_abort) break;
        float acc[kWsV][3];
#pragma unroll
        for (int q = 0; q < kWsV; ++q) acc[q][0] = acc[q][1] = acc[q][2] = 0.f;
        for (int c = 0; c < nc; ++c) {
            const int q = j * nc + c, b = q % kWsBufs, k = q / kWsBufs;
            if (!mbar_wait(box_full + 8u * b, (unsigned)(k & 1))) s_abort = 1;
            if (s_abort) break;
            ws_pull_unit<DP, OP, IT>(a, o, ctid, slot, c, rec[b], bufs + b * kWsCap, acc, D0, D1, D2);
            __syncwarp();
            if (lane == 0) mbar_arrive(box_empty + 8u * b);
        }
        if (s_abort) break;
    }
}

// 4-D map over an image stack (d0, d1, d2, planes) whose box is the fixed
// kWsWin* window; false when TMA cannot address the image.
bool encode_window_map(CUtensorMap* map, const float* base, const long long d[3], long long planes) {
    auto fn = encode_fn();
    if (!fn) return false;
    if ((reinterpret_cast<uintptr_t>(base) & 15) || (d[0] & 3)) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)d[0], (cuuint64_t)d[1], (cuuint64_t)d[2], (cuuint64_t)planes};
    for (int k = 0; k < 4; ++k)
        if (dims[k] == 0 || dims[k] > (1ULL << 32)) return false;
    const cuuint64_t strides[3] = {(cuuint64_t)d[0] * 4, (cuuint64_t)(d[0] * d[1]) * 4,
                                   (cuuint64_t)(d[0] * d[1] * d[2]) * 4};
    for (int k = 0; k < 3; ++k)
        if (strides[k] >= (1ULL << 40)) return false;
    const cuuint32_t box[4] = {(cuuint32_t)kWsWinX, (cuuint32_t)kWsWinY, (cuuint32_t)kWsWinZ, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

template <int DP, int OP, typename IT>
cudaError_t launch_ws_one(const LaunchArgs& a, const TileGrid& t, const CUtensorMap& phimap, cudaStream_t s) {
    CUtensorMap imgmap;
    std::memset(&imgmap, 0, sizeof imgmap);
    TileGrid tt = t;
    tt.img_tma = encode_window_map(&imgmap, a.in, a.g.d0, (long long)a.g.nc * a.g.nb) ? 1 : 0;
    auto kern = k_pull_ws<DP, OP, IT>;
    cudaError_t e = opt_in(kern, kWsSmem);
    if (e != cudaSuccess) return e;
    const int grid = tt.ntiles < sm_count() ? tt.ntiles : sm_count();
    kern<<<grid, kWsThreads, kWsSmem, s>>>(a, tt, phimap, imgmap);
    return cudaGetLastError();
}

}  // namespace
}  // namespace pp
