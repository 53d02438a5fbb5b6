// pp_ws.cuh -- warp-specialised persistent pull family: pull, pull_grad,
// pull_hess, the rrule contractions pull_grad_dot / pull_hess_dot, and the
// affine pull.
//
// Included after pp_tiled_impl.cuh (whose helpers it uses) by pp_ws_pull.cu,
// pp_ws_hess.cu, pp_ws_grad_dot.cu and pp_ws_hess_dot.cu.
//
// One CTA per SM: 15 consumer warps and one producer warp (512 threads, so
// every thread keeps 128 registers).  The CTA walks tiles of 8 x 8 x 30 sample
// voxels, four per consumer thread, in (tile, channel) units:
//   * the producer warp streams each tile's deformation into a ring of
//     shared-memory slots with one TMA copy per tile (mbarrier complete_tx);
//   * every consumer warp reduces the first taps of its own voxels of tile
//     j + 1 before it evaluates tile j and publishes the warp's bounds;
//   * the producer combines the fifteen records into the tile's footprint box
//     and, for a box inside the image that fits a fixed 24 x 16 x 40 window,
//     stages it with one TMA copy into one of two buffers while the consumers
//     still evaluate the previous unit; it then publishes the box record;
//   * boundary boxes whose margins mirror (DCT-II, DST-II) onto elements of the
//     box itself arrive by the same TMA copy, zero-filled outside the image,
//     and the consumers complete the margins in shared memory; other boundary
//     boxes (circulant margins) are gathered by all the consumers when they
//     take the unit, 16-byte chunks where a row is in range.  Both sit behind
//     consumer-only named barriers.
// Interior units therefore pass no CTA-wide barrier at all.  Boxes larger than
// a buffer take the per-voxel global path for that tile.
//
// Reference kernels replaced: pull_element / pullg_element / pullh_element
// (artifacts/C/pushpull.cu:33-109); per-voxel math pull1 / pullg1 / pullh1
// (artifacts/C/pushpull_dev.cu:61-117); the rrule contractions replace the
// pull_grad and pull_hess temporaries of the rrules (src/pushpull_pb.jl:11-35).
#pragma once

#include "pp_tiled_impl.cuh"

namespace pp {
namespace {

constexpr int kWsCons = 480;                   // consumer threads (15 warps)
constexpr int kWsThreads = kWsCons + 32;       // plus the producer warp
constexpr int kWsV = 4;                        // sample voxels per consumer thread
constexpr int kWsTz = 30;                      // tile: 8 x 8 x 30 sample voxels
constexpr int kWsNV = kWsCons * kWsV;          // 1920 voxels per tile
constexpr int kWsStages = 3;                   // deformation ring slots
constexpr int kWsBufs = 2;                     // box buffers
constexpr int kWsWinX = 24, kWsWinY = 16, kWsWinZ = 40;   // TMA image window (row pitch 24)
constexpr int kWsCap = kWsWinX * kWsWinY * kWsWinZ;         // floats per box buffer
constexpr size_t kWsSmem = (size_t)(kWsStages * 3 * kWsNV + kWsBufs * kWsCap) * sizeof(float);

__device__ __forceinline__ void mbar_arrive(unsigned bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Tile-local voxel lin (x fastest, 8 x 8 x 30) -> linear sample index, or -1.
template <typename IT>
__device__ __forceinline__ IT ws_index(const TileOrigin& o, int lin, int D0, int D1, int D2) {
    const int gx = o.x0 + (lin & 7), gy = o.y0 + ((lin >> 3) & 7), gz = o.z0 + (lin >> 6);
    if (gx >= D0 || gy >= D1 || gz >= D2) return (IT)-1;
    return (IT)gx + (IT)D0 * ((IT)gy + (IT)D1 * (IT)gz);
}

// Origin of linear tile T (x fastest, batch slowest) of the 8 x 8 x 30 grid.
__device__ __forceinline__ TileOrigin ws_origin(const TileGrid& t, int T) {
    const unsigned u = (unsigned)T;
    const unsigned q1 = (unsigned)(((unsigned long long)u * t.mx) >> t.sx);
    const unsigned q2 = (unsigned)(((unsigned long long)q1 * t.my) >> t.sy);
    const unsigned q3 = (unsigned)(((unsigned long long)q2 * t.mz) >> t.sz);
    TileOrigin r;
    r.x0 = (int)(u - q1 * (unsigned)t.ntx) << 3;
    r.y0 = (int)(q1 - q2 * (unsigned)t.nty) << 3;
    r.z0 = (int)(q2 - q3 * (unsigned)t.ntz) * kWsTz;
    r.b = (int)q3;
    return r;
}

// Sample positions of a tile's voxels: x = phi - 1 from the tile's ring slot,
// or (AFF, the affine ops) A * (i, j, k, 1) from the voxel's grid coordinates;
// either way with the validity test.
template <bool AFF>
struct WsPos {
    const float* slot;
    const AffineMap* A;
    __device__ __forceinline__ bool operator()(const Geometry& g, const TileOrigin& o, int lin, float& x0, float& x1,
                                               float& x2) const {
        if constexpr (AFF) {
            affine_position(*A, (float)(o.x0 + (lin & 7)), (float)(o.y0 + ((lin >> 3) & 7)), (float)(o.z0 + (lin >> 6)),
                            x0, x1, x2);
            return position_valid(x0, x1, x2, g);
        } else {
            return load_valid(slot[lin], slot[kWsNV + lin], slot[2 * kWsNV + lin], g, x0, x1, x2);
        }
    }
};

// First-tap bounds of one consumer thread's voxels of the tile, reduced over
// its warp (every lane ends with the warp's bounds).
template <int DP, typename IT, class POS>
__device__ __forceinline__ void ws_warp_bounds(const Geometry& g, const TileOrigin& o, const POS& pos, int ctid,
                                               int D0, int D1, int D2, int (&mn)[3], int (&mx)[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        mn[k] = INT_MAX;
        mx[k] = INT_MIN;
    }
#pragma unroll
    for (int q = 0; q < kWsV; ++q) {
        const int i = ctid + q * kWsCons;
        if (ws_index<IT>(o, i, D0, D1, D2) < 0) continue;
        float x[3];
        if (!pos(g, o, i, x[0], x[1], x[2])) continue;
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
}

// Footprint box of a tile from the consumer warps' bound records (producer
// warp; every lane ends with the same box).  win_ok: interior boxes may use
// the TMA window.
template <int DP>
__device__ __forceinline__ Box ws_tile_box(const Geometry& g, const int (*wrec)[6], bool win_ok, int lane) {
    constexpr int NW = kWsCons / 32;
    int mn[3], mx[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        mn[k] = __reduce_min_sync(0xffffffffu, lane < NW ? wrec[lane][k] : INT_MAX);
        mx[k] = __reduce_max_sync(0xffffffffu, lane < NW ? wrec[lane][3 + k] : INT_MIN);
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

// Gather one channel of a box into shared memory with `nthreads` threads
// (tid = 0 .. nthreads-1, nthreads a multiple of 32), folding (and signing)
// out-of-range taps; in-range 16-byte row chunks are one vector load each.
// Threads split over (row, chunk) pairs.
template <typename IT>
__device__ __forceinline__ void ws_stage_gather(const Box& box, const Geometry& g, int b0, int b1, int b2,
                                                const float* f0, float* sm, int tid, int nthreads) {
    const int ex = box.ext[0], ey = box.ext[1], ez = box.ext[2];
    const int n4 = (ex + 3) >> 2;
    const int nn = n4 < 1 ? 1 : (n4 > 32 ? 32 : n4);
    const int lg = 32 - __clz(nn - 1);          // threads per row = 1 << lg
    const int lpr = 1 << lg;
    const int sub = tid >> lg, e4 = tid & (lpr - 1), step = nthreads >> lg;
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

// A boundary box whose out-of-image margins all fold by a mirror (DCT-II or
// DST-II) onto elements inside the box itself can be loaded by the TMA window
// like an interior box (the margins arrive zero-filled) and completed in shared
// memory by ws_mirror_fixup.  True when the box fits the window and every
// margin qualifies; circulant margins (whose sources lie across the image) and
// margins wider than the in-image part take the gather instead.
__device__ __forceinline__ bool ws_mirror_ok(const Box& box, const Geometry& g, int b0, int b1, int b2) {
    if (box.mode != 1 || box.ext[0] > kWsWinX || box.ext[1] > kWsWinY || box.ext[2] > kWsWinZ) return false;
    const int bk[3] = {b0, b1, b2};
    const int lo[3] = {box.xo, box.lo[1], box.lo[2]};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const long long d = g.d0[k], l = lo[k], e = box.ext[k];
        const long long hl = l < 0 ? -l : 0, hr = l + e > d ? l + e - d : 0;
        if (hl == 0 && hr == 0) continue;
        if (bk[k] == 0) return false;                                    // circulant
        if (hl > d || hr > d) return false;                              // more than one reflection
        if (hl > 0 && l + e < 2 * hl) return false;                      // left sources [0, hl) outside the box
        if (hr > 0 && d - hr < l) return false;                          // right sources [d - hr, d) outside
    }
    return true;
}

// Fill the margins of a TMA-loaded boundary box (row pitch kWsWinX, plane pitch
// kWsWinX * kWsWinY) from their mirror images inside the box, x margins first
// (rows inside the image in y and z), then whole y-margin rows (planes inside
// in z), then whole z-margin planes, each step reading only elements the
// previous steps completed.  DST-II margins take the sign -1.  All consumer
// threads; named barrier 1 between the steps and at the end.
__device__ __forceinline__ void ws_mirror_fixup(const Box& box, const Geometry& g, int b0, int b1, int b2,
                                                float* sm, int tid, int nthreads) {
    constexpr int P = kWsWinX, Q = kWsWinX * kWsWinY;
    const int e0 = box.ext[0], e1 = box.ext[1], e2 = box.ext[2];
    const int lx = box.xo, ly = box.lo[1], lz = box.lo[2];
    const int dx = (int)g.d0[0], dy = (int)g.d0[1], dz = (int)g.d0[2];
    // x margins
    const int hlx = lx < 0 ? -lx : 0, hrx = lx + e0 > dx ? lx + e0 - dx : 0, nh = hlx + hrx;
    if (nh > 0) {
        const float sx = b0 == 2 ? -1.f : 1.f;
        const int items = nh * e1 * e2;
        for (int it = tid; it < items; it += nthreads) {
            const int row = it / nh, h = it - row * nh;
            const int rz = row / e1, ry = row - rz * e1;
            const int gy = ly + ry, gz = lz + rz;
            if (gy < 0 || gy >= dy || gz < 0 || gz >= dz) continue;   // a y or z margin row: later
            const int ex = h < hlx ? h : e0 - hrx + (h - hlx);
            const int gx = lx + ex;
            const int src = (gx < 0 ? -1 - gx : 2 * dx - 1 - gx) - lx;
            float* r = sm + rz * Q + ry * P;
            r[ex] = sx * r[src];
        }
        asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
    }
    // y margin rows of the planes inside the image
    const int hly = ly < 0 ? -ly : 0, hry = ly + e1 > dy ? ly + e1 - dy : 0, nhy = hly + hry;
    if (nhy > 0) {
        const float sy = b1 == 2 ? -1.f : 1.f;
        const int items = nhy * e2 * e0;
        for (int it = tid; it < items; it += nthreads) {
            const int rowi = it / e0, x = it - rowi * e0;
            const int rz = rowi / nhy, h = rowi - rz * nhy;
            const int gz = lz + rz;
            if (gz < 0 || gz >= dz) continue;
            const int ry = h < hly ? h : e1 - hry + (h - hly);
            const int gy = ly + ry;
            const int sry = (gy < 0 ? -1 - gy : 2 * dy - 1 - gy) - ly;
            sm[rz * Q + ry * P + x] = sy * sm[rz * Q + sry * P + x];
        }
        asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
    }
    // z margin planes
    const int hlz = lz < 0 ? -lz : 0, hrz = lz + e2 > dz ? lz + e2 - dz : 0, nhz = hlz + hrz;
    if (nhz > 0) {
        const float sz = b2 == 2 ? -1.f : 1.f;
        const int per = e1 * e0;
        const int items = nhz * per;
        for (int it = tid; it < items; it += nthreads) {
            const int h = it / per, rem = it - h * per;
            const int ry = rem / e0, x = rem - ry * e0;
            const int rz = h < hlz ? h : e2 - hrz + (h - hlz);
            const int gz = lz + rz;
            const int srz = (gz < 0 ? -1 - gz : 2 * dz - 1 - gz) - lz;
            sm[rz * Q + ry * P + x] = sz * sm[srz * Q + ry * P + x];
        }
        asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
    }
}

// One consumer thread, one (tile, channel) unit of the pull family: its four
// voxels against the staged box.  The dot ops accumulate over channels in the
// output itself: channel 0 writes its term, later channels (same thread, same
// voxels) read it back and add theirs, in the order the per-voxel kernels
// accumulate in registers.
template <int DP, int OP_, typename IT, class POS>
__device__ __forceinline__ void ws_pull_unit(const LaunchArgs& a, const TileOrigin& o, int ctid, const POS& pos,
                                             int c, const Box& box, const float* sm, int D0, int D1, int D2) {
    constexpr int OP = pull_base_op<OP_>();
    constexpr int NCOMP = pull_ncomp<OP_>();
    constexpr int ORD = op_order(OP);
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const bool last = c == g.nc - 1;
    // the box record in registers: the output stores would otherwise make the
    // compiler reload it from shared memory for every voxel
    const int bmode = box.mode, bxo = box.xo, by0 = box.lo[1], bz0 = box.lo[2], bP = box.P, bQ = box.Q;
    auto voxel = [&](int q) {
        const int lin = ctid + q * kWsCons;
        const IT v = ws_index<IT>(o, lin, D0, D1, D2);
        if (v < 0) return;
        float x0, x1, x2;
        if (!pos(g, o, lin, x0, x1, x2)) {
            if (!pull_is_dot<OP_>() || last) {
                float* out = pull_out<OP_>(a, o.b, c, (long long)v);
#pragma unroll
                for (int p = 0; p < NCOMP; ++p) out[(long long)p * n1] = qnan();
            }
            return;
        }
        if (bmode == 2) {   // box larger than a buffer: every channel from global memory, once
            if (c == 0) pull_voxel_lean<DP, OP_, IT>(a, o.b, (long long)v, x0, x1, x2);
            return;
        }
        if (bmode != 1) return;
        W3<DP, ORD> wx, wy, wz;
        const int ox = spline_taps32<DP, ORD>(x0, wx.w, wx.dw, wx.hw) - bxo;
        const int oy = spline_taps32<DP, ORD>(x1, wy.w, wy.dw, wy.hw) - by0;
        const int oz = spline_taps32<DP, ORD>(x2, wz.w, wz.dw, wz.hw) - bz0;
        const unsigned P4 = 4u * bP, Q4 = 4u * bQ;
        const unsigned p = smem_addr(sm) + 4u * (unsigned)(oz * bQ + oy * bP + ox);
        float r[6];
        contract_smem<OP, DP>(wx, wy, wz, p, P4, Q4, r);
        if constexpr (pull_is_dot<OP_>()) {
            float* out = pull_out<OP_>(a, o.b, 0, (long long)v);
            float acc[3] = {0.f, 0.f, 0.f};
            if (c > 0) {
                acc[0] = out[0];
                acc[1] = out[n1];
                acc[2] = out[2 * n1];
            }
            dot_accumulate<OP_>(a, o.b, c, (long long)v, r, acc);
            out[0] = acc[0];
            out[n1] = acc[1];
            out[2 * n1] = acc[2];
        } else {
            pull_store<OP>(pull_out<OP_>(a, o.b, c, (long long)v), n1, r);
        }
    };
#pragma unroll 1
    for (int q = 0; q < kWsV; ++q) voxel(q);
}

// AFF: the affine pull -- no deformation ring; positions from `aff`.
template <int DP, int OP, typename IT, bool AFF>
__global__ void __launch_bounds__(kWsThreads, 1) k_pull_ws(const __grid_constant__ LaunchArgs a,
                                                           const __grid_constant__ TileGrid t,
                                                           const __grid_constant__ CUtensorMap phimap,
                                                           const __grid_constant__ CUtensorMap imgmap,
                                                           const __grid_constant__ AffineMap aff) {
    extern __shared__ __align__(128) float4 smem4[];
    __shared__ __align__(8) unsigned long long bars[kWsStages + 2 * kWsBufs + 2];
    __shared__ Box rec[kWsBufs];
    __shared__ int wrec[2][kWsCons / 32][6];   // per-warp first-tap bounds, by tile parity
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
    const unsigned bnd_full = smem_addr(&bars[kWsStages + 2 * kWsBufs]);   // two, by tile parity
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int k = 0; k < kWsStages; ++k) mbar_init(phi_full + 8u * k, 1);
        for (int k = 0; k < kWsBufs; ++k) {
            mbar_init(box_full + 8u * k, 1);
            mbar_init(box_empty + 8u * k, kWsCons / 32);
        }
        mbar_init(bnd_full, kWsCons / 32);
        mbar_init(bnd_full + 8u, kWsCons / 32);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == kWsCons / 32) {
        // ---------------- producer warp ----------------
        auto load_phi = [&](int j) {   // lane 0: tile j's deformation into slot j % kWsStages
            if (!AFF && lane == 0) {
                const TileOrigin o = ws_origin(t, T0 + j * G);
                const unsigned bar = phi_full + 8u * (j % kWsStages);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_expect_tx(bar, (unsigned)(3 * kWsNV * sizeof(float)));
                tma_load_4d(smem_addr(ring + (j % kWsStages) * 3 * kWsNV), &phimap, bar, o.x0, o.y0, o.z0, 3 * o.b);
            }
        };
        for (int j = 0; j < kWsStages && j < ntl; ++j) load_phi(j);
        for (int j = 0; j < ntl && !s_abort; ++j) {
            const TileOrigin o = ws_origin(t, T0 + j * G);
            if (!mbar_wait(bnd_full + 8u * (j & 1), (unsigned)((j >> 1) & 1))) {
                s_abort = 1;
                break;
            }
            const Box box = ws_tile_box<DP>(g, wrec[j & 1], t.img_tma != 0, lane);
            for (int c = 0; c < nc; ++c) {
                const int q = j * nc + c, b = q % kWsBufs, k = q / kWsBufs;
                if (k >= 1 && !mbar_wait(box_empty + 8u * b, (unsigned)((k - 1) & 1))) {
                    s_abort = 1;
                    break;
                }
                // the consumers have finished unit q - 2, so every unit of tile
                // j - 2: its ring slot is free for tile j + 2
                if (c == 0 && j >= 2 && j - 2 + kWsStages < ntl) load_phi(j - 2 + kWsStages);
                // interior boxes, and boundary boxes whose margins are mirrors
                // of their own elements (tma = 2: completed by the consumers),
                // arrive by one TMA copy; the consumers gather all others
                // themselves when they take the unit
                Box ub = box;
                if (ub.mode == 1 && !ub.tma && t.img_tma) {
                    int b0, b1, b2;
                    bnd_code(a, c, b0, b1, b2);
                    if (ws_mirror_ok(ub, g, b0, b1, b2)) {
                        ub.tma = 2;
                        ub.P = kWsWinX;
                        ub.Q = kWsWinX * kWsWinY;
                        ub.size = kWsCap;
                    }
                }
                if (lane == 0) rec[b] = ub;
                float* buf = bufs + b * kWsCap;
                const unsigned fb = box_full + 8u * b;
                __syncwarp();
                if (lane == 0) {
                    if (ub.mode == 1 && ub.tma) {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        mbar_expect_tx(fb, (unsigned)(kWsCap * sizeof(float)));
                        tma_load_4d(smem_addr(buf), &imgmap, fb, ub.xo, ub.lo[1], ub.lo[2], o.b * nc + c);
                    } else {
                        mbar_arrive(fb);
                    }
                }
            }
        }
        return;
    }

    // ---------------- consumer warps ----------------
    // Each warp reduces the first-tap bounds of its voxels of tile j + 1 before
    // it evaluates tile j, so the producer can stage box j + 1 meanwhile.
    const int ctid = threadIdx.x;
    auto publish_bounds = [&](int j) -> bool {
        const TileOrigin o = ws_origin(t, T0 + j * G);
        const WsPos<AFF> pos{ring + (j % kWsStages) * 3 * kWsNV, &aff};
        if (!AFF && !mbar_wait(phi_full + 8u * (j % kWsStages), (unsigned)((j / kWsStages) & 1))) return false;
        int mn[3], mx[3];
        ws_warp_bounds<DP, IT>(g, o, pos, ctid, D0, D1, D2, mn, mx);
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                wrec[j & 1][warp][k] = mn[k];
                wrec[j & 1][warp][3 + k] = mx[k];
            }
            mbar_arrive(bnd_full + 8u * (j & 1));
        }
        return true;
    };
    if (!publish_bounds(0)) s_abort = 1;
    for (int j = 0; j < ntl && !s_abort; ++j) {
        const TileOrigin o = ws_origin(t, T0 + j * G);
        const WsPos<AFF> pos{ring + (j % kWsStages) * 3 * kWsNV, &aff};
        if (j + 1 < ntl && !publish_bounds(j + 1)) s_abort = 1;
        if (s_abort) break;
        for (int c = 0; c < nc; ++c) {
            const int q = j * nc + c, b = q % kWsBufs, k = q / kWsBufs;
            if (!mbar_wait(box_full + 8u * b, (unsigned)(k & 1))) s_abort = 1;
            if (s_abort) break;
            const Box& box = rec[b];
            float* buf = bufs + b * kWsCap;
            if (box.mode == 1 && box.tma != 1) {   // boundary box: all consumers complete or gather it
                int b0, b1, b2;
                bnd_code(a, c, b0, b1, b2);
                if (box.tma == 2) {
                    ws_mirror_fixup(box, g, b0, b1, b2, buf, ctid, kWsCons);
                } else {
                    ws_stage_gather<IT>(box, g, b0, b1, b2, a.in + ((long long)o.b * nc + c) * g.n0, buf, ctid,
                                        kWsCons);
                    asm volatile("bar.sync 1, %0;" ::"n"(kWsCons) : "memory");
                }
            }
            ws_pull_unit<DP, OP, IT>(a, o, ctid, pos, c, box, buf, D0, D1, D2);
            __syncwarp();
            if (lane == 0) mbar_arrive(box_empty + 8u * b);
        }
        if (s_abort) break;
    }
}

// Tile grid of 8 x 8 x 30 tiles over the sample grid (all batches), with the
// multiply-shift constants of ws_origin.
TileGrid ws_make_grid(const LaunchArgs& a) {
    TileGrid t;
    t.lx = 3;
    t.ly = 3;
    t.lz = 4;   // unused here: the z side of a tile is kWsTz
    t.ntx = (int)((a.g.d1[0] + 7) >> 3);
    t.nty = (int)((a.g.d1[1] + 7) >> 3);
    t.ntz = (int)((a.g.d1[2] + kWsTz - 1) / kWsTz);
    t.cap = kWsCap;
    t.ntiles = t.ntx * t.nty * t.ntz * a.g.nb;
    auto magic = [](int d, unsigned long long& m, int& sh) {
        int l = 0;
        while ((1LL << l) < d) ++l;
        sh = 31 + l;
        m = ((1ULL << sh) + (unsigned long long)d - 1) / (unsigned long long)d;
    };
    magic(t.ntx, t.mx, t.sx);
    magic(t.nty, t.my, t.sy);
    magic(t.ntz, t.mz, t.sz);
    t.pmod = 8;
    t.img_tma = 0;
    return t;
}

// 4-D map over the deformation stack (d1, 3 * nb) whose box is one tile's
// three components (8, 8, 15, 3); false when TMA cannot address it.
bool encode_ws_phi_map(CUtensorMap* map, const float* base, const long long d[3], long long planes) {
    EncodeFn fn = encode_fn();
    if (!fn) return false;
    if ((reinterpret_cast<uintptr_t>(base) & 15) || (d[0] & 3)) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)d[0], (cuuint64_t)d[1], (cuuint64_t)d[2], (cuuint64_t)planes};
    for (int k = 0; k < 4; ++k)
        if (dims[k] == 0 || dims[k] > (1ULL << 32)) return false;
    const cuuint64_t strides[3] = {(cuuint64_t)d[0] * 4, (cuuint64_t)(d[0] * d[1]) * 4,
                                   (cuuint64_t)(d[0] * d[1] * d[2]) * 4};
    for (int k = 0; k < 3; ++k)
        if (strides[k] >= (1ULL << 40)) return false;
    const cuuint32_t box[4] = {8, 8, (cuuint32_t)kWsTz, 3};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
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

template <int DP, int OP, typename IT, bool AFF>
cudaError_t launch_ws_one(const LaunchArgs& a, const TileGrid& t, const CUtensorMap& phimap, const AffineMap& aff,
                          cudaStream_t s) {
    CUtensorMap imgmap;
    std::memset(&imgmap, 0, sizeof imgmap);
    TileGrid tt = t;
    tt.img_tma = encode_window_map(&imgmap, a.in, a.g.d0, (long long)a.g.nc * a.g.nb) ? 1 : 0;
    auto kern = k_pull_ws<DP, OP, IT, AFF>;
    cudaError_t e = opt_in(kern, kWsSmem);
    if (e != cudaSuccess) return e;
    const int grid = tt.ntiles < sm_count() ? tt.ntiles : sm_count();
    kern<<<grid, kWsThreads, kWsSmem, s>>>(a, tt, phimap, imgmap, aff);
    return cudaGetLastError();
}

template <int OP, typename IT, bool AFF = false>
cudaError_t ws_dispatch(const LaunchArgs& a, const TileGrid& t, const CUtensorMap& phimap, cudaStream_t s,
                        const AffineMap& aff = AffineMap{}) {
    switch (a.g.dp[0]) {
        case 1: return launch_ws_one<1, OP, IT, AFF>(a, t, phimap, aff, s);
        case 2: return launch_ws_one<2, OP, IT, AFF>(a, t, phimap, aff, s);
        case 3: return launch_ws_one<3, OP, IT, AFF>(a, t, phimap, aff, s);
        case 4: return launch_ws_one<4, OP, IT, AFF>(a, t, phimap, aff, s);
        default: return launch_ws_one<5, OP, IT, AFF>(a, t, phimap, aff, s);
    }
}

// One op of the warp-specialised family on 32-bit or 64-bit voxel indices.
template <int OP>
cudaError_t ws_dispatch_op(const LaunchArgs& a, const TileGrid& t, const CUtensorMap& phimap, cudaStream_t s) {
    const bool small = a.g.n0 < (1LL << 31) - 1 && a.g.n1 < (1LL << 31) - 1;
    return small ? ws_dispatch<OP, int>(a, t, phimap, s) : ws_dispatch<OP, long long>(a, t, phimap, s);
}

}  // namespace
}  // namespace pp
