// pp_tiled_impl.cuh -- shared-memory tiled pull family and privatised push family.
//
// Included by the pp_tiled*.cu translation units, each of which instantiates
// one group of kernels (so the library compiles in parallel); everything here
// has internal linkage, the device status word included (one per unit, read
// and combined by read_device_status).
//
// A CTA owns a TX x TY x TZ tile of sample voxels (power-of-two sides, up to
// 256*V voxels for 256 threads).  It reads the tile's deformation once,
// reduces the integer first taps to the tile's footprint box in the image
//   [min o, max o + dp - 1]  per dimension,
// and, when the box fits its shared-memory budget:
//   pull:  stages the box once per channel -- boundary folding and the DST-II
//          sign are applied while staging, so taps index the box directly with
//          no per-tap modulo -- then evaluates every voxel from shared memory;
//   push:  zeroes a box-sized accumulator, scatters every voxel's weighted taps
//          into it with shared-memory atomics, then flushes the box to the
//          image with one global reduction per non-zero element (4-wide vector
//          reductions on aligned interior runs) instead of dp^3 global atomics
//          per voxel.
// Tiles whose footprint does not fit (large local expansion, far-out
// coordinates) take the per-voxel global path for that tile only.
//
// Latency: each CTA is persistent and walks a sequence of tiles.  The
// deformation of the next kStages tiles (and, for push, their channel-0 values)
// streams into a ring of shared-memory slots with TMA bulk tensor copies that
// complete on mbarriers, so several tiles' worth of HBM reads are in flight per
// SM while the current tile computes.  Pull additionally stages the next tile's
// image box with cp.async into a second buffer.
//
// Bank layout: lanes of a warp cover TX consecutive x of the tile and
// 32/TX consecutive tile rows in y.  The box row pitch P is chosen with
// P % 32 == TX % 32, so for a smooth deformation the rows of one warp land in
// disjoint bank ranges (TX = 32: bank = x mod 32 in every row).
//
// Reference kernels replaced: pull_element / pullg_element / pullh_element /
// push_element / pushg_element (artifacts/C/pushpull.cu:33-163); per-voxel math
// pull1 / pullg1 / pullh1 / push1 / pushg1 (artifacts/C/pushpull_dev.cu:61-179).
#include <climits>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "pp_tiled.cuh"
#include "pp_voxel.cuh"

namespace pp {
namespace {

// Device status word of this translation unit: bits record bounded waits that
// gave up (read and cleared through read_device_status).
__device__ unsigned int g_device_status;

unsigned unit_status(bool reset) {
    unsigned v = 0;
    if (cudaMemcpyFromSymbol(&v, g_device_status, sizeof v) != cudaSuccess) return 0xffffffffu;
    if (reset) {
        const unsigned z = 0;
        cudaMemcpyToSymbol(g_device_status, &z, sizeof z);
    }
    return v;
}

constexpr int kThreads = 256;
constexpr int kStages = 4;                 // tiles of the ring in flight per CTA
constexpr unsigned kStatusWaitTimeout = 1u;
constexpr int kClamp = 1 << 29;    // first taps are clamped to +-kClamp for the box reduction
// Fixed image window for TMA-staged pull boxes: row pitch 24 (24 % 32 places
// the 4 rows of an 8-wide warp tile in disjoint bank ranges), 16 rows, 16 planes.
constexpr int kTmaBoxX = 24, kTmaBoxY = 16, kTmaBoxZ = 16;
constexpr int kTmaBoxFloats = kTmaBoxX * kTmaBoxY * kTmaBoxZ;

template <int DP, int ORD>
struct W3 {
    float w[DP];
    float dw[ORD >= 1 ? DP : 1];
    float hw[ORD >= 2 ? DP : 1];
};

// One spline row of DP consecutive box elements, addressed with immediate
// offsets from one shared-memory base address (one asm statement per row).
template <int DP>
__device__ __forceinline__ void lds_row(unsigned a, float (&f)[DP]) {
    if constexpr (DP == 1) {
        asm volatile("ld.shared.f32 %0, [%1];" : "=f"(f[0]) : "r"(a));
    } else if constexpr (DP == 2) {
        asm volatile("ld.shared.f32 %0, [%2];\n\tld.shared.f32 %1, [%2+4];" : "=f"(f[0]), "=f"(f[1]) : "r"(a));
    } else if constexpr (DP == 3) {
        asm volatile("ld.shared.f32 %0, [%3];\n\tld.shared.f32 %1, [%3+4];\n\tld.shared.f32 %2, [%3+8];"
                     : "=f"(f[0]), "=f"(f[1]), "=f"(f[2]) : "r"(a));
    } else if constexpr (DP == 4) {
        asm volatile("ld.shared.f32 %0, [%4];\n\tld.shared.f32 %1, [%4+4];\n\tld.shared.f32 %2, [%4+8];\n\t"
                     "ld.shared.f32 %3, [%4+12];"
                     : "=f"(f[0]), "=f"(f[1]), "=f"(f[2]), "=f"(f[3]) : "r"(a));
    } else {
        asm volatile("ld.shared.f32 %0, [%5];\n\tld.shared.f32 %1, [%5+4];\n\tld.shared.f32 %2, [%5+8];\n\t"
                     "ld.shared.f32 %3, [%5+12];\n\tld.shared.f32 %4, [%5+16];"
                     : "=f"(f[0]), "=f"(f[1]), "=f"(f[2]), "=f"(f[3]), "=f"(f[4]) : "r"(a));
    }
}

// Integer reductions of DP consecutive box words (one asm statement per row).
template <int DP>
__device__ __forceinline__ void red_row_s32(unsigned a, const int (&v)[DP]) {
    if constexpr (DP == 1) {
        asm volatile("red.shared.add.s32 [%0], %1;" ::"r"(a), "r"(v[0]) : "memory");
    } else if constexpr (DP == 2) {
        asm volatile("red.shared.add.s32 [%0], %1;\n\tred.shared.add.s32 [%0+4], %2;" ::"r"(a), "r"(v[0]), "r"(v[1])
                     : "memory");
    } else if constexpr (DP == 3) {
        asm volatile("red.shared.add.s32 [%0], %1;\n\tred.shared.add.s32 [%0+4], %2;\n\t"
                     "red.shared.add.s32 [%0+8], %3;" ::"r"(a), "r"(v[0]), "r"(v[1]), "r"(v[2])
                     : "memory");
    } else if constexpr (DP == 4) {
        asm volatile("red.shared.add.s32 [%0], %1;\n\tred.shared.add.s32 [%0+4], %2;\n\t"
                     "red.shared.add.s32 [%0+8], %3;\n\tred.shared.add.s32 [%0+12], %4;" ::"r"(a), "r"(v[0]),
                     "r"(v[1]), "r"(v[2]), "r"(v[3])
                     : "memory");
    } else {
        asm volatile("red.shared.add.s32 [%0], %1;\n\tred.shared.add.s32 [%0+4], %2;\n\t"
                     "red.shared.add.s32 [%0+8], %3;\n\tred.shared.add.s32 [%0+12], %4;\n\t"
                     "red.shared.add.s32 [%0+16], %5;" ::"r"(a), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4])
                     : "memory");
    }
}

struct Box {
    int lo[3];      // minima of the first taps
    int xo;         // x origin of the box in shared memory: lo[0] rounded down to a multiple of 4
    int ext[3];     // box extent (x counted from xo)
    int P, Q, size; // row pitch (P % 32 == pmod, P % 4 == 0), plane pitch (multiple of 32), floats
    int mode;       // 0 no valid voxel, 1 shared memory, 2 per-voxel global fallback
    int interior;   // bit k: the box lies inside the image along dimension k (no folding)
    int tma;        // 1: the box is a fixed window loaded by one TMA copy; 2: the same, with mirrored margins to complete
    float S;        // block sum of the caller's per-thread value (push: bound on sum |contribution|)
    int E;          // scale exponent of the fixed-point accumulator for S (see scale_exponent)
    int wsc;        // push: 1 = scatter one voxel per warp instruction (contracted tile)
};

__device__ __forceinline__ int clamp_tap(long long o) {
    return (int)(o < -kClamp ? -kClamp : (o > kClamp ? kClamp : o));
}

__device__ __forceinline__ int first_tap_i(float x, int DP) {
    return clamp_tap((long long)ceilf(__fsub_rn(x, 0.5f * (float)DP)));
}

// Exponent E of the fixed-point accumulator scale for a bound S on the sum of
// |contributions|: S < 2^E.  INT_MAX: nothing to accumulate (S == 0);
// INT_MIN: S non-finite or outside the range the scale factors cover, so the
// tile accumulates in float instead.
__device__ __forceinline__ int scale_exponent(float S) {
    if (S == 0.f) return INT_MAX;
    if (!(S > 0.f) || !finitef(S)) return INT_MIN;
    int E;
    frexpf(S * 1.0009765625f, &E);
    return (E < -80 || E > 100) ? INT_MIN : E;
}

// ---- pitches for the warp-cooperative scatter -------------------------------
// One voxel per warp instruction, one tap per lane: lane l of pass p takes tap
// t = 32 p + l, (i, j, k) = t in radix DP, at box element base + i + P j + Q k.
// The taps of one voxel never share an element, and for (P mod 32, Q mod 32)
// pairs whose bit is set below (bit Q of entry P, one row per DP = 3, 4, 5) the
// 32 lanes of every pass also fall in 32 distinct shared-memory banks, so each
// reduction is a single wavefront whatever the deformation does.
__device__ const unsigned kScatterQMask[3][32] = {
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00e00e00u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00200800u,
     0x00000000u, 0x20000008u, 0x20000008u, 0x22044088u, 0x00000000u, 0x00000000u, 0x00200800u, 0x00000000u,
     0x00000000u, 0x00000000u, 0x00200800u, 0x00000000u, 0x00000000u, 0x22044088u, 0x20000008u, 0x20000008u,
     0x00000000u, 0x00200800u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00e00e00u, 0x00000000u, 0x00000000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00010000u, 0x00000000u, 0x00000000u, 0x00000000u,
     0x10101010u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00010000u, 0x00000000u, 0x00000000u, 0x00000000u,
     0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00010000u, 0x00000000u, 0x00000000u, 0x00000000u,
     0x10101010u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00010000u, 0x00000000u, 0x00000000u, 0x00000000u},
    {0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x02000000u, 0x00000000u, 0x00000000u,
     0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u,
     0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u,
     0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u, 0x00000000u},
};

// Smallest row pitch P >= the row's 4-element groups (the flush reads whole
// groups of 4) and plane pitch Q >= P * e1 of a conflict-free pair.
template <int DP>
__device__ __forceinline__ void scatter_pitch(long long e0, long long e1, long long& P, long long& Q) {
    const unsigned* mask = kScatterQMask[DP - 3];
    P = (e0 + 3) & ~3LL;
    while (mask[P & 31] == 0u) ++P;
    const unsigned m = mask[P & 31];
    Q = P * e1;
    while (!((m >> (Q & 31)) & 1u)) ++Q;
}

// Block-wide reduction of the first-tap bounds into the footprint box.
// `words` = shared-memory words needed per box element (1 for pull, 2 for push).
// Also sums `ssum` over the block into box.S (fixed order) and sets box.E.
// WSCATTER (push): a tile whose box has fewer elements than the tile has
// voxels (a contracting deformation, many voxels per element) gets the
// warp-cooperative scatter when its accumulator and the voxel records
// (rec_floats, kept at the top of the budget) fit: box.wsc = 1 and the
// conflict-free pitches of scatter_pitch.
template <int DP, bool WSCATTER = false>
__device__ __forceinline__ void reduce_box(int (&mn)[3], int (&mx)[3], const TileGrid& t, const Geometry& g,
                                           int words, Box& box, int (&red)[8][7], float ssum = 0.f,
                                           int nv_tile = 0, int rec_floats = 0) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        mn[k] = __reduce_min_sync(0xffffffffu, mn[k]);
        mx[k] = __reduce_max_sync(0xffffffffu, mx[k]);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) ssum += __shfl_xor_sync(0xffffffffu, ssum, off);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            red[warp][k] = mn[k];
            red[warp][3 + k] = mx[k];
        }
        red[warp][6] = __float_as_int(ssum);
    }
    __syncthreads();
    if (warp == 0) {
        // warp 0 combines the per-warp records (lane w < 8 holds warp w's)
        constexpr int NW = kThreads / 32;
        int lo[3], hi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = __reduce_min_sync(0xffffffffu, lane < NW ? red[lane][k] : INT_MAX);
            hi[k] = __reduce_max_sync(0xffffffffu, lane < NW ? red[lane][3 + k] : INT_MIN);
        }
        // the scale bound is summed in a fixed order (warp 0, 1, ...): lane 0 alone
        float S = 0.f;
        if (lane == 0)
            for (int w = 0; w < NW; ++w) S += __int_as_float(red[w][6]);
        if (lane == 0) {
        box.S = S;
        box.E = scale_exponent(S);
        if (lo[0] > hi[0]) {
            box.mode = 0;
            box.tma = 0;
            box.wsc = 0;
        } else {
            const int xo = lo[0] & ~3;
            long long e[3];
            e[0] = (long long)hi[0] + DP - xo;
            e[1] = (long long)hi[1] + DP - lo[1];
            e[2] = (long long)hi[2] + DP - lo[2];
            int interior = 0;
            if (xo >= 0 && (long long)hi[0] + DP <= g.d0[0]) interior |= 1;
            if (lo[1] >= 0 && (long long)hi[1] + DP <= g.d0[1]) interior |= 2;
            if (lo[2] >= 0 && (long long)hi[2] + DP <= g.d0[2]) interior |= 4;
            // P % 32 == pmod and Q % 32 == 0 keep the warp's rows and planes in
            // disjoint banks; when that padding would not fit, pack tightly.
            long long P = 0, Q = 0;
            box.wsc = 0;
            if constexpr (WSCATTER) {
                if (e[0] * e[1] * e[2] < nv_tile) {
                    scatter_pitch<DP>(e[0], e[1], P, Q);
                    if (Q * e[2] * words + rec_floats <= t.cap) box.wsc = 1;
                }
            }
            if (!box.wsc) {
                P = (e[0] + 3) & ~3LL;
                long long Pp = P + (((t.pmod - (int)(P & 31)) + 32) & 31);
                Q = (Pp * e[1] + 31) & ~31LL;
                if (Q * e[2] * words <= t.cap) {
                    P = Pp;
                } else {
                    Q = (P * e[1] + 3) & ~3LL;
                }
            }
            long long size = Q * e[2];
            const bool fits = e[0] <= 4096 && e[1] <= 4096 && e[2] <= 4096 && size * words <= t.cap;
            box.mode = fits ? 1 : 2;
            box.tma = 0;
            if (words == 1 && t.img_tma && interior == 7 && e[0] <= kTmaBoxX && e[1] <= kTmaBoxY &&
                e[2] <= kTmaBoxZ) {
                box.mode = 1;
                box.tma = 1;
                P = kTmaBoxX;
                Q = kTmaBoxX * kTmaBoxY;
                size = kTmaBoxFloats;
            }
            const bool staged = box.mode == 1;
            box.lo[0] = lo[0];
            box.lo[1] = lo[1];
            box.lo[2] = lo[2];
            box.xo = xo;
#pragma unroll
            for (int k = 0; k < 3; ++k) box.ext[k] = staged ? (int)e[k] : 0;
            box.P = staged ? (int)P : 0;
            box.Q = staged ? (int)Q : 0;
            box.size = staged ? (int)size : 0;
            box.interior = interior;
        }
        }
    }
    __syncthreads();
}

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}

__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem_src) : "memory");
}

// Rows of the box are distributed over warps; within a warp a group of `lpr`
// lanes (a power of two) shares a row.
struct RowWalk {
    int lg, sub, e0;   // lanes per row = 1 << lg
    int ry, rz;        // this lane group's current row
    int sy, sz;        // row step split into (y, z) parts
    int ey;
    __device__ __forceinline__ RowWalk(int items_per_row, int ey_) {
        const int n = items_per_row < 1 ? 1 : (items_per_row > 32 ? 32 : items_per_row);
        lg = 32 - __clz(n - 1);                       // ceil(log2 n)
        const int lane = threadIdx.x & 31;
        sub = lane >> lg;
        e0 = lane & ((1 << lg) - 1);
        ey = ey_;
        const int first = (threadIdx.x >> 5) * (32 >> lg) + sub;
        const int step = (kThreads / 32) * (32 >> lg);
        rz = first / ey;
        ry = first - rz * ey;
        sz = step / ey;
        sy = step - sz * ey;
    }
    __device__ __forceinline__ int lpr() const { return 1 << lg; }
    __device__ __forceinline__ void next() {
        ry += sy;
        rz += sz;
        if (ry >= ey) {
            ry -= ey;
            ++rz;
        }
    }
};

// Folded walk over the box: fn(sm_index, global_index, sign) once per element.
template <typename IT, class FN>
__device__ __forceinline__ void walk_box(const Box& box, const Geometry& g, int b0, int b1, int b2, FN fn) {
    const int ex = box.ext[0], ey = box.ext[1], ez = box.ext[2];
    RowWalk rw(ex, ey);
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);
    const bool xin = box.interior & 1, yin = box.interior & 2, zin = box.interior & 4;
    for (; rw.rz < ez; rw.next()) {
        const int rz = rw.rz, ry = rw.ry;
        float sgy = 1.f, sgz = 1.f;
        const IT gy = yin ? (IT)(box.lo[1] + ry) : (IT)fold_tap(b1, (long long)box.lo[1] + ry, g.d0[1], sgy);
        const IT gz = zin ? (IT)(box.lo[2] + rz) : (IT)fold_tap(b2, (long long)box.lo[2] + rz, g.d0[2], sgz);
        const IT rowg = gz * sz + gy * sy;
        const int rsm = rz * box.Q + ry * box.P;
        const float syz = sgy * sgz;
        if (xin) {
            const IT base = rowg + (IT)box.xo;
            for (int e = rw.e0; e < ex; e += rw.lpr()) fn(rsm + e, base + (IT)e, syz);
        } else {
            for (int e = rw.e0; e < ex; e += rw.lpr()) {
                float sgx;
                const IT gx = (IT)fold_tap(b0, (long long)box.xo + e, g.d0[0], sgx);
                fn(rsm + e, rowg + gx, syz * sgx);
            }
        }
    }
}

// Stage one channel of the image box into shared memory without waiting: the
// caller commits the cp.async group and waits for it before the box is read
// (the pull kernels overlap the next tile's staging with this tile's work).
// Interior boxes of a 16-byte aligned image with d0[0] % 4 == 0 copy whole
// 16-byte row chunks; other boxes fold (and sign) per element.
template <typename IT>
__device__ __forceinline__ void stage_box(const Box& box, const Geometry& g, int b0, int b1, int b2,
                                          const float* f0, float* sm) {
    if (box.interior == 7 && (g.d0[0] & 3) == 0 && (reinterpret_cast<uintptr_t>(f0) & 15) == 0) {
        const int ey = box.ext[1], ez = box.ext[2];
        const int n4 = (box.ext[0] + 3) >> 2;
        RowWalk rw(n4, ey);
        const IT sy = (IT)g.d0[0];
        const IT sz = (IT)(g.d0[0] * g.d0[1]);
        for (; rw.rz < ez; rw.next()) {
            const int rz = rw.rz, ry = rw.ry;
            const float* src = f0 + ((IT)(box.lo[2] + rz) * sz + (IT)(box.lo[1] + ry) * sy + (IT)box.xo);
            float* dst = sm + (rz * box.Q + ry * box.P);
            for (int ch = rw.e0; ch < n4; ch += rw.lpr()) cp_async16(dst + 4 * ch, src + 4 * ch);
        }
        return;
    }
    // folded boxes: elements with sign +1 are copied asynchronously as well;
    // mirrored DST-II elements (sign -1 or 0) are loaded and signed here
    walk_box<IT>(box, g, b0, b1, b2, [&](int si, IT gi, float s) {
        if (s == 1.f) cp_async4(sm + si, f0 + gi);
        else sm[si] = s * __ldg(f0 + gi);
    });
}

// ---- push accumulation -----------------------------------------------------
// Each box element holds two int32 words (hi, lo) of a fixed-point sum.  With
// S >= the sum of |contribution| over the tile's channel (B-spline weights are
// non-negative and sum to one per axis; derivative weights sum to at most 2 in
// absolute value) and S < 2^E, a contribution c is split as
//     c = hi * q1 + lo * q2 + rounding,  q1 = 2^(E-22), q2 = 2^(E-43),
// |hi| <= 2^22 and |lo| <= 2^20, so 512 contributions per element cannot
// overflow and the rounding error per element is at most 2^(E-35), i.e.
// below 3e-11 of S.  Both words use native integer shared atomics.  Where E
// is out of range (S = 0, non-finite, or extreme) the tile uses float atomics.
constexpr float kMagic = 12582912.0f;     // 1.5 * 2^23: float -> nearest int for |y| <= 2^22
constexpr int kMagicBits = 0x4B400000;

__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }   // -126 <= k <= 127

struct FixedScale {
    float inv_q1, q1, inv_q2, q2;
    __device__ __forceinline__ void set(int E) {
        inv_q1 = pow2f(22 - E);
        q1 = pow2f(E - 22);
        inv_q2 = pow2f(43 - E);
        q2 = pow2f(E - 43);
    }
};

__device__ __forceinline__ float fixed_value(int h, int l, const FixedScale& fs) {
    return fmaf(__int2float_rn(h), fs.q1, __int2float_rn(l) * fs.q2);
}

// Flush one channel's accumulator box into the image with global reductions:
// interior rows of an aligned image use 4-wide vector reductions on aligned
// groups, all-zero groups are skipped.  `val(si)` reads box element si.
template <typename IT, class VAL>
__device__ __forceinline__ void flush_box(const Box& box, const Geometry& g, int b0, int b1, int b2, float* f0,
                                          VAL val) {
    if ((box.interior & 1) && (g.d0[0] & 3) == 0 && (reinterpret_cast<uintptr_t>(f0) & 15) == 0) {
        const int ey = box.ext[1], ez = box.ext[2];
        const int n4 = (box.ext[0] + 3) >> 2;        // rows start at xo (16-byte aligned); whole groups
        RowWalk rw(n4, ey);
        const IT sy = (IT)g.d0[0];
        const IT sz = (IT)(g.d0[0] * g.d0[1]);
        for (; rw.rz < ez; rw.next()) {
            const int rz = rw.rz, ry = rw.ry;
            float sgy = 1.f, sgz = 1.f;
            const IT gy = (box.interior & 2) ? (IT)(box.lo[1] + ry)
                                             : (IT)fold_tap(b1, (long long)box.lo[1] + ry, g.d0[1], sgy);
            const IT gz = (box.interior & 4) ? (IT)(box.lo[2] + rz)
                                             : (IT)fold_tap(b2, (long long)box.lo[2] + rz, g.d0[2], sgz);
            const float s = sgy * sgz;
            float* grow = f0 + (gz * sz + gy * sy + (IT)box.xo);
            const int rsm = rz * box.Q + ry * box.P;
            for (int ch = rw.e0; ch < n4; ch += rw.lpr()) {
                const int e = 4 * ch;
                // elements past the box row (e >= ext) are zero in the accumulator
                const float4 v = make_float4(s * val(rsm + e), s * val(rsm + e + 1), s * val(rsm + e + 2),
                                             s * val(rsm + e + 3));
                if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f)
                    atomicAdd(reinterpret_cast<float4*>(grow + e), v);
            }
        }
        return;
    }
    walk_box<IT>(box, g, b0, b1, b2, [&](int si, IT gi, float s) {
        const float v = val(si);
        if (v != 0.f) atomicAdd(f0 + gi, s * v);
    });
}

// Flush (and clear) a two-word fixed-point accumulator box into the image.
// Rows of an x-interior box of an aligned image go as 16-byte groups: both
// words of 4 elements in two 16-byte loads, cleared by two 16-byte stores, one
// 4-wide global reduction (all-zero groups skipped).  Other boxes: the
// element-wise walk.
template <typename IT>
__device__ __forceinline__ void flush_fixed(const Box& box, const Geometry& g, int b0, int b1, int b2, float* f0,
                                            int* acc_hi, int* acc_lo, const FixedScale& fs) {
    const bool vec = (box.interior & 1) && (g.d0[0] & 3) == 0 && (reinterpret_cast<uintptr_t>(f0) & 15) == 0 &&
                     ((box.P | box.Q | box.size) & 3) == 0;
    if (!vec) {
        flush_box<IT>(box, g, b0, b1, b2, f0, [&](int si) {
            const float v = fixed_value(acc_hi[si], acc_lo[si], fs);
            acc_hi[si] = 0;
            acc_lo[si] = 0;
            return v;
        });
        return;
    }
    const int ey = box.ext[1], ez = box.ext[2];
    const int n4 = (box.ext[0] + 3) >> 2;
    RowWalk rw(n4, ey);
    if (rw.e0 >= n4) return;   // lanes per row >= n4: at most one group of each row per thread
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);
    const int e = 4 * rw.e0;
    for (; rw.rz < ez; rw.next()) {
        const int rz = rw.rz, ry = rw.ry;
        const int si = rz * box.Q + ry * box.P + e;
        const int4 h = *reinterpret_cast<const int4*>(acc_hi + si);
        const int4 l = *reinterpret_cast<const int4*>(acc_lo + si);
        *reinterpret_cast<int4*>(acc_hi + si) = make_int4(0, 0, 0, 0);
        *reinterpret_cast<int4*>(acc_lo + si) = make_int4(0, 0, 0, 0);
        if ((h.x | h.y | h.z | h.w | l.x | l.y | l.z | l.w) == 0) continue;
        float sgy = 1.f, sgz = 1.f;
        const IT gy = (box.interior & 2) ? (IT)(box.lo[1] + ry)
                                         : (IT)fold_tap(b1, (long long)box.lo[1] + ry, g.d0[1], sgy);
        const IT gz = (box.interior & 4) ? (IT)(box.lo[2] + rz)
                                         : (IT)fold_tap(b2, (long long)box.lo[2] + rz, g.d0[2], sgz);
        const float sg = sgy * sgz;
        const float4 v = make_float4(sg * fixed_value(h.x, l.x, fs), sg * fixed_value(h.y, l.y, fs),
                                     sg * fixed_value(h.z, l.z, fs), sg * fixed_value(h.w, l.w, fs));
        atomicAdd(reinterpret_cast<float4*>(f0 + (gz * sz + gy * sy + (IT)box.xo) + e), v);
    }
}

// ---- tiles -----------------------------------------------------------------
struct TileOrigin {
    int b;            // batch
    int x0, y0, z0;   // first sample voxel of the tile
};

// linear tile index (x fastest, batch slowest) -> tile origin
__device__ __forceinline__ TileOrigin tile_origin(const TileGrid& t, int T) {
    const unsigned u = (unsigned)T;
    const unsigned q1 = (unsigned)(((unsigned long long)u * t.mx) >> t.sx);
    const unsigned q2 = (unsigned)(((unsigned long long)q1 * t.my) >> t.sy);
    const unsigned q3 = (unsigned)(((unsigned long long)q2 * t.mz) >> t.sz);
    TileOrigin r;
    r.x0 = (int)(u - q1 * (unsigned)t.ntx) << t.lx;
    r.y0 = (int)(q1 - q2 * (unsigned)t.nty) << t.ly;
    r.z0 = (int)(q2 - q3 * (unsigned)t.ntz) << t.lz;
    r.b = (int)q3;
    return r;
}

// This thread's tile-local voxel coordinates (fixed for the kernel's lifetime)
// and the sample-grid dimensions as 32-bit integers.
template <int V>
struct ThreadVox {
    int vx[V], vy[V], vz[V];
    int D0, D1, D2;
    __device__ __forceinline__ ThreadVox(const TileGrid& t, const Geometry& g) {
#pragma unroll
        for (int q = 0; q < V; ++q) {
            const int lin = threadIdx.x + q * kThreads;
            vx[q] = lin & ((1 << t.lx) - 1);
            vy[q] = (lin >> t.lx) & ((1 << t.ly) - 1);
            vz[q] = lin >> (t.lx + t.ly);
        }
        D0 = (int)g.d1[0];
        D1 = (int)g.d1[1];
        D2 = (int)g.d1[2];
    }
    // index() for a runtime slot lin = threadIdx.x + q * kThreads (no register arrays)
    template <typename IT>
    __device__ __forceinline__ IT index_lin(const TileOrigin& o, int lin, const TileGrid& t) const {
        const int gx = o.x0 + (lin & ((1 << t.lx) - 1));
        const int gy = o.y0 + ((lin >> t.lx) & ((1 << t.ly) - 1));
        const int gz = o.z0 + (lin >> (t.lx + t.ly));
        if (gx >= D0 || gy >= D1 || gz >= D2) return (IT)-1;
        return (IT)gx + (IT)D0 * ((IT)gy + (IT)D1 * (IT)gz);
    }
    // linear sample index of voxel q within its batch, or -1 outside the grid
    template <typename IT>
    __device__ __forceinline__ IT index(const TileOrigin& o, int q) const {
        const int gx = o.x0 + vx[q], gy = o.y0 + vy[q], gz = o.z0 + vz[q];
        if (gx >= D0 || gy >= D1 || gz >= D2) return (IT)-1;
        return (IT)gx + (IT)D0 * ((IT)gy + (IT)D1 * (IT)gz);
    }
};

template <int DP, int OP, typename IT>
__device__ __noinline__ void push_tile_fallback(const LaunchArgs& a, int b, long long v, float x0, float x1,
                                                float x2) {
    push_voxel_global<DP, OP, IT>(a, b, v, x0, x1, x2);
}

// ---- tile ring: per-tile deformation (and push values) several tiles ahead ----
//
// Slot k of the ring holds one tile laid out as [component][z][y][x] -- exactly
// the order of a 4-D TMA box (TX, TY, TZ, C) -- so the thread owning tile-local
// voxel `lin` reads component k at slot + k*NV + lin.  With TMA, thread 0 fills
// a slot with one bulk tensor copy per tensor that completes on the slot's
// mbarrier; without it (unaligned geometry) the threads fill it with plain loads.

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after `limit` clock cycles, records the failure in
// the device status word and returns false.  A kernel whose wait gave up skips
// its remaining work and returns; copies it had already issued may still land
// in its shared memory, so after a recorded timeout the context is suspect and
// the caller should treat its outputs as undefined.
constexpr long long kWaitCycles = 4000000000LL;   // about two seconds
__device__ __forceinline__ bool mbar_wait_limit(unsigned bar, unsigned parity, long long limit) {
    if (mbar_try(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try(bar, parity)) {
        if (clock64() - t0 > limit) {
            atomicOr(&g_device_status, kStatusWaitTimeout);
            return false;
        }
    }
    return true;
}
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
    return mbar_wait_limit(bar, parity, kWaitCycles);
}
__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap* map, unsigned bar, int x, int y, int z,
                                            int w) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
        : "memory");
}

struct Ring {
    float* base;       // first slot
    int slot_floats;   // floats per slot
    unsigned bars;     // shared address of the first mbarrier
};

// Fill ring slot (j % kStages) with tile T: deformation components 0..2 and
// NVAL value components of channel 0 of `vals` (layout (d1, NVAL, nc, nb); the
// push input, or the fused step's target).  Called by every thread.  AFF (the
// affine ops): the values only, the deformation part of the slot stays unused.
template <int V, int NVAL, bool TMA, typename IT, bool AFF = false>
__device__ __forceinline__ void ring_fill(const Ring& r, int j, int T, const LaunchArgs& a, const TileGrid& t,
                                          const ThreadVox<V>& tv, const CUtensorMap& phimap,
                                          const CUtensorMap& valmap, const float* vals) {
    constexpr int NV = kThreads * V;
    float* slot = r.base + (j % kStages) * r.slot_floats;
    const TileOrigin o = tile_origin(t, T);
    if constexpr (TMA) {
        if (threadIdx.x == 0) {
            const unsigned bar = r.bars + 8u * (j % kStages);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_expect_tx(bar, (unsigned)(((AFF ? 0 : 3) + NVAL) * NV * sizeof(float)));
            if constexpr (!AFF) tma_load_4d(smem_addr(slot), &phimap, bar, o.x0, o.y0, o.z0, 3 * o.b);
            if constexpr (NVAL > 0)
                tma_load_4d(smem_addr(slot + 3 * NV), &valmap, bar, o.x0, o.y0, o.z0, NVAL * a.g.nc * o.b);
        }
    } else {
        const long long n1 = a.g.n1;
        const float* phi = AFF ? nullptr : a.phi + (long long)o.b * 3 * n1;
        const float* val = vals + (long long)o.b * a.g.nc * NVAL * n1;
#pragma unroll
        for (int q = 0; q < V; ++q) {
            const int lin = threadIdx.x + q * kThreads;
            const IT v = tv.template index<IT>(o, q);
            if constexpr (!AFF) {
#pragma unroll
                for (int k = 0; k < 3; ++k) slot[k * NV + lin] = v < 0 ? 0.f : __ldg(phi + v + k * n1);
            }
#pragma unroll
            for (int k = 0; k < NVAL; ++k) slot[(3 + k) * NV + lin] = v < 0 ? 0.f : __ldg(val + v + k * n1);
        }
    }
}

template <bool TMA>
__device__ __forceinline__ bool ring_wait(const Ring& r, int j) {
    if constexpr (TMA) return mbar_wait(r.bars + 8u * (j % kStages), (unsigned)((j / kStages) & 1));
    return true;
}

// Sample positions of a tile's voxels: x = phi - 1 from the tile's ring slot,
// or (AFF, the affine ops) A * (i, j, k, 1) from the voxel's grid coordinates;
// either way with the validity test.
template <int NV, bool AFF>
struct TilePos {
    const float* slot;
    const AffineMap* A;
    int lx, ly;
    __device__ __forceinline__ bool operator()(const Geometry& g, const TileOrigin& o, int lin, float& x0, float& x1,
                                               float& x2) const {
        if constexpr (AFF) {
            const int gx = o.x0 + (lin & ((1 << lx) - 1));
            const int gy = o.y0 + ((lin >> lx) & ((1 << ly) - 1));
            const int gz = o.z0 + (lin >> (lx + ly));
            affine_position(*A, (float)gx, (float)gy, (float)gz, x0, x1, x2);
            return position_valid(x0, x1, x2, g);
        } else {
            return load_valid(slot[lin], slot[NV + lin], slot[2 * NV + lin], g, x0, x1, x2);
        }
    }
};

// First-tap bounds of this thread's valid voxels of a tile.
template <int DP, int V, typename IT, class POS>
__device__ __forceinline__ void tile_bounds_pos(const Geometry& g, const TileOrigin& o, const ThreadVox<V>& tv,
                                                const POS& pos, int (&mn)[3], int (&mx)[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        mn[k] = INT_MAX;
        mx[k] = INT_MIN;
    }
#pragma unroll
    for (int q = 0; q < V; ++q) {
        const int lin = threadIdx.x + q * kThreads;
        if (tv.template index<IT>(o, q) < 0) continue;
        float x[3];
        if (!pos(g, o, lin, x[0], x[1], x[2])) continue;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int f = first_tap32(x[k], DP);
            const int c = f < -kClamp ? -kClamp : (f > kClamp ? kClamp : f);
            mn[k] = min(mn[k], c);
            mx[k] = max(mx[k], c);
        }
    }
}

// ... of the tile whose deformation is in `slot`.
template <int DP, int V, typename IT>
__device__ __forceinline__ void tile_bounds(const Geometry& g, const TileOrigin& o, const ThreadVox<V>& tv,
                                            const float* slot, int (&mn)[3], int (&mx)[3]) {
    tile_bounds_pos<DP, V, IT>(g, o, tv, TilePos<kThreads * V, false>{slot, nullptr, 0, 0}, mn, mx);
}

// The patch contraction of contract() (pp_voxel.cuh) with the z loop rolled:
// the z weights rotate through slot 0 and `next()` advances the loader to the
// next plane, so only one plane of rows is in flight (a fully unrolled patch
// needs more registers than two resident CTAs per SM leave).  Rows are taken in
// pairs on the packed f32x2 pipe.  `row(j, f)` loads row j of the current plane
// into f[0..DP).
template <int OP, int DP, class WT, class ROW, class NEXT>
__device__ __forceinline__ void contract_rolled(const WT& ax, const WT& ay, WT az, ROW row, NEXT next,
                                                float (&r)[6]) {
    constexpr int ORD = op_order(OP);
    constexpr int NJ = OP == kPull ? 1 : (ORD == 1 ? 3 : 6);   // y-level accumulators
#pragma unroll
    for (int q = 0; q < 6; ++q) r[q] = 0.f;
    // x weights duplicated into f32x2 pairs once: rows are contracted two at a
    // time on the packed pipe (lane 0: row j, lane 1: row j + 1)
    float2 wx2[DP], dwx2[ORD >= 1 ? DP : 1], hwx2[ORD >= 2 ? DP : 1];
#pragma unroll
    for (int i = 0; i < DP; ++i) {
        wx2[i] = make_float2(ax.w[i], ax.w[i]);
        if constexpr (ORD >= 1) dwx2[i] = make_float2(ax.dw[i], ax.dw[i]);
        if constexpr (ORD >= 2) hwx2[i] = make_float2(ax.hw[i], ax.hw[i]);
    }
    // pull keeps two planes in flight; the derivative ops, with more
    // accumulators, one (two would need more registers than 2 CTAs/SM leave)
    constexpr int KU = OP == kPull ? 2 : 1;
#pragma unroll KU
    for (int k = 0; k < DP; ++k) {
        float2 J[NJ];
#pragma unroll
        for (int q = 0; q < NJ; ++q) J[q] = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j + 1 < DP; j += 2) {
            float fa[DP], fb[DP];
            row(j, fa);
            row(j + 1, fb);
            float2 I0 = make_float2(0.f, 0.f), I1 = I0, I2 = I0;
#pragma unroll
            for (int i = 0; i < DP; ++i) {
                const float2 f2 = make_float2(fa[i], fb[i]);
                I0 = __ffma2_rn(wx2[i], f2, I0);
                if constexpr (ORD >= 1) I1 = __ffma2_rn(dwx2[i], f2, I1);
                if constexpr (ORD >= 2) I2 = __ffma2_rn(hwx2[i], f2, I2);
            }
            const float2 wy = make_float2(ay.w[j], ay.w[j + 1]);
            if constexpr (OP == kPull) {
                J[0] = __ffma2_rn(wy, I0, J[0]);
            } else if constexpr (ORD == 1) {
                const float2 dwy = make_float2(ay.dw[j], ay.dw[j + 1]);
                J[0] = __ffma2_rn(wy, I1, J[0]);
                J[1] = __ffma2_rn(dwy, I0, J[1]);
                J[2] = __ffma2_rn(wy, I0, J[2]);
            } else {
                const float2 dwy = make_float2(ay.dw[j], ay.dw[j + 1]);
                const float2 hwy = make_float2(ay.hw[j], ay.hw[j + 1]);
                J[0] = __ffma2_rn(wy, I2, J[0]);
                J[1] = __ffma2_rn(hwy, I0, J[1]);
                J[2] = __ffma2_rn(wy, I0, J[2]);
                J[3] = __ffma2_rn(dwy, I1, J[3]);
                J[4] = __ffma2_rn(wy, I1, J[4]);
                J[5] = __ffma2_rn(dwy, I0, J[5]);
            }
        }
        if constexpr (DP & 1) {   // the last row alone, into lane 0
            constexpr int j = DP - 1;
            float f[DP];
            row(j, f);
            float i0 = 0.f, i1 = 0.f, i2 = 0.f;
#pragma unroll
            for (int i = 0; i < DP; ++i) {
                i0 = fmaf(ax.w[i], f[i], i0);
                if constexpr (ORD >= 1) i1 = fmaf(ax.dw[i], f[i], i1);
                if constexpr (ORD >= 2) i2 = fmaf(ax.hw[i], f[i], i2);
            }
            if constexpr (OP == kPull) {
                J[0].x = fmaf(ay.w[j], i0, J[0].x);
            } else if constexpr (ORD == 1) {
                J[0].x = fmaf(ay.w[j], i1, J[0].x);
                J[1].x = fmaf(ay.dw[j], i0, J[1].x);
                J[2].x = fmaf(ay.w[j], i0, J[2].x);
            } else {
                J[0].x = fmaf(ay.w[j], i2, J[0].x);
                J[1].x = fmaf(ay.hw[j], i0, J[1].x);
                J[2].x = fmaf(ay.w[j], i0, J[2].x);
                J[3].x = fmaf(ay.dw[j], i1, J[3].x);
                J[4].x = fmaf(ay.w[j], i1, J[4].x);
                J[5].x = fmaf(ay.dw[j], i0, J[5].x);
            }
        }
        float jv[NJ];
#pragma unroll
        for (int q = 0; q < NJ; ++q) jv[q] = J[q].x + J[q].y;
        if constexpr (OP == kPull) {
            r[0] = fmaf(az.w[0], jv[0], r[0]);
        } else if constexpr (ORD == 1) {
            r[0] = fmaf(az.w[0], jv[0], r[0]);
            r[1] = fmaf(az.w[0], jv[1], r[1]);
            r[2] = fmaf(az.dw[0], jv[2], r[2]);
            if constexpr (OP == kPullValGrad) r[3] = fmaf(az.w[0], jv[2], r[3]);
        } else {
            r[0] = fmaf(az.w[0], jv[0], r[0]);
            r[1] = fmaf(az.w[0], jv[1], r[1]);
            r[2] = fmaf(az.hw[0], jv[2], r[2]);
            r[3] = fmaf(az.w[0], jv[3], r[3]);
            r[4] = fmaf(az.dw[0], jv[4], r[4]);
            r[5] = fmaf(az.dw[0], jv[5], r[5]);
        }
#pragma unroll
        for (int i = 0; i + 1 < DP; ++i) {
            az.w[i] = az.w[i + 1];
            if constexpr (ORD >= 1) az.dw[i] = az.dw[i + 1];
            if constexpr (ORD >= 2) az.hw[i] = az.hw[i + 1];
        }
        next();
    }
}

// contract_rolled over the shared box: row (k, j) starts at p + k*Q4 + j*P4.
template <int OP, int DP, class WT>
__device__ __forceinline__ void contract_smem(const WT& ax, const WT& ay, const WT& az, unsigned p, unsigned P4,
                                              unsigned Q4, float (&r)[6]) {
    contract_rolled<OP, DP>(
        ax, ay, az, [&](int j, float (&f)[DP]) { lds_row<DP>(p + j * P4, f); }, [&]() { p += Q4; }, r);
}

// pull_voxel_global (pp_voxel.cuh) for the tiles whose box does not fit, inlined
// into the tiled kernels with the rolled contraction so that it costs them no
// registers (a call, or the fully unrolled global gather, made the whole
// kernel spill).
template <int DP, int OP_, typename IT>
__device__ __forceinline__ void pull_voxel_lean(const LaunchArgs& a, int b, long long v, float x0, float x1,
                                                float x2) {
    constexpr int OP = pull_base_op<OP_>();
    constexpr int ORD = op_order(OP);
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);
    float acc[3] = {0.f, 0.f, 0.f};
    Axis<DP, ORD, IT> ax, ay, az;
#pragma unroll 1
    for (int c = 0; c < g.nc; ++c) {
        int b0, b1, b2;
        bnd_code(a, c, b0, b1, b2);
        ax.setup(x0, g.dp[0], b0, g.d0[0], (IT)1);
        ay.setup(x1, g.dp[1], b1, g.d0[1], sy);
        az.setup(x2, g.dp[2], b2, g.d0[2], sz);
        const float* f0 = a.in + ((long long)b * g.nc + c) * g.n0;
        IT zo[DP];
#pragma unroll
        for (int i = 0; i < DP; ++i) zo[i] = az.off[i];
        float r[6];
        contract_rolled<OP, DP>(
            ax, ay, az,
            [&](int j, float (&f)[DP]) {
#pragma unroll
                for (int i = 0; i < DP; ++i) f[i] = __ldg(f0 + (zo[0] + ay.off[j] + ax.off[i]));
            },
            [&]() {
#pragma unroll
                for (int i = 0; i + 1 < DP; ++i) zo[i] = zo[i + 1];
            },
            r);
        if constexpr (pull_is_dot<OP_>()) dot_accumulate<OP_>(a, b, c, v, r, acc);
        else pull_store<OP>(pull_out<OP_>(a, b, c, v), n1, r);
    }
    if constexpr (pull_is_dot<OP_>()) {
        float* o = pull_out<OP_>(a, b, 0, v);
        o[0] = acc[0];
        o[n1] = acc[1];
        o[2 * n1] = acc[2];
    }
}

// push_voxel_global (pp_voxel.cuh) for plain push, inlined with the z loop
// rolled (weights and offsets rotate through slot 0) so that the fallback of the
// batched kernel pins no registers across a call.  The values are read with
// plain loads: the batched kernel wrote them earlier in the same launch.
template <int DP, typename IT>
__device__ __forceinline__ void push_voxel_lean(const LaunchArgs& a, int b, long long v, float x0, float x1,
                                                float x2) {
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);
#pragma unroll 1
    for (int c = 0; c < g.nc; ++c) {
        const float v0 = a.in[((long long)b * g.nc + c) * n1 + v];
        if (!finitef(v0)) continue;
        int b0, b1, b2;
        bnd_code(a, c, b0, b1, b2);
        Axis<DP, 0, IT> ax, ay, az;
        ax.setup(x0, g.dp[0], b0, g.d0[0], (IT)1);
        ay.setup(x1, g.dp[1], b1, g.d0[1], sy);
        az.setup(x2, g.dp[2], b2, g.d0[2], sz);
        float* f0 = a.out + ((long long)b * g.nc + c) * g.n0;
#pragma unroll 1
        for (int k = 0; k < DP; ++k) {
#pragma unroll
            for (int j = 0; j < DP; ++j) {
                const float cb = v0 * (ay.w[j] * az.w[0]);
#pragma unroll
                for (int i = 0; i < DP; ++i) atomicAdd(f0 + (az.off[0] + ay.off[j] + ax.off[i]), cb * ax.w[i]);
            }
#pragma unroll
            for (int i = 0; i + 1 < DP; ++i) {
                az.w[i] = az.w[i + 1];
                az.off[i] = az.off[i + 1];
            }
        }
    }
}

// A whole tile whose footprint box does not fit in shared memory: every voxel
// from global memory, all channels.
template <int DP, int OP, int V, typename IT>
__device__ __forceinline__ void pull_tile_global(const LaunchArgs& a, const TileOrigin& o, const ThreadVox<V>& tv,
                                                 const TileGrid& t, const float* slot) {
    constexpr int NV = kThreads * V;
#pragma unroll 1
    for (int q = 0; q < V; ++q) {
        const int lin = threadIdx.x + q * kThreads;
        const IT v = tv.template index_lin<IT>(o, lin, t);
        if (v < 0) continue;
        float x0, x1, x2;
        if (!load_valid(slot[lin], slot[NV + lin], slot[2 * NV + lin], a.g, x0, x1, x2))
            pull_voxel_nan<OP>(a, o.b, (long long)v);
        else
            pull_voxel_lean<DP, OP, IT>(a, o.b, (long long)v, x0, x1, x2);
    }
}

// Evaluate channel c of a tile for the pull family (dot ops accumulate into
// acc[q] and store after the last channel).
template <int DP, int OP_, int V, typename IT>
__device__ __forceinline__ void pull_compute(const LaunchArgs& a, const TileOrigin& o, const ThreadVox<V>& tv,
                                             const TileGrid& t, const float* slot, int c, const Box& box,
                                             const float* sm, float (&acc)[V][3]) {
    constexpr int OP = pull_base_op<OP_>();
    constexpr int NCOMP = pull_ncomp<OP_>();
    constexpr int NV = kThreads * V;
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const bool last = c == g.nc - 1;
    auto voxel = [&](int q) {
        const int lin = threadIdx.x + q * kThreads;
        const IT v = tv.template index_lin<IT>(o, lin, t);
        if (v < 0) return;
        float x0, x1, x2;
        if (!load_valid(slot[lin], slot[NV + lin], slot[2 * NV + lin], g, x0, x1, x2)) {
            if (!pull_is_dot<OP_>() || last) {
                float* out = pull_out<OP_>(a, o.b, c, (long long)v);
#pragma unroll
                for (int p = 0; p < NCOMP; ++p) out[(long long)p * n1] = qnan();
            }
            return;
        }
        if (box.mode != 1) return;   // mode 0: no valid voxel; mode 2 tiles never get here
        constexpr int ORD = op_order(OP);
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
        // acc[q] stays in registers only with a compile-time q
#pragma unroll
        for (int q = 0; q < V; ++q) voxel(q);
    } else {
        // one voxel at a time: interleaving the V voxels' patches needs more
        // registers than two resident CTAs per SM leave
#pragma unroll 1
        for (int q = 0; q < V; ++q) voxel(q);
    }
}

// Persistent, software-pipelined pull family.  CTA i walks tiles i, i+G, i+2G, ...
// (G = grid size).  The deformation of the next kStages tiles is in flight in the
// tile ring; while tile j is evaluated from one box buffer, the box of tile j+1
// is being staged into the other with cp.async.
template <int DP, int OP, int V, typename IT, bool TMA>
__global__ void __launch_bounds__(kThreads, 2) k_pull_tiled(const __grid_constant__ LaunchArgs a,
                                                            const __grid_constant__ TileGrid t,
                                                            const __grid_constant__ CUtensorMap phimap,
                                                            const __grid_constant__ CUtensorMap imgmap) {
    extern __shared__ __align__(128) float4 smem4[];
    constexpr int NV = kThreads * V;
    __shared__ int red[8][7];
    __shared__ Box boxm[2];
    __shared__ int s_abort;
    const Geometry& g = a.g;
    const int G = gridDim.x;
    const int T0 = blockIdx.x;
    if (T0 >= t.ntiles) return;
    const int ntl = (t.ntiles - T0 + G - 1) / G;
    const ThreadVox<V> tv(t, g);

    float* sm = reinterpret_cast<float*>(smem4);
    Ring ring;
    ring.base = sm;
    ring.slot_floats = 3 * NV;
    float* bufs = sm + kStages * 3 * NV;
    ring.bars = smem_addr(bufs + 2 * t.cap);
    const unsigned bbar = ring.bars + 8u * kStages;   // one mbarrier per box buffer (TMA-staged boxes)
    unsigned bphase = 0;                              // bit b: parity of buffer b's next TMA completion
    if (threadIdx.x == 0) {
        s_abort = 0;
        if (TMA) {
            for (int k = 0; k < kStages; ++k) mbar_init(ring.bars + 8u * k, 1);
        }
        mbar_init(bbar, 1);
        mbar_init(bbar + 8u, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    for (int j = 0; j < kStages && j < ntl; ++j)
        ring_fill<V, 0, TMA, IT>(ring, j, T0 + j * G, a, t, tv, phimap, phimap, a.in);
    if (!TMA) __syncthreads();

    // one TMA copy of channel c's fixed image window into buffer `buf` (thread 0)
    auto tma_box = [&](const Box& box, int b, int c, int buf) {
        if (threadIdx.x == 0) {
            const unsigned bar = bbar + 8u * buf;
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_expect_tx(bar, (unsigned)(kTmaBoxFloats * sizeof(float)));
            tma_load_4d(smem_addr(bufs + buf * t.cap), &imgmap, bar, box.xo, box.lo[1], box.lo[2], b * g.nc + c);
        }
    };
    // every thread: wait for buffer buf's TMA copy
    auto tma_wait = [&](int buf) {
        if (!mbar_wait(bbar + 8u * buf, (bphase >> buf) & 1u)) s_abort = 1;
        bphase ^= 1u << buf;
    };

    // box of tile j (its deformation must be in the ring), staged into buffer j & 1
    auto prepare = [&](int j) {
        const TileOrigin o = tile_origin(t, T0 + j * G);
        const float* slot = ring.base + (j % kStages) * ring.slot_floats;
        if (!ring_wait<TMA>(ring, j)) s_abort = 1;
        int mn[3], mx[3];
        tile_bounds<DP, V, IT>(g, o, tv, slot, mn, mx);
        reduce_box<DP>(mn, mx, t, g, 1, boxm[j & 1], red);
        if (boxm[j & 1].mode == 1) {
            if (boxm[j & 1].tma) {
                tma_box(boxm[j & 1], o.b, 0, j & 1);
            } else {
                int b0, b1, b2;
                bnd_code(a, 0, b0, b1, b2);
                stage_box<IT>(boxm[j & 1], g, b0, b1, b2, a.in + (long long)o.b * g.nc * g.n0,
                              bufs + (j & 1) * t.cap);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };

    prepare(0);
    for (int j = 0; j < ntl; ++j) {
        if (j + 1 < ntl) {
            prepare(j + 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        if (boxm[j & 1].tma) tma_wait(j & 1);   // the record was published by prepare(j)'s barrier
        __syncthreads();   // box j is in its buffer
        if (s_abort) break;
        const TileOrigin o = tile_origin(t, T0 + j * G);
        const float* slot = ring.base + (j % kStages) * ring.slot_floats;
        const Box& box = boxm[j & 1];
        float* buf = bufs + (j & 1) * t.cap;
        if (box.mode == 2) {
            pull_tile_global<DP, OP, V, IT>(a, o, tv, t, slot);
            __syncthreads();   // ring slot j is free
            if (j + kStages < ntl)
                ring_fill<V, 0, TMA, IT>(ring, j + kStages, T0 + (j + kStages) * G, a, t, tv, phimap, phimap, a.in);
            if (!TMA) __syncthreads();
            continue;
        }
        float acc[V][3];
#pragma unroll
        for (int q = 0; q < V; ++q) acc[q][0] = acc[q][1] = acc[q][2] = 0.f;
        pull_compute<DP, OP, V, IT>(a, o, tv, t, slot, 0, box, buf, acc);
        for (int c = 1; c < g.nc; ++c) {
            __syncthreads();   // channel c-1 reads of the buffer are done
            if (box.mode == 1) {
                if (box.tma) {
                    tma_box(box, o.b, c, j & 1);
                    tma_wait(j & 1);
                } else {
                    int b0, b1, b2;
                    bnd_code(a, c, b0, b1, b2);
                    stage_box<IT>(box, g, b0, b1, b2, a.in + ((long long)o.b * g.nc + c) * g.n0, buf);
                    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
                }
            }
            __syncthreads();
            if (s_abort) break;
            pull_compute<DP, OP, V, IT>(a, o, tv, t, slot, c, box, buf, acc);
        }
        if (s_abort) break;
        __syncthreads();   // ring slot j and buffer j & 1 are free
        if (j + kStages < ntl)
            ring_fill<V, 0, TMA, IT>(ring, j + kStages, T0 + (j + kStages) * G, a, t, tv, phimap, phimap, a.in);
        if (!TMA) __syncthreads();
    }
}

// Scatter one voxel into the push accumulator (box-relative first taps ox, oy, oz).
// FIXED: two int32 words per element (values pre-scaled to q1 units); otherwise float.
// WT: any weight set with w (and dw for push_grad) of DP taps.
template <int DP, int OP, bool FIXED, class WT>
__device__ __forceinline__ void push_scatter(const WT& wx, const WT& wy, const WT& wz, float v0, float v1, float v2,
                                             unsigned base, unsigned P4, unsigned Q4, unsigned lo_off) {
#pragma unroll
    for (int k = 0; k < DP; ++k) {
#pragma unroll
        for (int j = 0; j < DP; ++j) {
            float ca, cb;
            if constexpr (OP == kPushGrad) {
                ca = v0 * (wy.w[j] * wz.w[k]);
                cb = v1 * (wy.dw[j] * wz.w[k]) + v2 * (wy.w[j] * wz.dw[k]);
            } else {
                ca = 0.f;
                cb = v0 * (wy.w[j] * wz.w[k]);
            }
            const unsigned row = base + k * Q4 + j * P4;
            if constexpr (FIXED) {
                int h[DP], l[DP];
                // taps in pairs with the packed f32x2 pipe (each lane rounds exactly
                // like the scalar sequence of the odd tap below)
#pragma unroll
                for (int i = 0; i + 1 < DP; i += 2) {
                    float2 y2;
                    if constexpr (OP == kPushGrad)
                        y2 = __ffma2_rn(make_float2(ca, ca), make_float2(wx.dw[i], wx.dw[i + 1]),
                                        __fmul2_rn(make_float2(cb, cb), make_float2(wx.w[i], wx.w[i + 1])));
                    else
                        y2 = __fmul2_rn(make_float2(cb, cb), make_float2(wx.w[i], wx.w[i + 1]));
                    const float2 t1 = __fadd2_rn(y2, make_float2(kMagic, kMagic));
                    const float2 u = __fadd2_rn(t1, make_float2(-kMagic, -kMagic));
                    const float2 r = __ffma2_rn(u, make_float2(-1.f, -1.f), y2);
                    const float2 l2 = __ffma2_rn(r, make_float2(2097152.0f, 2097152.0f), make_float2(kMagic, kMagic));
                    h[i] = __float_as_int(t1.x) - kMagicBits;
                    h[i + 1] = __float_as_int(t1.y) - kMagicBits;
                    l[i] = __float_as_int(l2.x) - kMagicBits;
                    l[i + 1] = __float_as_int(l2.y) - kMagicBits;
                }
                if constexpr (DP & 1) {
                    constexpr int i = DP - 1;
                    float y;
                    if constexpr (OP == kPushGrad) y = fmaf(ca, wx.dw[i], cb * wx.w[i]);
                    else y = cb * wx.w[i];
                    // y in q1 units, |y| <= 2^22: hi = round(y), lo = round((y - hi) * 2^21)
                    const float t1 = __fadd_rn(y, kMagic);
                    const float r = __fsub_rn(y, __fsub_rn(t1, kMagic));
                    h[i] = __float_as_int(t1) - kMagicBits;
                    l[i] = __float_as_int(__fmaf_rn(r, 2097152.0f, kMagic)) - kMagicBits;
                }
                red_row_s32<DP>(row, h);
                red_row_s32<DP>(row + lo_off, l);
            } else {
#pragma unroll
                for (int i = 0; i < DP; ++i) {
                    float y;
                    if constexpr (OP == kPushGrad) y = fmaf(ca, wx.dw[i], cb * wx.w[i]);
                    else y = cb * wx.w[i];
                    red_shared_f32(row + 4u * i, y);
                }
            }
        }
    }
}

// Push ops and degrees that scatter one voxel per warp instruction: push and
// push_grad at DP = 3 and 4 (a degree-4 box would need pitches of 37 elements or
// more).
template <int DP, int OP>
__host__ __device__ constexpr bool warp_scatter() {
    return DP == 3 || DP == 4;
}

// float4 record arrays per voxel of the warp-cooperative scatter: push keeps
// x, y (times the scaled value) and z weights; push_grad keeps v0 dw_x, v1 w_x,
// v2 w_x (values scaled), then w_y, dw_y, w_z, dw_z.
template <int OP>
__host__ __device__ constexpr int scatter_records() {
    return OP == kPushGrad ? 7 : 3;
}

// Warp-cooperative scatter of a tile's recorded voxels into the fixed-point
// (or, when !fixed, float) accumulator: warp w takes voxels w, w + 8, ...; lane
// l of pass p adds tap t = 32 p + l of that voxel.  With the box pitches chosen
// by scatter_pitch the 32 reductions of a pass hit 32 distinct elements in 32
// distinct banks.
// Shared-memory reductions for the warp-cooperative scatter: no compiler memory
// barrier, so the record loads of the next voxels can be issued ahead of them
// (the records and the accumulator are disjoint; the phases are separated by
// __syncthreads).
__device__ __forceinline__ void red_s32_nb(unsigned a, int v) {
    asm volatile("red.shared.add.s32 [%0], %1;" ::"r"(a), "r"(v));
}
__device__ __forceinline__ void red_f32_nb(unsigned a, float v) {
    asm volatile("red.shared.add.f32 [%0], %1;" ::"r"(a), "f"(v));
}

template <int DP, int OP, int DPP, int NV>
__device__ __forceinline__ void warp_scatter_tile(const float* rec, const int* rb, int P, int Q, unsigned acc_base,
                                                  unsigned lo_off, bool fixed) {
    constexpr int T = DP * DP * DP;
    constexpr int PASSES = (T + 31) / 32;
    constexpr int NW = kThreads / 32;
    constexpr int U = OP == kPushGrad ? 1 : 2;   // voxels per warp iteration (registers)
    static_assert(NV % (U * NW) == 0, "whole warp iterations");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int ti[PASSES], tj[PASSES], tk[PASSES], off[PASSES];
#pragma unroll
    for (int p = 0; p < PASSES; ++p) {
        const int tt = p * 32 + lane < T ? p * 32 + lane : 0;
        ti[p] = tt % DP;
        tj[p] = (tt / DP) % DP;
        tk[p] = tt / (DP * DP);
        off[p] = ti[p] + P * tj[p] + Q * tk[p];
    }
    // U voxels per iteration: all record loads first, then the reductions
    for (int s0 = warp; s0 < NV; s0 += U * NW) {
        int bv[U];
        float y[U][PASSES];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int sidx = s0 + u * NW;
            bv[u] = rb[sidx];
            const float* R = rec + sidx * DPP;   // record array r of this voxel at R + r * DPP * NV
            constexpr int RS = DPP * NV;
            if constexpr (OP == kPushGrad) {
                // v0 dwx wy wz + v1 wx dwy wz + v2 wx wy dwz = wz (wy A + dwy B) + dwz (wy C)
#pragma unroll
                for (int p = 0; p < PASSES; ++p) {
                    const float A = R[ti[p]], B = R[RS + ti[p]], C = R[2 * RS + ti[p]];
                    const float Y = R[3 * RS + tj[p]], DY = R[4 * RS + tj[p]];
                    const float Z = R[5 * RS + tk[p]], DZ = R[6 * RS + tk[p]];
                    y[u][p] = fmaf(Z, fmaf(Y, A, DY * B), DZ * (Y * C));
                }
            } else {
#pragma unroll
                for (int p = 0; p < PASSES; ++p) y[u][p] = (R[ti[p]] * R[RS + tj[p]]) * R[2 * RS + tk[p]];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (bv[u] < 0) continue;   // warp-uniform: every lane read the same record
#pragma unroll
            for (int p = 0; p < PASSES; ++p) {
                if (p * 32 + lane >= T) continue;
                const unsigned a = acc_base + 4u * (unsigned)(bv[u] + off[p]);
                if (fixed) {
                    // y in q1 units, |y| <= 2^22: hi = round(y), lo = round((y - hi) * 2^21)
                    const float t1 = __fadd_rn(y[u][p], kMagic);
                    const float r = __fsub_rn(y[u][p], __fsub_rn(t1, kMagic));
                    red_s32_nb(a, __float_as_int(t1) - kMagicBits);
                    red_s32_nb(a + lo_off, __float_as_int(__fmaf_rn(r, 2097152.0f, kMagic)) - kMagicBits);
                } else {
                    red_f32_nb(a, y[u][p]);
                }
            }
        }
    }
}

// Persistent push family.  The ring holds each tile's deformation and its
// channel-0 values kStages tiles ahead; the tile scatters into the shared
// accumulator and flushes it with global reductions.  The flush clears every
// element it reads, so the accumulator is zero again for the next tile.
// AFF: the affine push -- positions A * (i, j, k, 1) from `aff`, no deformation.
template <int DP, int OP, int V, typename IT, bool TMA, bool AFF = false>
__global__ void __launch_bounds__(kThreads, 2) k_push_tiled(const __grid_constant__ LaunchArgs a,
                                                            const __grid_constant__ TileGrid t,
                                                            const __grid_constant__ CUtensorMap phimap,
                                                            const __grid_constant__ CUtensorMap valmap,
                                                            const __grid_constant__ AffineMap aff) {
    extern __shared__ __align__(128) float4 smem4[];
    constexpr int ORD = OP == kPushGrad ? 1 : 0;
    constexpr int NCOMP = OP == kPushGrad ? 3 : 1;
    constexpr int NV = kThreads * V;
    // contracted tiles of push and push_grad at degrees 2 and 3 scatter one voxel
    // per warp instruction (see kScatterQMask); other tiles and degrees one voxel
    // per thread
    constexpr bool WSC = warp_scatter<DP, OP>();
    constexpr int DPP = 4;   // record stride per axis (DP <= 4 under WSC)
    __shared__ int red[8][7];
    __shared__ float sred[8];
    __shared__ Box box;
    __shared__ int s_abort;
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const int G = gridDim.x;
    const int T0 = blockIdx.x;
    if (T0 >= t.ntiles) return;
    const int ntl = (t.ntiles - T0 + G - 1) / G;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const ThreadVox<V> tv(t, g);

    float* sm = reinterpret_cast<float*>(smem4);
    Ring ring;
    ring.base = sm;
    ring.slot_floats = (3 + NCOMP) * NV;
    float* accf = sm + kStages * (3 + NCOMP) * NV;
    ring.bars = smem_addr(accf + t.cap);
    // voxel records of the warp-cooperative scatter (contracted tiles only), at
    // the top of the accumulator budget: the float4 arrays of scatter_records,
    // then the box-relative first tap (-1: skip)
    constexpr int NREC = scatter_records<OP>();
    constexpr int kRec = (NREC * DPP + 1) * NV;
    float* rx = accf + (WSC ? t.cap - kRec : 0);
    int* rb = reinterpret_cast<int*>(rx + NREC * DPP * NV);
    for (int i = threadIdx.x; i < (t.cap >> 2); i += kThreads)
        reinterpret_cast<float4*>(accf)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (threadIdx.x == 0) {
        s_abort = 0;
        if (TMA) {
            for (int k = 0; k < kStages; ++k) mbar_init(ring.bars + 8u * k, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
    }
    __syncthreads();
    for (int j = 0; j < kStages && j < ntl; ++j)
        ring_fill<V, NCOMP, TMA, IT, AFF>(ring, j, T0 + j * G, a, t, tv, phimap, valmap, a.in);
    if (!TMA) __syncthreads();

    const unsigned acc_base = smem_addr(accf);
    for (int j = 0; j < ntl; ++j) {
        const TileOrigin o = tile_origin(t, T0 + j * G);
        const float* slot = ring.base + (j % kStages) * ring.slot_floats;
        if (!ring_wait<TMA>(ring, j)) s_abort = 1;
        const TilePos<NV, AFF> pos{slot, &aff, t.lx, t.ly};
        // deformation validity, first-tap bounds and the channel-0 scale bound
        int mn[3], mx[3];
        tile_bounds_pos<DP, V, IT>(g, o, tv, pos, mn, mx);
        float bound0 = 0.f;
#pragma unroll
        for (int q = 0; q < V; ++q) {
            const int lin = threadIdx.x + q * kThreads;
            float x0, x1, x2;
            if (tv.template index<IT>(o, q) < 0 ||
                !pos(g, o, lin, x0, x1, x2))
                continue;
            bool fin = true;
            float s1 = 0.f;
#pragma unroll
            for (int p = 0; p < NCOMP; ++p) {
                const float v = slot[(3 + p) * NV + lin];
                fin = fin && finitef(v);
                s1 += fabsf(v);
            }
            if (fin) bound0 += OP == kPushGrad ? 2.f * s1 : s1;
        }
        reduce_box<DP, WSC>(mn, mx, t, g, 2, box, red, bound0, NV, WSC ? kRec : 0);
        if (s_abort) break;
        if (box.mode == 2) {
#pragma unroll
            for (int q = 0; q < V; ++q) {
                const IT v = tv.template index<IT>(o, q);
                const int lin = threadIdx.x + q * kThreads;
                float x0, x1, x2;
                if (v >= 0 && pos(g, o, lin, x0, x1, x2))
                    push_tile_fallback<DP, OP, IT>(a, o.b, (long long)v, x0, x1, x2);
            }
        } else if (box.mode == 1) {
            const unsigned lo_off = 4u * (unsigned)box.size;
            int* acc_hi = reinterpret_cast<int*>(accf);
            int* acc_lo = acc_hi + box.size;
            const float* inb = a.in + (long long)o.b * g.nc * NCOMP * n1;
            // the box geometry in registers: the scatter's reductions are memory
            // barriers to the compiler, which would reload it from shared memory
            const int bxo = box.xo, by0 = box.lo[1], bz0 = box.lo[2], bP = box.P, bQ = box.Q;
            for (int c = 0; c < g.nc; ++c) {
                int b0, b1, b2;
                bnd_code(a, c, b0, b1, b2);
                int E = box.E;
                if (c > 0) {
                    // values of channel c straight from global memory, and their scale bound
                    float bound = 0.f;
#pragma unroll
                    for (int q = 0; q < V; ++q) {
                        const IT v = tv.template index<IT>(o, q);
                        const int lin = threadIdx.x + q * kThreads;
                        float x0, x1, x2;
                        if (v < 0 || !pos(g, o, lin, x0, x1, x2))
                            continue;
                        bool fin = true;
                        float s1 = 0.f;
#pragma unroll
                        for (int p = 0; p < NCOMP; ++p) {
                            const float vv = __ldg(inb + (long long)c * NCOMP * n1 + v + p * n1);
                            fin = fin && finitef(vv);
                            s1 += fabsf(vv);
                        }
                        if (fin) bound += OP == kPushGrad ? 2.f * s1 : s1;
                    }
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1) bound += __shfl_xor_sync(0xffffffffu, bound, off);
                    __syncthreads();   // the previous channel's flush is done
                    if (lane == 0) sred[warp] = bound;
                    __syncthreads();
                    float S = 0.f;
                    for (int w = 0; w < kThreads / 32; ++w) S += sred[w];
                    E = scale_exponent(S);
                }
                if (E == INT_MAX) continue;   // every value of this channel is zero or skipped
                const bool fixed = E != INT_MIN;
                FixedScale fs;
                fs.set(fixed ? E : 0);
                auto thread_scatter = [&]() {
#pragma unroll
                for (int q = 0; q < V; ++q) {
                    const IT v = tv.template index<IT>(o, q);
                    const int lin = threadIdx.x + q * kThreads;
                    float x0, x1, x2;
                    if (v < 0 || !pos(g, o, lin, x0, x1, x2)) continue;
                    float val[NCOMP];
                    bool fin = true;
#pragma unroll
                    for (int p = 0; p < NCOMP; ++p) {
                        val[p] = c == 0 ? slot[(3 + p) * NV + lin] : __ldg(inb + (long long)c * NCOMP * n1 + v + p * n1);
                        fin = fin && finitef(val[p]);
                    }
                    if (!fin) continue;
                    W3<DP, ORD> wx, wy, wz;
                    const int ox = spline_taps32<DP, ORD>(x0, wx.w, wx.dw, wx.hw) - bxo;
                    const int oy = spline_taps32<DP, ORD>(x1, wy.w, wy.dw, wy.hw) - by0;
                    const int oz = spline_taps32<DP, ORD>(x2, wz.w, wz.dw, wz.hw) - bz0;
                    const unsigned P4 = 4u * bP, Q4 = 4u * bQ;
                    const unsigned base = acc_base + 4u * (unsigned)(oz * bQ + oy * bP + ox);
                    const float sc = fixed ? fs.inv_q1 : 1.f;
                    const float w0 = val[0] * sc;
                    const float w1 = NCOMP > 1 ? val[NCOMP > 1 ? 1 : 0] * sc : 0.f;
                    const float w2 = NCOMP > 2 ? val[NCOMP > 2 ? 2 : 0] * sc : 0.f;
                    if (fixed) push_scatter<DP, OP, true>(wx, wy, wz, w0, w1, w2, base, P4, Q4, lo_off);
                    else push_scatter<DP, OP, false>(wx, wy, wz, w0, w1, w2, base, P4, Q4, lo_off);
                }
                };
                if constexpr (WSC) {
                if (box.wsc) {
                    const float sc = fixed ? fs.inv_q1 : 1.f;
                    // each thread records its own voxels ...
#pragma unroll
                    for (int q = 0; q < V; ++q) {
                        const IT v = tv.template index<IT>(o, q);
                        const int lin = threadIdx.x + q * kThreads;
                        int base = -1;
                        float x0, x1, x2;
                        if (v >= 0 && pos(g, o, lin, x0, x1, x2)) {
                            float val[NCOMP];
                            bool fin = true;
#pragma unroll
                            for (int p = 0; p < NCOMP; ++p) {
                                val[p] = c == 0 ? slot[(3 + p) * NV + lin]
                                                : __ldg(inb + (long long)c * NCOMP * n1 + v + p * n1);
                                fin = fin && finitef(val[p]);
                            }
                            if (fin) {
                                // one 16-byte store per record array (DPP = 4; unused taps 0),
                                // one axis at a time
                                auto w4 = [&](const float* w, float m) {
                                    return make_float4(w[0] * m, DP > 1 ? w[DP > 1 ? 1 : 0] * m : 0.f,
                                                       DP > 2 ? w[DP > 2 ? 2 : 0] * m : 0.f,
                                                       DP > 3 ? w[DP > 3 ? 3 : 0] * m : 0.f);
                                };
                                float4* R4 = reinterpret_cast<float4*>(rx) + lin;
                                W3<DP, ORD> wa;
                                const int ox = spline_taps32<DP, ORD>(x0, wa.w, wa.dw, wa.hw) - bxo;
                                if constexpr (OP == kPushGrad) {
                                    R4[0] = w4(wa.dw, val[0] * sc);
                                    R4[NV] = w4(wa.w, val[NCOMP > 1 ? 1 : 0] * sc);
                                    R4[2 * NV] = w4(wa.w, val[NCOMP > 2 ? 2 : 0] * sc);
                                } else {
                                    R4[0] = w4(wa.w, 1.f);
                                }
                                const int oy = spline_taps32<DP, ORD>(x1, wa.w, wa.dw, wa.hw) - by0;
                                if constexpr (OP == kPushGrad) {
                                    R4[3 * NV] = w4(wa.w, 1.f);
                                    R4[4 * NV] = w4(wa.dw, 1.f);
                                } else {
                                    R4[NV] = w4(wa.w, val[0] * sc);
                                }
                                const int oz = spline_taps32<DP, ORD>(x2, wa.w, wa.dw, wa.hw) - bz0;
                                if constexpr (OP == kPushGrad) {
                                    R4[5 * NV] = w4(wa.w, 1.f);
                                    R4[6 * NV] = w4(wa.dw, 1.f);
                                } else {
                                    R4[2 * NV] = w4(wa.w, 1.f);
                                }
                                base = oz * bQ + oy * bP + ox;
                            }
                        }
                        rb[lin] = base;
                    }
                    __syncthreads();   // records complete
                    // ... then every warp scatters whole voxels, one tap per lane
                    warp_scatter_tile<DP, OP, DPP, NV>(rx, rb, bP, bQ, acc_base, lo_off, fixed);
                } else {
                    thread_scatter();
                }
                } else {
                    thread_scatter();
                }
                __syncthreads();   // the scatter is complete
                float* f0 = a.out + ((long long)o.b * g.nc + c) * g.n0;
                if (fixed)
                    flush_fixed<IT>(box, g, b0, b1, b2, f0, acc_hi, acc_lo, fs);
                else
                    flush_box<IT>(box, g, b0, b1, b2, f0, [&](int si) {
                        const float v = accf[si];
                        accf[si] = 0.f;
                        return v;
                    });
            }
        }
        if constexpr (WSC) {
            if (box.mode == 1 && box.wsc) {   // the records sat in the accumulator budget: clear them
                __syncthreads();
                for (int i = threadIdx.x; i < kRec / 4; i += kThreads)
                    reinterpret_cast<float4*>(rx)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
        __syncthreads();   // ring slot j is free and the accumulator is clear
        if (j + kStages < ntl)
            ring_fill<V, NCOMP, TMA, IT, AFF>(ring, j + kStages, T0 + (j + kStages) * G, a, t, tv, phimap, valmap,
                                              a.in);
        if (!TMA) __syncthreads();
    }
}

// ---- fused forward + adjoint step ------------------------------------------
//
// loss = sum_{b,c,v} (pull(f_c, phi)[v] - g_c[v])^2, df = push(2 r), and
// dphi[v] = sum_c 2 r_c grad pull(f_c)[v]: the forward pull, the pull rrule's
// two cotangents (src/pushpull_pb.jl:11-18) and the loss of the differentiable
// step in one pass.  The image box is staged once per (tile, channel) and serves
// both the value and the gradient; delta = 2 r is scattered into the shared
// accumulator of the same box and flushed with global reductions.

// Per-voxel global-memory version of one channel (tiles whose box does not fit):
// returns the residual r and the gradient; scatters 2 r into df with atomics.
// Inlined, with the rolled contraction and a rolled z loop in the scatter, so
// that the fallback costs the tiled kernel no registers.
template <int DP, typename IT>
__device__ __forceinline__ float fused_voxel_global(const LaunchArgs& a, int b, int c, long long v, float x0,
                                                    float x1, float x2, float gv, float (&grad)[3]) {
    const Geometry& g = a.g;
    const IT sy = (IT)g.d0[0];
    const IT sz = (IT)(g.d0[0] * g.d0[1]);
    int b0, b1, b2;
    bnd_code(a, c, b0, b1, b2);
    Axis<DP, 1, IT> ax, ay, az;
    ax.setup(x0, g.dp[0], b0, g.d0[0], (IT)1);
    ay.setup(x1, g.dp[1], b1, g.d0[1], sy);
    az.setup(x2, g.dp[2], b2, g.d0[2], sz);
    const float* f0 = a.in + ((long long)b * g.nc + c) * g.n0;
    IT zo[DP];
#pragma unroll
    for (int i = 0; i < DP; ++i) zo[i] = az.off[i];
    float r[6];
    contract_rolled<kPullValGrad, DP>(
        ax, ay, az,
        [&](int j, float (&f)[DP]) {
#pragma unroll
            for (int i = 0; i < DP; ++i) f[i] = __ldg(f0 + (zo[0] + ay.off[j] + ax.off[i]));
        },
        [&]() {
#pragma unroll
            for (int i = 0; i + 1 < DP; ++i) zo[i] = zo[i + 1];
        },
        r);
    grad[0] = r[0];
    grad[1] = r[1];
    grad[2] = r[2];
    const float res = r[3] - gv;
    const float d = 2.f * res;
    if (finitef(d)) {
        float* df = a.out + ((long long)b * g.nc + c) * g.n0;
#pragma unroll 1
        for (int k = 0; k < DP; ++k) {
#pragma unroll
            for (int j = 0; j < DP; ++j) {
                const float cb = d * (ay.w[j] * az.w[0]);
#pragma unroll
                for (int i = 0; i < DP; ++i) atomicAdd(df + (az.off[0] + ay.off[j] + ax.off[i]), cb * ax.w[i]);
            }
#pragma unroll
            for (int i = 0; i + 1 < DP; ++i) {
                az.w[i] = az.w[i + 1];
                az.off[i] = az.off[i + 1];
            }
        }
    }
    return res;
}

template <int DP, int V, typename IT, bool TMA>
__global__ void __launch_bounds__(kThreads, DP <= 3 ? 3 : 2) k_fused_tiled(const __grid_constant__ LaunchArgs a,
                                                             const __grid_constant__ TileGrid t,
                                                             const __grid_constant__ CUtensorMap phimap,
                                                             const __grid_constant__ CUtensorMap gmap) {
    extern __shared__ __align__(128) float4 smem4[];
    constexpr int NV = kThreads * V;
    __shared__ int red[8][7];
    __shared__ float sred[8];
    __shared__ double dred[8];
    __shared__ Box boxm[2];
    __shared__ int s_abort;
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const int G = gridDim.x;
    const int T0 = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ntl = T0 < t.ntiles ? (t.ntiles - T0 + G - 1) / G : 0;
    const ThreadVox<V> tv(t, g);
    double loss = 0.0;

    float* sm = reinterpret_cast<float*>(smem4);
    Ring ring;
    ring.base = sm;
    ring.slot_floats = 4 * NV;                       // deformation + channel-0 target
    float* bufs = sm + kStages * 4 * NV;              // image box, double buffered
    float* accf = bufs + 2 * t.cap;                   // adjoint accumulator: 2 words per element
    ring.bars = smem_addr(accf + 2 * t.cap);
    for (int i = threadIdx.x; i < (2 * t.cap) >> 2; i += kThreads)
        reinterpret_cast<float4*>(accf)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (threadIdx.x == 0) {
        s_abort = 0;
        if (TMA) {
            for (int k = 0; k < kStages; ++k) mbar_init(ring.bars + 8u * k, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
    }
    __syncthreads();
    for (int j = 0; j < kStages && j < ntl; ++j)
        ring_fill<V, 1, TMA, IT>(ring, j, T0 + j * G, a, t, tv, phimap, gmap, a.up);
    if (!TMA) __syncthreads();

    // Box of tile j and the channel-0 scale bound: |r| <= max|f| + |g| because the
    // B-spline weights are non-negative and sum to one, so the sum of |2 r w|
    // over a voxel's taps is at most 2 (max|f| + |g|).
    auto prepare = [&](int j) {
        const TileOrigin o = tile_origin(t, T0 + j * G);
        const float* slot = ring.base + (j % kStages) * ring.slot_floats;
        if (!ring_wait<TMA>(ring, j)) s_abort = 1;
        int mn[3], mx[3];
        tile_bounds<DP, V, IT>(g, o, tv, slot, mn, mx);
        const float M = __uint_as_float(a.fmax[(long long)o.b * g.nc]);
        float bound = 0.f;
#pragma unroll
        for (int q = 0; q < V; ++q) {
            const int lin = threadIdx.x + q * kThreads;
            float x0, x1, x2;
            if (tv.template index<IT>(o, q) >= 0 &&
                load_valid(slot[lin], slot[NV + lin], slot[2 * NV + lin], g, x0, x1, x2))
                bound += 2.f * (M + fabsf(slot[3 * NV + lin]));
        }
        reduce_box<DP>(mn, mx, t, g, 1, boxm[j & 1], red, bound);
        if (boxm[j & 1].mode == 1) {
            int b0, b1, b2;
            bnd_code(a, 0, b0, b1, b2);
            stage_box<IT>(boxm[j & 1], g, b0, b1, b2, a.in + (long long)o.b * g.nc * g.n0, bufs + (j & 1) * t.cap);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };

    if (ntl > 0) prepare(0);
    const unsigned acc_base = smem_addr(accf);
    int* acc_hi = reinterpret_cast<int*>(accf);
    for (int j = 0; j < ntl; ++j) {
        if (j + 1 < ntl) {
            prepare(j + 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        __syncthreads();   // box j is in its buffer
        if (s_abort) break;
        const TileOrigin o = tile_origin(t, T0 + j * G);
        const float* slot = ring.base + (j % kStages) * ring.slot_floats;
        const Box& box = boxm[j & 1];
        float* buf = bufs + (j & 1) * t.cap;
        const unsigned lo_off = 4u * (unsigned)box.size;
        int* acc_lo = acc_hi + box.size;
        float dphi[V][3];
        unsigned valid = 0;
#pragma unroll
        for (int q = 0; q < V; ++q) dphi[q][0] = dphi[q][1] = dphi[q][2] = 0.f;
        for (int c = 0; c < g.nc; ++c) {
            int b0, b1, b2;
            bnd_code(a, c, b0, b1, b2);
            const float* gc = a.up + ((long long)o.b * g.nc + c) * n1;
            int E = box.E;
            if (c > 0) {
                __syncthreads();   // channel c-1 is done with the box and the accumulator
                if (box.mode == 1) {
                    stage_box<IT>(box, g, b0, b1, b2, a.in + ((long long)o.b * g.nc + c) * g.n0, buf);
                    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
                }
                const float M = __uint_as_float(a.fmax[(long long)o.b * g.nc + c]);
                float bound = 0.f;
#pragma unroll
                for (int q = 0; q < V; ++q) {
                    const IT v = tv.template index<IT>(o, q);
                    if (v >= 0 && (valid >> q & 1)) bound += 2.f * (M + fabsf(__ldg(gc + v)));
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) bound += __shfl_xor_sync(0xffffffffu, bound, off);
                if (lane == 0) sred[warp] = bound;
                __syncthreads();   // the box of channel c and every warp's bound are in
                float S = 0.f;
                for (int w = 0; w < kThreads / 32; ++w) S += sred[w];
                E = scale_exponent(S);
            }
            const bool fixed = E != INT_MIN && E != INT_MAX;
            FixedScale fs;
            fs.set(fixed ? E : 0);
#pragma unroll
            for (int q = 0; q < V; ++q) {
                const IT v = tv.template index<IT>(o, q);
                if (v < 0) continue;
                const int lin = threadIdx.x + q * kThreads;
                float x0, x1, x2;
                if (!load_valid(slot[lin], slot[NV + lin], slot[2 * NV + lin], g, x0, x1, x2)) {
                    loss += (double)qnan();   // pull is NaN here, and so is the loss
                    continue;
                }
                valid |= 1u << q;
                const float gv = c == 0 ? slot[3 * NV + lin] : __ldg(gc + v);
                float res, grad[3];
                if (box.mode == 1) {
                    W3<DP, 1> wx, wy, wz;
                    const int ox = spline_taps32<DP, 1>(x0, wx.w, wx.dw, wx.hw) - box.xo;
                    const int oy = spline_taps32<DP, 1>(x1, wy.w, wy.dw, wy.hw) - box.lo[1];
                    const int oz = spline_taps32<DP, 1>(x2, wz.w, wz.dw, wz.hw) - box.lo[2];
                    const unsigned P4 = 4u * box.P, Q4 = 4u * box.Q;
                    const unsigned off = 4u * (unsigned)(oz * box.Q + oy * box.P + ox);
                    const unsigned p = smem_addr(buf) + off;
                    float r[6];
                    contract_smem<kPullValGrad, DP>(wx, wy, wz, p, P4, Q4, r);
                    res = r[3] - gv;
                    grad[0] = r[0];
                    grad[1] = r[1];
                    grad[2] = r[2];
                    const float d = 2.f * res;
                    if (finitef(d) && E != INT_MAX) {
                        if (fixed)
                            push_scatter<DP, kPush, true>(wx, wy, wz, d * fs.inv_q1, 0.f, 0.f, acc_base + off, P4, Q4,
                                                          lo_off);
                        else
                            push_scatter<DP, kPush, false>(wx, wy, wz, d, 0.f, 0.f, acc_base + off, P4, Q4, lo_off);
                    }
                } else {
                    res = fused_voxel_global<DP, IT>(a, o.b, c, (long long)v, x0, x1, x2, gv, grad);
                }
                loss += (double)(res * res);
                const float d = 2.f * res;
                dphi[q][0] = fmaf(d, grad[0], dphi[q][0]);
                dphi[q][1] = fmaf(d, grad[1], dphi[q][1]);
                dphi[q][2] = fmaf(d, grad[2], dphi[q][2]);
            }
            __syncthreads();   // the scatter is complete
            if (box.mode == 1 && E != INT_MAX) {
                float* df = a.out + ((long long)o.b * g.nc + c) * g.n0;
                if (fixed)
                    flush_fixed<IT>(box, g, b0, b1, b2, df, acc_hi, acc_lo, fs);
                else
                    flush_box<IT>(box, g, b0, b1, b2, df, [&](int si) {
                        const float v = accf[si];
                        accf[si] = 0.f;
                        return v;
                    });
            }
        }
        // deformation cotangent of every sample voxel of the tile
        float* dp = a.out2 + (long long)o.b * 3 * n1;
#pragma unroll
        for (int q = 0; q < V; ++q) {
            const IT v = tv.template index<IT>(o, q);
            if (v < 0) continue;
            const bool ok = valid >> q & 1;
            dp[v] = ok ? dphi[q][0] : qnan();
            dp[v + n1] = ok ? dphi[q][1] : qnan();
            dp[v + 2 * n1] = ok ? dphi[q][2] : qnan();
        }
        __syncthreads();   // ring slot j, the box buffer and the accumulator are free
        if (j + kStages < ntl)
            ring_fill<V, 1, TMA, IT>(ring, j + kStages, T0 + (j + kStages) * G, a, t, tv, phimap, gmap, a.up);
        if (!TMA) __syncthreads();
    }
    // this CTA's loss partial
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
    if (lane == 0) dred[warp] = loss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) sum += dred[w];
        a.partial[blockIdx.x] = sum;
    }
}


#ifdef PP_TILED_BATCH
// ---- batched uneven workload ------------------------------------------------
//
// Tiles of all items form one queue; a CTA takes the next tile with an atomic
// counter (dynamic load balance over volumes of uneven size and degree),
// evaluates pull for the tile from its staged image box, writes f1, and pushes
// the same values through the same box into the shared accumulator, which it
// flushes into the item's output.  Shared memory is split into a fixed
// accumulator region (two words per element) and the image box.

template <int DP>
__device__ __forceinline__ void batch_tile(const BatchItem& it, int lt, float* sm, int cap, Box& box,
                                           int (&red)[8][7], float (&sred)[8]) {
    constexpr int V = 2;
    constexpr int NV = kThreads * V;
    const LaunchArgs& a = it.pull;
    const LaunchArgs& pb = it.push;
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const TileGrid& t = it.t;
    const ThreadVox<V> tv(t, g);
    const TileOrigin o = tile_origin(t, lt);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int accw = ((2 * cap / 3) + 3) & ~3;   // accumulator words (fixed region)
    float* accf = sm;
    float* fbox = sm + accw;

    float X[V][3];
    int iv[V];
    unsigned ok = 0;
    int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
#pragma unroll
    for (int q = 0; q < V; ++q) {
        iv[q] = tv.template index<int>(o, q);
        if (iv[q] < 0) continue;
        const float* phi = a.phi + iv[q];
        if (!load_valid(__ldg(phi), __ldg(phi + n1), __ldg(phi + 2 * n1), g, X[q][0], X[q][1], X[q][2])) continue;
        ok |= 1u << q;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int f = first_tap32(X[q][k], DP);
            const int cl = f < -kClamp ? -kClamp : (f > kClamp ? kClamp : f);
            mn[k] = min(mn[k], cl);
            mx[k] = max(mx[k], cl);
        }
    }
    reduce_box<DP>(mn, mx, t, g, 3, box, red);   // 3 words per element: 2 accumulator + 1 image
    if (box.mode != 1) {
#pragma unroll
        for (int q = 0; q < V; ++q) {
            if (iv[q] < 0) continue;
            if (!(ok >> q & 1)) {
                pull_voxel_nan<kPull>(a, 0, iv[q]);
                continue;
            }
            pull_voxel_lean<DP, kPull, int>(a, 0, iv[q], X[q][0], X[q][1], X[q][2]);
            push_voxel_lean<DP, int>(pb, 0, iv[q], X[q][0], X[q][1], X[q][2]);
        }
        __syncthreads();   // box record reused by the next tile
        return;
    }
    const unsigned acc_base = smem_addr(accf);
    const unsigned lo_off = 4u * (unsigned)box.size;
    int* acc_hi = reinterpret_cast<int*>(accf);
    int* acc_lo = acc_hi + box.size;
    for (int c = 0; c < g.nc; ++c) {
        int b0, b1, b2;
        bnd_code(a, c, b0, b1, b2);
        stage_box<int>(box, g, b0, b1, b2, a.in + (long long)c * g.n0, fbox);
        asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();
        float val[V];
        float bound = 0.f;
        float* f1 = a.out + (long long)c * n1;
#pragma unroll
        for (int q = 0; q < V; ++q) {
            val[q] = 0.f;
            if (iv[q] < 0) continue;
            if (!(ok >> q & 1)) {
                f1[iv[q]] = qnan();
                continue;
            }
            W3<DP, 0> wx, wy, wz;
            const int ox = spline_taps32<DP, 0>(X[q][0], wx.w, wx.dw, wx.hw) - box.xo;
            const int oy = spline_taps32<DP, 0>(X[q][1], wy.w, wy.dw, wy.hw) - box.lo[1];
            const int oz = spline_taps32<DP, 0>(X[q][2], wz.w, wz.dw, wz.hw) - box.lo[2];
            const unsigned P4 = 4u * box.P, Q4 = 4u * box.Q;
            const unsigned p = smem_addr(fbox) + 4u * (unsigned)(oz * box.Q + oy * box.P + ox);
            float r[6];
            contract_smem<kPull, DP>(wx, wy, wz, p, P4, Q4, r);
            f1[iv[q]] = r[0];
            val[q] = r[0];
            if (finitef(r[0])) bound += fabsf(r[0]);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) bound += __shfl_xor_sync(0xffffffffu, bound, off);
        if (lane == 0) sred[warp] = bound;
        __syncthreads();   // bounds in; the image box is no longer read
        float S = 0.f;
        for (int w = 0; w < kThreads / 32; ++w) S += sred[w];
        const int E = scale_exponent(S);
        if (E != INT_MAX) {
            const bool fixed = E != INT_MIN;
            FixedScale fs;
            fs.set(fixed ? E : 0);
#pragma unroll
            for (int q = 0; q < V; ++q) {
                if (!(ok >> q & 1) || !finitef(val[q])) continue;
                W3<DP, 0> wx, wy, wz;
                const int ox = spline_taps32<DP, 0>(X[q][0], wx.w, wx.dw, wx.hw) - box.xo;
                const int oy = spline_taps32<DP, 0>(X[q][1], wy.w, wy.dw, wy.hw) - box.lo[1];
                const int oz = spline_taps32<DP, 0>(X[q][2], wz.w, wz.dw, wz.hw) - box.lo[2];
                const unsigned P4 = 4u * box.P, Q4 = 4u * box.Q;
                const unsigned base = acc_base + 4u * (unsigned)(oz * box.Q + oy * box.P + ox);
                if (fixed) push_scatter<DP, kPush, true>(wx, wy, wz, val[q] * fs.inv_q1, 0.f, 0.f, base, P4, Q4, lo_off);
                else push_scatter<DP, kPush, false>(wx, wy, wz, val[q], 0.f, 0.f, base, P4, Q4, lo_off);
            }
            __syncthreads();   // the scatter is complete
            float* out = pb.out + (long long)c * g.n0;
            if (fixed)
                flush_box<int>(box, g, b0, b1, b2, out, [&](int si) {
                    const float v = fixed_value(acc_hi[si], acc_lo[si], fs);
                    acc_hi[si] = 0;
                    acc_lo[si] = 0;
                    return v;
                });
            else
                flush_box<int>(box, g, b0, b1, b2, out, [&](int si) {
                    const float v = accf[si];
                    accf[si] = 0.f;
                    return v;
                });
        }
        __syncthreads();   // accumulator clear, image box and sred reusable
    }
}

// A tile of an item with per-dimension degrees: every voxel from global memory
// (runtime degree per axis), each channel pulled and its value pushed straight
// back with global atomics.
__device__ __noinline__ void batch_tile_any(const BatchItem& it, int lt) {
    constexpr int V = 2;
    const LaunchArgs& a = it.pull;
    const Geometry& g = a.g;
    const long long n1 = g.n1;
    const TileGrid& t = it.t;
    const ThreadVox<V> tv(t, g);
    const TileOrigin o = tile_origin(t, lt);
    const int sy = (int)g.d0[0], sz = (int)(g.d0[0] * g.d0[1]);
#pragma unroll 1
    for (int q = 0; q < V; ++q) {
        const int v = tv.template index<int>(o, q);
        if (v < 0) continue;
        const float* phi = a.phi + v;
        float x0, x1, x2;
        if (!load_valid(__ldg(phi), __ldg(phi + n1), __ldg(phi + 2 * n1), g, x0, x1, x2)) {
            pull_voxel_nan<kPull>(a, 0, v);
            continue;
        }
        Axis<0, 0, int> ax, ay, az;
        constexpr int N = Axis<0, 0, int>::N;
        int prev = -1;
#pragma unroll 1
        for (int c = 0; c < g.nc; ++c) {
            int b0, b1, b2;
            const int code = bnd_code(a, c, b0, b1, b2);
            if (code != prev) {
                ax.setup(x0, g.dp[0], b0, g.d0[0], 1);
                ay.setup(x1, g.dp[1], b1, g.d0[1], sy);
                az.setup(x2, g.dp[2], b2, g.d0[2], sz);
                prev = code;
            }
            const float* f0 = a.in + (long long)c * g.n0;
            float r[6];
            contract<kPull, N>(ax, ay, az, ax.n, ay.n, az.n, true,
                               [&](int k, int j, int i) { return __ldg(f0 + (az.off[k] + ay.off[j] + ax.off[i])); }, r);
            a.out[(long long)c * n1 + v] = r[0];
            if (!finitef(r[0])) continue;
            float* out = it.push.out + (long long)c * g.n0;
#pragma unroll 1
            for (int k = 0; k < az.n; ++k) {
#pragma unroll 1
                for (int j = 0; j < ay.n; ++j) {
                    const float cb = r[0] * (ay.w[j] * az.w[k]);
                    float* row = out + (az.off[k] + ay.off[j]);
#pragma unroll 1
                    for (int i = 0; i < ax.n; ++i) atomicAdd(row + ax.off[i], cb * ax.w[i]);
                }
            }
        }
    }
}

__global__ void __launch_bounds__(kThreads, 2) k_batch(const BatchItem* __restrict__ items, int nitems, int total,
                                                       unsigned* counter, int cap) {
    extern __shared__ __align__(128) float4 smem4[];
    __shared__ int red[8][7];
    __shared__ float sred[8];
    __shared__ Box box;
    __shared__ int s_tile;
    float* sm = reinterpret_cast<float*>(smem4);
    const int accw = ((2 * cap / 3) + 3) & ~3;
    for (int i = threadIdx.x; i < (accw >> 2); i += kThreads)
        reinterpret_cast<float4*>(sm)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int T = s_tile;
        __syncthreads();   // every thread has read the tile before the next claim
        if (T >= total) break;
        int lo = 0, hi = nitems - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (items[mid].tile_begin <= T) lo = mid;
            else hi = mid - 1;
        }
        const BatchItem& it = items[lo];
        const int lt = T - it.tile_begin;
        switch (it.dp) {
            case 0: batch_tile_any(it, lt); break;
            case 1: batch_tile<1>(it, lt, sm, cap, box, red, sred); break;
            case 2: batch_tile<2>(it, lt, sm, cap, box, red, sred); break;
            case 3: batch_tile<3>(it, lt, sm, cap, box, red, sred); break;
            case 4: batch_tile<4>(it, lt, sm, cap, box, red, sred); break;
            default: batch_tile<5>(it, lt, sm, cap, box, red, sred); break;
        }
    }
}
#endif  // PP_TILED_BATCH

TileGrid make_grid(const LaunchArgs& a, const TileCfg& c) {
    TileGrid t;
    t.lx = c.lx;
    t.ly = c.ly;
    t.lz = c.lz;
    t.ntx = (int)((a.g.d1[0] + (1 << c.lx) - 1) >> c.lx);
    t.nty = (int)((a.g.d1[1] + (1 << c.ly) - 1) >> c.ly);
    t.ntz = (int)((a.g.d1[2] + (1 << c.lz) - 1) >> c.lz);
    t.cap = c.cap;
    t.ntiles = t.ntx * t.nty * t.ntz * a.g.nb;
    auto magic = [](int d, unsigned long long& m, int& sh) {
        int l = 0;
        while ((1LL << l) < d) ++l;                        // l = ceil(log2 d)
        sh = 31 + l;
        m = ((1ULL << sh) + (unsigned long long)d - 1) / (unsigned long long)d;
    };
    magic(t.ntx, t.mx, t.sx);
    magic(t.nty, t.my, t.sy);
    magic(t.ntz, t.mz, t.sz);
    const int tx = 1 << c.lx;
    t.pmod = tx >= 32 ? 0 : tx;
    t.img_tma = 0;
    return t;
}

// Raise a kernel's dynamic shared-memory limit once per (device, kernel) to the
// largest size requested so far.
template <typename K>
cudaError_t opt_in(K kern, size_t smem) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> configured;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const auto key = std::make_pair(dev, reinterpret_cast<const void*>(kern));
    std::lock_guard<std::mutex> lk(mu);
    auto it = configured.find(key);
    if (it != configured.end() && it->second >= smem) return cudaSuccess;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured[key] = smem;
    return cudaSuccess;
}

// ---- TMA tensor maps (encoded on the host through the driver entry point) ----
using EncodeFn = PFN_cuTensorMapEncodeTiled_v12000;

EncodeFn encode_fn() {
    static std::once_flag once;
    static EncodeFn fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
    });
    return fn;
}

// 4-D map over a column-major volume stack (d0, d1, d2, planes) with a box of
// one tile (TX, TY, TZ, comps).  Requires a 16-byte aligned base and d0 % 4 == 0.
bool encode_tile_map(CUtensorMap* map, const float* base, const long long d[3], long long planes,
                     const TileGrid& t, int comps) {
    EncodeFn fn = encode_fn();
    if (!fn) return false;
    if ((reinterpret_cast<uintptr_t>(base) & 15) || (d[0] & 3) || (1 << t.lx) < 4) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)d[0], (cuuint64_t)d[1], (cuuint64_t)d[2], (cuuint64_t)planes};
    for (int k = 0; k < 4; ++k)
        if (dims[k] == 0 || dims[k] > (1ULL << 32)) return false;
    const cuuint64_t strides[3] = {(cuuint64_t)d[0] * 4, (cuuint64_t)(d[0] * d[1]) * 4,
                                   (cuuint64_t)(d[0] * d[1] * d[2]) * 4};
    for (int k = 0; k < 3; ++k)
        if (strides[k] >= (1ULL << 40)) return false;
    const cuuint32_t box[4] = {(cuuint32_t)(1 << t.lx), (cuuint32_t)(1 << t.ly), (cuuint32_t)(1 << t.lz),
                               (cuuint32_t)comps};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// Tensor map of an image (d0[0], d0[1], d0[2], planes) with the fixed
// kTmaBox* window as its box; false when TMA cannot address it (base or row
// stride not 16-byte aligned, dimensions out of range).
bool encode_box_map(CUtensorMap* map, const float* base, const long long d[3], long long planes) {
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
    const cuuint32_t box[4] = {(cuuint32_t)kTmaBoxX, (cuuint32_t)kTmaBoxY, (cuuint32_t)kTmaBoxZ, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

template <typename K, typename... Args>
cudaError_t launch_persistent(K kern, const TileGrid& t, size_t smem, cudaStream_t s, const Args&... args) {
    cudaError_t e = opt_in(kern, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long want = (long long)sm_count() * per_sm;
    const int grid = (int)(t.ntiles < want ? t.ntiles : want);
    kern<<<grid, kThreads, smem, s>>>(args...);
    return cudaGetLastError();
}

// AFF (push only): the affine push, positions from `aff` instead of a.phi.
template <int DP, int OP, int V, typename IT, bool PUSH, bool AFF = false>
cudaError_t launch_v(const LaunchArgs& a, const TileGrid& t, cudaStream_t s, const AffineMap& aff = AffineMap{}) {
    constexpr int NV = kThreads * V;
    CUtensorMap phimap, valmap;
    std::memset(&phimap, 0, sizeof phimap);
    std::memset(&valmap, 0, sizeof valmap);
    const long long nb = a.g.nb, nc = a.g.nc;
    bool tma = AFF || encode_tile_map(&phimap, a.phi, a.g.d1, 3 * nb, t, 3);
    if constexpr (PUSH) {
        constexpr int NCOMP = OP == kPushGrad ? 3 : 1;
        tma = tma && encode_tile_map(&valmap, a.in, a.g.d1, NCOMP * nc * nb, t, NCOMP);
        const size_t smem = (size_t)kStages * (3 + NCOMP) * NV * 4 + (size_t)t.cap * 4 + 8 * kStages;
        if (tma) return launch_persistent(k_push_tiled<DP, OP, V, IT, true, AFF>, t, smem, s, a, t, phimap, valmap, aff);
        return launch_persistent(k_push_tiled<DP, OP, V, IT, false, AFF>, t, smem, s, a, t, phimap, valmap, aff);
    } else {
        static_assert(!AFF, "affine pull runs on the warp-specialised kernels");
        // interior boxes as one TMA copy of a fixed window when the tile is 8 wide
        // (the window's row pitch is bank-conflict free for 8-wide warp tiles)
        CUtensorMap imgmap;
        std::memset(&imgmap, 0, sizeof imgmap);
        TileGrid tt = t;
        tt.img_tma = t.lx == 3 && t.cap >= kTmaBoxFloats && (t.cap & 31) == 0 &&
                     encode_box_map(&imgmap, a.in, a.g.d0, nc * nb);
        const size_t smem = (size_t)kStages * 3 * NV * 4 + 2 * (size_t)t.cap * 4 + 8 * kStages + 16;
        if (tma) return launch_persistent(k_pull_tiled<DP, OP, V, IT, true>, tt, smem, s, a, tt, phimap, imgmap);
        return launch_persistent(k_pull_tiled<DP, OP, V, IT, false>, tt, smem, s, a, tt, phimap, imgmap);
    }
}

template <int DP, int V, typename IT>
cudaError_t launch_fused_v(const LaunchArgs& a, const TileGrid& t, cudaStream_t s, int grid) {
    constexpr int NV = kThreads * V;
    CUtensorMap phimap, gmap;
    std::memset(&phimap, 0, sizeof phimap);
    std::memset(&gmap, 0, sizeof gmap);
    const long long nb = a.g.nb, nc = a.g.nc;
    const bool tma = encode_tile_map(&phimap, a.phi, a.g.d1, 3 * nb, t, 3) &&
                     encode_tile_map(&gmap, a.up, a.g.d1, nc * nb, t, 1);
    const size_t smem = (size_t)kStages * 4 * NV * 4 + 4 * (size_t)t.cap * 4 + 8 * kStages;
    cudaError_t e;
    if (tma) {
        auto k = k_fused_tiled<DP, V, IT, true>;
        if ((e = opt_in(k, smem)) != cudaSuccess) return e;
        k<<<grid, kThreads, smem, s>>>(a, t, phimap, gmap);
    } else {
        auto k = k_fused_tiled<DP, V, IT, false>;
        if ((e = opt_in(k, smem)) != cudaSuccess) return e;
        k<<<grid, kThreads, smem, s>>>(a, t, phimap, gmap);
    }
    return cudaGetLastError();
}

template <int DP, typename IT>
cudaError_t launch_fused_dp(const LaunchArgs& a, const TileCfg& c, cudaStream_t s, int grid) {
    const TileGrid t = make_grid(a, c);
    if ((1 << (c.lx + c.ly + c.lz)) > kThreads) return launch_fused_v<DP, 2, IT>(a, t, s, grid);
    return launch_fused_v<DP, 1, IT>(a, t, s, grid);
}

template <int DP, int OP, typename IT, bool PUSH, bool AFF = false>
cudaError_t launch_one(const LaunchArgs& a, const TileCfg& c, cudaStream_t s, const AffineMap& aff) {
    const TileGrid t = make_grid(a, c);
    const int vox = 1 << (c.lx + c.ly + c.lz);
    if (vox > kThreads) return launch_v<DP, OP, 2, IT, PUSH, AFF>(a, t, s, aff);
    return launch_v<DP, OP, 1, IT, PUSH, AFF>(a, t, s, aff);
}

template <int OP, typename IT, bool PUSH, bool AFF = false>
cudaError_t dispatch(const LaunchArgs& a, const TileCfg& t, cudaStream_t s, const AffineMap& aff = AffineMap{}) {
    switch (a.g.dp[0]) {
        case 1: return launch_one<1, OP, IT, PUSH, AFF>(a, t, s, aff);
        case 2: return launch_one<2, OP, IT, PUSH, AFF>(a, t, s, aff);
        case 3: return launch_one<3, OP, IT, PUSH, AFF>(a, t, s, aff);
        case 4: return launch_one<4, OP, IT, PUSH, AFF>(a, t, s, aff);
        default: return launch_one<5, OP, IT, PUSH, AFF>(a, t, s, aff);
    }
}

}  // namespace
}  // namespace pp
