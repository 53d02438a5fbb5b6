/*
 * pushpull_gb300.h -- C ABI of the GB300 B-spline pull / push library.
 *
 * Two layers, both plain C types (no CUDA or torch types in any signature):
 *
 * 1. Native layer (pp_*): DEVICE pointers, the whole (channel, batch) set in
 *    one stream-ordered call, status codes.  This is what the CUDA-side
 *    binding calls: it replaces the CUDA.jl extension's per-(channel, batch)
 *    cudacall of the reference PTX kernels (ext/pushpull_gpu.jl:15-259) and its
 *    module-global __constant__ settings (ext/pushpull_gpu.jl:268-274, 380-383).
 *
 * 2. Compatibility layer: the exact symbols and signatures of the reference's
 *    CPU library (artifacts/C/pushpull.h:1-14, plus pullh at pushpull.c:70)
 *    on HOST pointers, one (channel, batch) slice per call, so the reference's
 *    own ccall sites (src/pushpull_cpu.jl:45, 100, 140, 195, 251, 294, 337)
 *    bind to this library unchanged.  Each call copies its inputs to the
 *    device, runs the GB300 kernel and copies the result back before returning.
 *
 * Array layout everywhere is the reference's Julia column-major layout:
 *   image      f   (d0[0], d0[1], d0[2], nc, nb)
 *   deformation phi (d1[0], d1[1], d1[2], 3, nb), 1-based voxel coordinates,
 *                   component k of voxel i at phi[i + k*n1]
 *   samples    f1  (d1[0], d1[1], d1[2], nc, nb)
 *   gradients  g   (d1[0], d1[1], d1[2], 3, nc, nb)
 *   Hessians   h   (d1[0], d1[1], d1[2], 3, 3, nc, nb)
 * Settings: deg[k] in 0..4 per dimension; boundary codes 0 circulant,
 * 1 reflect (DCT-II), 2 antisymmetric reflect (DST-II), three per channel
 * (nbnd == 1: one triple for every channel, nbnd == nc: one per channel);
 * ext 0/1 (src/pushpull_general.jl:15-60).
 *
 * Thread safety: native calls keep no state besides the thread-local error
 * string and are safe from any thread on any stream.  Compatibility calls use
 * a per-thread device workspace and stream.
 */
#ifndef PUSHPULL_GB300_H
#define PUSHPULL_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned long long pp_usize;   /* USIZE_t of artifacts/C/pushpull.h:1 */

enum pp_status {
    PP_OK = 0,
    PP_ERR_NULL = 1,          /* a required pointer is NULL                         */
    PP_ERR_DIMS = 2,          /* a dimension is zero where data is needed / overflow */
    PP_ERR_DEGREE = 3,        /* degree outside 0..4                                 */
    PP_ERR_BOUND = 4,         /* boundary code outside {0,1,2}                       */
    PP_ERR_CHANNELS = 5,      /* nc/nb < 1 or nbnd not in {1, nc}                    */
    PP_ERR_ALIGN = 6,         /* float pointer not 4-byte aligned                    */
    PP_ERR_CUDA = 7,          /* a CUDA runtime call failed                          */
    PP_ERR_UNSUPPORTED = 8,   /* request outside what this library supports          */
    PP_ERR_TOO_LARGE = 9,     /* request exceeds a fixed capacity                    */
    PP_ERR_TIMEOUT = 10       /* a bounded device-side wait gave up                  */
};

/* ------------------------------------------------------------------------ */
/* Native layer: device pointers, stream ordered (stream = cudaStream_t or 0) */
/* ------------------------------------------------------------------------ */

/* f1 = pull(f0, phi): replaces pull (src/pushpull_cpu.jl:17-53,
 * ext/pushpull_gpu.jl:15-51; per-voxel pull, artifacts/C/pushpull.c:14-33).
 * Invalid voxels (non-finite phi, or outside the band when ext == 0) get NaN. */
int pp_pull(float *f1, const float *phi, const float *f0,
            const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
            const int *bnd, int nbnd, const int deg[3], int ext, void *stream);

/* g1 = pull_grad(f0, phi), 3 planar components per channel: replaces pull_grad
 * (src/pushpull_cpu.jl:69-108, ext/pushpull_gpu.jl:66-101; pullg, pushpull.c:37-66). */
int pp_pull_grad(float *g1, const float *phi, const float *f0,
                 const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
                 const int *bnd, int nbnd, const int deg[3], int ext, void *stream);

/* h1 = pull_hess(f0, phi), symmetric 3x3 (9 planar components) per channel:
 * replaces pull_hess (src/pushpull_cpu.jl:111-148; pullh, pushpull.c:70-102). */
int pp_pull_hess(float *h1, const float *phi, const float *f0,
                 const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
                 const int *bnd, int nbnd, const int deg[3], int ext, void *stream);

/* dphi = sum_c up_c * grad pull(f0_c, phi), written as (d1[0], d1[1], d1[2], 3, nb):
 * the deformation cotangent of pull (rrule, src/pushpull_pb.jl:15-17: sum over
 * channels of delta .* pull_grad) and of push (:508-510 with up = f1 and f0 =
 * delta), computed without the (d1, 3, nc, nb) pull_grad temporary.
 * up has the layout of a pull output, (d1, nc, nb).  Invalid voxels get NaN. */
int pp_pull_grad_dot(float *dphi, const float *phi, const float *f0, const float *up,
                     const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
                     const int *bnd, int nbnd, const int deg[3], int ext, void *stream);

/* dphi[p] = sum_c sum_q H_c[p,q] up_c[q], H_c the Hessian of pull(f0_c, phi):
 * the deformation cotangent of pull_grad (rrule, src/pushpull_pb.jl:26-35,
 * sum over channels and q of delta .* pull_hess).  up has the layout of a
 * pull_grad output, (d1, 3, nc, nb); dphi is (d1, 3, nb). */
int pp_pull_hess_dot(float *dphi, const float *phi, const float *f0, const float *up,
                     const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
                     const int *bnd, int nbnd, const int deg[3], int ext, void *stream);

/* f0 (+)= push(f1, phi): replaces push (src/pushpull_cpu.jl:165-203,
 * ext/pushpull_gpu.jl:167-204; push, pushpull.c:106-123).  accumulate != 0 adds
 * into the caller's f0 (the reference contract: the caller zero-fills);
 * accumulate == 0 zeroes f0 on the stream first.  Non-finite f1 values and
 * invalid voxels are skipped. */
int pp_push(float *f0, const float *phi, const float *f1,
            const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
            const int *bnd, int nbnd, const int deg[3], int ext,
            int accumulate, void *stream);

/* g0 (+)= push_grad(g1, phi), the adjoint of pull_grad: replaces push_grad
 * (src/pushpull_cpu.jl:220-259, ext/pushpull_gpu.jl:221-259; pushg_element,
 * artifacts/C/pushpull.cu:145-163).  Voxels with a non-finite gradient
 * component are skipped. */
int pp_push_grad(float *g0, const float *phi, const float *g1,
                 const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
                 const int *bnd, int nbnd, const int deg[3], int ext,
                 int accumulate, void *stream);

/* f0 (+)= push(f1, phi) and c0 (+)= push(1, phi) in one pass: the count image
 * holds the (signed) weight each image voxel received, from the same voxels
 * as f0 (non-finite f1 values and invalid voxels contribute to neither).
 * Replaces pushc_element (artifacts/C/pushpull.cu:128-142; push1 with c0,
 * pushpull_dev.cu:140-154), which normalised multigrid restriction needs
 * (src/multigrid.jl:26-31 pushes the values, then ones).  c0 has the layout of
 * f0.  Per-voxel kernel with global reductions. */
int pp_push_count(float *f0, float *c0, const float *phi, const float *f1,
                  const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
                  const int *bnd, int nbnd, const int deg[3], int ext,
                  int accumulate, void *stream);

/* Fused forward + adjoint step of the loss sum((pull(f0, phi) - g)^2):
 *   *loss (device double) = sum over batch, channel and voxel of r^2, r = pull(f0, phi) - g
 *   df   (d0, nc, nb)  (+)= push(2 r, phi)               -- the f0 cotangent
 *   dphi (d1, 3, nb)     = sum_c 2 r_c grad pull(f0_c)    -- the phi cotangent
 * in one pass over phi, f0 and g.  Replaces the reference's differentiable
 * step built from pull, the pull rrule (src/pushpull_pb.jl:11-18: push and
 * pull_grad) and two broadcasts.  g has the layout of a pull output, (d1, nc, nb).
 * Invalid voxels make the loss NaN and their dphi NaN; non-finite residuals are
 * not pushed.  accumulate applies to df only.  The loss is reduced in a fixed
 * order and is reproducible from run to run.  Uses stream-ordered scratch (one
 * double per CTA, one float per image volume) from a memory pool this library
 * owns per device. */
int pp_fused_step(double *loss, float *df, float *dphi, const float *f0, const float *phi, const float *g,
                  const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
                  const int *bnd, int nbnd, const int deg[3], int ext, int accumulate, void *stream);

/* pp_fused_step for callers that must not allocate device memory.  No
 * counterpart in the reference: it exists for programs whose own caching
 * allocator already holds (nearly) all device memory, or whose request path
 * forbids allocation, so a library allocating scratch would fail or fragment
 * their pool.  Same arguments, results and errors as pp_fused_step; its
 * scratch is an 80 KiB array compiled into the library (every device that
 * loads the library keeps it until the process exits), so it calls no
 * allocator.  Limits: at most PP_NOALLOC_MAX_PARTIALS loss partials (one per
 * thread block: at most 1216 per batch element on 152 SMs) and at most
 * PP_NOALLOC_MAX_PLANES planes nc * nb; beyond them it returns
 * PP_ERR_TOO_LARGE without launching.  The first call on each device looks up
 * the array's device address, so make it before any stream capture.  All calls
 * share the one array: calls that overlap on the GPU (different streams or
 * host threads without ordering between them) race and give wrong losses. */
#define PP_NOALLOC_MAX_PARTIALS 8192
#define PP_NOALLOC_MAX_PLANES 4096
int pp_fused_step_noalloc(double *loss, float *df, float *dphi, const float *f0, const float *phi,
                          const float *g, const pp_usize d0[3], const pp_usize d1[3], int nc, int nb,
                          const int *bnd, int nbnd, const int deg[3], int ext, int accumulate, void *stream);

/* ---- affine resampling --------------------------------------------------- */
/* Pull / push through the affine map x = Aff * (i, j, k, 1) of sample voxel
 * (i, j, k) instead of a stored deformation.  Aff: HOST pointer to 12 floats,
 * the 3x4 column-major matrix already adjusted to 0-based indices (the
 * reference's adjust_affine, src/pushpull_cpu.jl:357-362); it is passed to the
 * kernel by value.  Positions are rounded exactly as the reference CPU code
 * (xj = Aff[3]*j + Aff[6]*k + Aff[9], then x = xj + Aff[0]*i).  Validity, NaN
 * and skipping rules as pp_pull / pp_push.  Isotropic degrees run on the tiled
 * kernels of pp_pull / pp_push with the positions computed in place (the tile
 * registry's pull and push entries decide, as for the deformation ops); other
 * settings on per-voxel kernels.  Replaces affine_pull_element /
 * affine_push_element (artifacts/C/pushpull.cu:187-231) and the per-slice
 * ccall loops of src/pushpull_cpu.jl:268-349. */
int pp_pull_affine(float *f1, const float *f0, const float *Aff, const pp_usize d0[3], const pp_usize d1[3],
                   int nc, int nb, const int *bnd, int nbnd, const int deg[3], int ext, void *stream);
int pp_push_affine(float *f0, const float *f1, const float *Aff, const pp_usize d0[3], const pp_usize d1[3],
                   int nc, int nb, const int *bnd, int nbnd, const int deg[3], int ext, int accumulate,
                   void *stream);

/* ---- batched uneven workload ------------------------------------------- */
/* One (image, deformation) pair of a batch: f1 = pull(f0, phi) is written and
 * out (+)= push(f1, phi) is accumulated, all device pointers, single batch.
 * Items may differ in size, channels, degrees and bounds (e.g. registration
 * pairs and their multigrid pyramid levels), as the reference's per-array
 * calls allow (src/pushpull_general.jl:33-54, ext/pushpull_gpu.jl:37-49).
 * Zero-initialised trailing fields keep the isotropic, one-triple form. */
typedef struct {
    const float *f0;      /* (d0, nc)     */
    const float *phi;     /* (d1, 3)      */
    float *f1;            /* (d1, nc)     */
    float *out;           /* (d0, nc)     */
    pp_usize d0[3], d1[3];
    int nc, deg;          /* channels; degree 0..4 in every dimension, or -1: per dimension in deg3 */
    int bnd[3], ext;      /* boundary codes (every channel unless nbnd > 1), extrapolate */
    int deg3[3];          /* per-dimension degrees when deg == -1 */
    int nbnd;             /* 0 or 1: bnd for every channel; nc: per-channel triples in bnds */
    const int *bnds;      /* host, 3 * nbnd codes (channel-major) when nbnd > 1 */
} pp_batch_item;

typedef struct pp_batch pp_batch;

/* Build a plan: item descriptors go to device memory once.  zero_outputs != 0
 * zeroes every out before each run.  No reference counterpart: the reference
 * loops over arrays and levels on the host (ext/pushpull_gpu.jl:37-49,
 * src/multigrid.jl:21-55). */
int pp_batch_create(pp_batch **plan, const pp_batch_item *items, int n, int zero_outputs);
/* Total tiles of the plan (the unit of work of its persistent launch). */
int pp_batch_tiles(const pp_batch *plan);
/* Run the plan: every tile of every item in one persistent launch (tiles are
 * claimed from a device work counter, balancing uneven items). */
int pp_batch_run(pp_batch *plan, void *stream);
/* Capture one run into a CUDA graph held by the plan (runs it once eagerly
 * first); pp_batch_launch replays the graph. */
int pp_batch_capture(pp_batch *plan, void *stream);
int pp_batch_launch(pp_batch *plan, void *stream);
void pp_batch_destroy(pp_batch *plan);

/* ---- kernel selection ------------------------------------------------- */
/* Ops for the tile registry. */
enum pp_op { PP_OP_PULL = 0, PP_OP_PULL_GRAD = 1, PP_OP_PULL_HESS = 2, PP_OP_PUSH = 3, PP_OP_PUSH_GRAD = 4,
             PP_OP_FUSED = 5 };
/* PP_PATH_AUTO: shared-memory tiled kernels where the degree is isotropic,
 * per-voxel global-memory kernels otherwise; PP_PATH_DIRECT: always the latter. */
enum pp_path { PP_PATH_AUTO = 0, PP_PATH_DIRECT = 1 };

/* Tile of sample voxels per CTA (2^lx x 2^ly x 2^lz, 32..512 voxels) and the
 * shared-memory budget of its image footprint box in floats, for one op
 * (-1: all ops) and one isotropic degree (-1: all degrees).  cap_floats == 0
 * selects the per-voxel kernels for that (op, degree); this is the default for
 * degree 0 and for the push family and the fused step at degree 1, where
 * gathering straight from L2 beats staging a box.  The code (lx, ly, lz) =
 * (3, 3, 4) selects, for pull, pull_grad and pull_hess (and through their
 * entries pull_grad_dot and pull_hess_dot), the
 * warp-specialised kernels (one producer warp streams the deformation and
 * stages footprint boxes by TMA while fifteen consumer warps evaluate 8x8x30
 * tiles; their box budget is fixed); it is the default at degrees 1..4.  No
 * reference counterpart (the reference launches one thread per voxel with no
 * tiling, ext/pushpull_gpu.jl:386-391); used by the autotuner. */
int pp_set_tile(int op, int deg, int lx, int ly, int lz, int cap_floats);
int pp_get_tile(int op, int deg, int *lx, int *ly, int *lz, int *cap_floats);
/* Autotuner: times the per-voxel kernels and every candidate tile shape and
 * shared-memory budget for op (PP_OP_PULL .. PP_OP_PUSH_GRAD) on the caller's
 * own arguments (same meaning as the op's entry point; push ops run with
 * accumulate = 0, so out is overwritten), reps timed runs each with CUDA
 * events, installs the fastest configuration for (op, deg[0]) (cap 0 when the
 * per-voxel kernels won) and returns best = {lx, ly, lz, cap, path} (path
 * PP_PATH_DIRECT when the per-voxel kernels were fastest) and its mean time in
 * ms.  Synchronises the stream. */
int pp_autotune(int op, float *out, const float *phi, const float *in, const pp_usize d0[3], const pp_usize d1[3],
                int nc, int nb, const int *bnd, int nbnd, const int deg[3], int ext, int reps, void *stream,
                int *best, float *best_ms);
/* Kernel family choice for all later calls in the process (PP_PATH_*). */
int pp_set_path(int path);

/* Message of the last failing call on this thread ("" when none). */
const char *pp_last_error(void);

/* Device status word of the current device (bit 0: a bounded device-side wait
 * gave up; such a kernel skips its remaining work and returns).  reset != 0
 * clears it.  Returns 0xffffffff if it cannot be read.  No reference
 * counterpart (the reference kernels never wait). */
unsigned pp_device_status(int reset);

/* Test of the timeout path of the bounded device-side waits: launches one warp
 * that waits on a shared-memory barrier nothing will complete, giving up after
 * limit_cycles SM clock cycles (1 .. 2^31, about a second at most).  The wait
 * records bit 0 of the device status word and the kernel returns normally, so
 * the context stays usable; read the bit with pp_device_status.  No reference
 * counterpart (the reference kernels never wait). */
int pp_test_bounded_wait(long long limit_cycles, void *stream);

/* Library version: major*10000 + minor*100 + patch. */
int pp_version(void);

/* ------------------------------------------------------------------------ */
/* Compatibility layer: the reference CPU ABI on HOST pointers                */
/* (artifacts/C/pushpull.h:3-14).  dp[k] = degree + 1; n1 = sample voxels.    */
/* On failure nothing is written, a message goes to stderr and to             */
/* pp_last_error().                                                           */
/* ------------------------------------------------------------------------ */
void pull (float *f1, const float *phi, const float *f0,
           const pp_usize *d0, const pp_usize n1, const int *bnd, const pp_usize *dp, const int ext);
void pullg(float *g1, const float *phi, const float *f0,
           const pp_usize *d0, const pp_usize n1, const int *bnd, const pp_usize *dp, const int ext);
void pullh(float *h1, const float *phi, const float *f0,
           const pp_usize *d0, const pp_usize n1, const int *bnd, const pp_usize *dp, const int ext);
void push (float *f0, const float *phi, const float *f1,
           const pp_usize *d0, const pp_usize n1, const int *bnd, const pp_usize *dp, const int ext);
void pushg(float *g0, const float *phi, const float *g1,
           const pp_usize *d0, const pp_usize n1, const int *bnd, const pp_usize *dp, const int ext);
/* artifacts/C/pushpull.h:11-14 (pushpull.c:176-243): Aff is the 3x4 column-major
 * matrix already adjusted to 0-based indices (src/pushpull_cpu.jl:357-362);
 * d1 = sample grid, n1 = d1[0]*d1[1]*d1[2]. */
void pull_affine(float *f1, const float *f0, const pp_usize *d0, const pp_usize n1,
                 const pp_usize *d1, const float *Aff, const int *bnd, const pp_usize *dp, const int ext);
void push_affine(float *f0, const float *f1, const pp_usize *d0, const pp_usize n1,
                 const pp_usize *d1, const float *Aff, const int *bnd, const pp_usize *dp, const int ext);

#ifdef __cplusplus
}
#endif
#endif /* PUSHPULL_GB300_H */
