/*
 * pp_oracle.h -- CPU restatement of PushPull.jl's B-spline pull / push.
 *
 * TEST INFRASTRUCTURE ONLY.  The shipped library never links or calls this
 * code.  Only the tests, the smoke check and the benchmark's CPU-baseline leg
 * load it, as the parity reference or as the timed CPU port.
 *
 * Layout and arguments follow the reference C ABI (artifacts/C/pushpull.h:1-14):
 * one (batch, channel) slice per call, column-major volumes, the deformation
 * planar with component k of voxel i at phi[i + k*n1], 1-based coordinates,
 * dp[k] = degree + 1, bnd[k] in {0 circulant, 1 DCT-II, 2 DST-II}.
 *
 * ora_*   FP64 oracle.  x = phi - 1 in float32, the validity mask and the
 *         integer first tap are computed exactly as the reference does, so
 *         NaN masks and degree-0 picks match bit for bit.  B-spline weights
 *         come from the closed form of the centred B-spline (truncated-power
 *         sum) evaluated in double, and every sum is taken in double.
 * port_*  FP32 port with the reference's signatures: float arithmetic, one
 *         voxel at a time, a per-tap boundary modulo and a local patch, the
 *         same work pattern as artifacts/C/pushpull.c.  It is the timed CPU
 *         baseline where the reference itself cannot be compiled.
 */
#ifndef PP_ORACLE_H
#define PP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned long long pp_usize;   /* USIZE_t, artifacts/C/cuheader.h:14 */

/* ---- FP64 oracle (outputs in double; push variants accumulate) ---------- */
void ora_pull (double *f1, const float *phi, const float *f0, const pp_usize *d0,
               pp_usize n1, const int *bnd, const pp_usize *dp, int ext);
void ora_pullg(double *g1, const float *phi, const float *f0, const pp_usize *d0,
               pp_usize n1, const int *bnd, const pp_usize *dp, int ext);
void ora_pullh(double *h1, const float *phi, const float *f0, const pp_usize *d0,
               pp_usize n1, const int *bnd, const pp_usize *dp, int ext);
void ora_push (double *f0, const float *phi, const float *f1, const pp_usize *d0,
               pp_usize n1, const int *bnd, const pp_usize *dp, int ext);
void ora_pushg(double *g0, const float *phi, const float *g1, const pp_usize *d0,
               pp_usize n1, const int *bnd, const pp_usize *dp, int ext);
/* one-voxel pull at an arbitrary (float32) 1-based position, for finite differences */
double ora_pull_at(const float pos[3], const float *f0, const pp_usize *d0,
                   const int *bnd, const pp_usize *dp, int ext);
/* affine sampling: x = A(i,j,k) with A already shifted to 0-based (pushpull.c:176-244) */
void ora_pull_affine(double *f1, const float *f0, const pp_usize *d0, pp_usize n1,
                     const pp_usize *d1, const float *A, const int *bnd,
                     const pp_usize *dp, int ext);
void ora_push_affine(double *f0, const float *f1, const pp_usize *d0, pp_usize n1,
                     const pp_usize *d1, const float *A, const int *bnd,
                     const pp_usize *dp, int ext);

/* ---- FP32 port (reference signatures, float outputs) -------------------- */
void port_pull (float *f1, const float *phi, const float *f0, const pp_usize *d0,
                pp_usize n1, const int *bnd, const pp_usize *dp, int ext);
void port_pullg(float *g1, const float *phi, const float *f0, const pp_usize *d0,
                pp_usize n1, const int *bnd, const pp_usize *dp, int ext);
void port_push (float *f0, const float *phi, const float *f1, const pp_usize *d0,
                pp_usize n1, const int *bnd, const pp_usize *dp, int ext);
void port_pushg(float *g0, const float *phi, const float *g1, const pp_usize *d0,
                pp_usize n1, const int *bnd, const pp_usize *dp, int ext);

#ifdef __cplusplus
}
#endif
#endif
