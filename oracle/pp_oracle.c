/*
 * pp_oracle.c -- CPU restatement of PushPull.jl's B-spline pull / push.
 *
 * TEST INFRASTRUCTURE ONLY (see pp_oracle.h).  Reference files cited by path
 * within the PushPull.jl project.
 *
 * Semantics restated here (artifacts/C/pushpull.c, bspline.cu, patch.cu,
 * pushpull_dev.cu):
 *   x_k   = phi[i + k*n1] - 1.0f                      (float32, pushpull.c:24-26)
 *   valid = all x_k finite and, when ext == 0,
 *           -0.01f <= x_k <= (float)d0_k - 0.99f       (pushpull.c:6-9)
 *   first tap o_k = (int64) ceilf(x_k - 0.5f*dp_k)      (bspline.cu:66)
 *   taps o_k .. o_k+dp_k-1, each mapped into [0, d0_k) by the boundary rule
 *   with a sign (patch.cu:5-59): 0 circulant, 1 mirror (DCT-II), 2 mirror with
 *   a sign flip on the mirrored half (DST-II); any other code acts as 1.
 *   pull  = sum w_i w_j w_k s f0[tap]     invalid -> NaN  (pushpull_dev.cu:61-70)
 *   pullg = gradient of that sum in voxel units, NaN x3   (pushpull_dev.cu:73-88)
 *   pullh = 3x3 Hessian, 9 planar comps, NaN x9           (pushpull.c:70-102)
 *   push  = adjoint of pull; skips non-finite values and invalid voxels
 *           (pushpull.c:106-123)
 *   pushg = adjoint of pullg; skips invalid voxels and non-finite gradients.
 *           (The reference CPU pushg at pushpull.c:144 tests !ISFINITE(g[1]) and
 *           so adds nothing for finite input; its GPU twin, pushpull.cu:145-163,
 *           adds every valid voxel.  The restatement follows the evident intent.)
 */
#include "pp_oracle.h"

#include <math.h>
#include <stddef.h>
#include <string.h>

typedef long long pp_ssize;

#define MAXDP 5

/* ------------------------------------------------------------------------- */
/* shared index logic (kept in float exactly like the reference)             */
/* ------------------------------------------------------------------------- */

static int voxel_valid(const float x[3], const pp_usize *d0, int ext)
{
    int k;
    for (k = 0; k < 3; ++k)
        if (!isfinite(x[k])) return 0;
    if (ext) return 1;
    for (k = 0; k < 3; ++k) {
        float hi = (float)d0[k] - 0.99f;
        if (!(x[k] >= -0.01f && x[k] <= hi)) return 0;
    }
    return 1;
}

static pp_ssize first_tap(pp_usize dp, float x)
{
    float s = x - 0.5f * (float)dp;
    return (pp_ssize)ceilf(s);
}

/* map an unbounded tap index into [0, d) with a sign */
static pp_usize fold_index(int bnd, pp_ssize i, pp_usize d, int *sign)
{
    pp_ssize n = (pp_ssize)d, r;
    if (bnd == 0) {
        r = i % n;
        if (r < 0) r += n;
        *sign = 1;
        return (pp_usize)r;
    }
    r = i % (2 * n);
    if (r < 0) r += 2 * n;
    if (r < n) {
        *sign = 1;
        return (pp_usize)r;
    }
    *sign = (bnd == 2) ? -1 : 1;
    return (pp_usize)(2 * n - 1 - r);
}

/* ------------------------------------------------------------------------- */
/* FP64 oracle                                                                */
/* ------------------------------------------------------------------------- */

static const double kBinom[6][6] = {
    {1, 0, 0, 0, 0, 0},  {1, 1, 0, 0, 0, 0},  {1, 2, 1, 0, 0, 0},
    {1, 3, 3, 1, 0, 0},  {1, 4, 6, 4, 1, 0},  {1, 5, 10, 10, 5, 1}};
static const double kFact[5] = {1, 1, 2, 6, 24};

/* centred B-spline of degree n at u.  n = 0 uses the half-open box (-1/2, 1/2],
 * which is the convention the reference's first-tap rule implies.  n >= 1 uses
 * the truncated-power form
 *     beta_n(u) = 1/n! sum_k (-1)^k C(n+1,k) (u + (n+1)/2 - k)_+^n
 * evaluated on -|u| so that only the few leading terms are non-zero. */
static double bspline(int n, double u)
{
    double h, v, s = 0.0;
    int k, p;
    if (n < 0) return 0.0;
    if (n == 0) return (u > -0.5 && u <= 0.5) ? 1.0 : 0.0;
    h = 0.5 * (double)(n + 1);
    v = -fabs(u);
    if (v <= -h) return 0.0;
    for (k = 0; k <= n + 1; ++k) {
        double a = v + h - (double)k, an = 1.0;
        if (a <= 0.0) break;
        for (p = 0; p < n; ++p) an *= a;
        s += ((k & 1) ? -1.0 : 1.0) * kBinom[n + 1][k] * an;
    }
    return s / kFact[n];
}

typedef struct {
    int      dp;
    pp_ssize o;                 /* first (unbounded) tap */
    double   w[MAXDP], dw[MAXDP], hw[MAXDP];
    pp_usize idx[MAXDP];        /* folded tap index */
    double   sg[MAXDP];         /* boundary sign */
} axis64;

/* weights from derivative identities of the B-spline:
 *   beta_n'  = beta_{n-1}(u+1/2) - beta_{n-1}(u-1/2)
 *   beta_n'' = beta_{n-2}(u+1) - 2 beta_{n-2}(u) + beta_{n-2}(u-1)
 * degree 0 has zero derivatives and degree 1 a zero second derivative, as in
 * the reference (bspline.cu:154-156, 220-226).  Degree 1 (first derivative)
 * and degree 2 (second derivative) have piecewise-constant derivatives; for
 * them the reference's constants are used at every t, (-1, 1)
 * (bspline.cu:150-153) and (1, -2, 1) (bspline.cu:227-232), because the
 * identity would be evaluated on a knot of the lower-degree spline when float
 * rounding of a very large coordinate puts t on a knot (t = 0 for degree 1). */
static void axis64_setup(axis64 *a, int dp, float x, int bnd, pp_usize d)
{
    int k, n = dp - 1, sgn;
    double t;
    a->dp = dp;
    a->o  = first_tap((pp_usize)dp, x);
    t = (double)x - (double)a->o;
    for (k = 0; k < dp; ++k) {
        double u = t - (double)k;
        a->w[k]  = (n == 0) ? 1.0 : bspline(n, u);
        a->dw[k] = (n == 0) ? 0.0
                 : (n == 1) ? (k == 0 ? -1.0 : 1.0)
                 : bspline(n - 1, u + 0.5) - bspline(n - 1, u - 0.5);
        a->hw[k] = (n <= 1) ? 0.0
                 : (n == 2) ? (k == 1 ? -2.0 : 1.0)
                 : bspline(n - 2, u + 1.0) - 2.0 * bspline(n - 2, u) + bspline(n - 2, u - 1.0);
        a->idx[k] = fold_index(bnd, a->o + k, d, &sgn);
        a->sg[k]  = (double)sgn;
    }
}

static void load_x(float x[3], const float *phi, pp_usize i, pp_usize n1)
{
    x[0] = phi[i] - 1.0f;
    x[1] = phi[i + n1] - 1.0f;
    x[2] = phi[i + 2 * n1] - 1.0f;
}

static void setup3(axis64 ax[3], const float x[3], const int *bnd,
                   const pp_usize *dp, const pp_usize *d0)
{
    int k;
    for (k = 0; k < 3; ++k) axis64_setup(&ax[k], (int)dp[k], x[k], bnd[k], d0[k]);
}

/* sum over the patch of (a_i b_j c_k) s f0[tap]; selectors: 0 w, 1 dw, 2 hw */
static double patch_sum(const axis64 ax[3], const float *f0, const pp_usize *d0,
                        int si, int sj, int sk)
{
    const double *wi = si == 0 ? ax[0].w : si == 1 ? ax[0].dw : ax[0].hw;
    const double *wj = sj == 0 ? ax[1].w : sj == 1 ? ax[1].dw : ax[1].hw;
    const double *wk = sk == 0 ? ax[2].w : sk == 1 ? ax[2].dw : ax[2].hw;
    double acc = 0.0;
    int i, j, k;
    for (k = 0; k < ax[2].dp; ++k)
        for (j = 0; j < ax[1].dp; ++j) {
            pp_usize row = d0[0] * (ax[1].idx[j] + d0[1] * ax[2].idx[k]);
            double   wjk = wj[j] * wk[k] * ax[1].sg[j] * ax[2].sg[k];
            for (i = 0; i < ax[0].dp; ++i)
                acc += wi[i] * ax[0].sg[i] * wjk * (double)f0[row + ax[0].idx[i]];
        }
    return acc;
}

static void patch_scatter(const axis64 ax[3], double *f0, const pp_usize *d0,
                          const double g[3], int gradient)
{
    int i, j, k;
    for (k = 0; k < ax[2].dp; ++k)
        for (j = 0; j < ax[1].dp; ++j) {
            pp_usize row = d0[0] * (ax[1].idx[j] + d0[1] * ax[2].idx[k]);
            double   sjk = ax[1].sg[j] * ax[2].sg[k];
            for (i = 0; i < ax[0].dp; ++i) {
                double v;
                if (gradient)
                    v = g[0] * ax[0].dw[i] * ax[1].w[j] * ax[2].w[k]
                      + g[1] * ax[0].w[i] * ax[1].dw[j] * ax[2].w[k]
                      + g[2] * ax[0].w[i] * ax[1].w[j] * ax[2].dw[k];
                else
                    v = g[0] * ax[0].w[i] * ax[1].w[j] * ax[2].w[k];
                f0[row + ax[0].idx[i]] += v * ax[0].sg[i] * sjk;
            }
        }
}

void ora_pull(double *f1, const float *phi, const float *f0, const pp_usize *d0,
              pp_usize n1, const int *bnd, const pp_usize *dp, int ext)
{
    pp_usize i;
    for (i = 0; i < n1; ++i) {
        float  x[3];
        axis64 ax[3];
        load_x(x, phi, i, n1);
        if (!voxel_valid(x, d0, ext)) { f1[i] = NAN; continue; }
        setup3(ax, x, bnd, dp, d0);
        f1[i] = patch_sum(ax, f0, d0, 0, 0, 0);
    }
}

double ora_pull_at(const float pos[3], const float *f0, const pp_usize *d0,
                   const int *bnd, const pp_usize *dp, int ext)
{
    float  x[3];
    axis64 ax[3];
    x[0] = pos[0] - 1.0f;
    x[1] = pos[1] - 1.0f;
    x[2] = pos[2] - 1.0f;
    if (!voxel_valid(x, d0, ext)) return NAN;
    setup3(ax, x, bnd, dp, d0);
    return patch_sum(ax, f0, d0, 0, 0, 0);
}

void ora_pullg(double *g1, const float *phi, const float *f0, const pp_usize *d0,
               pp_usize n1, const int *bnd, const pp_usize *dp, int ext)
{
    pp_usize i;
    for (i = 0; i < n1; ++i) {
        float  x[3];
        axis64 ax[3];
        load_x(x, phi, i, n1);
        if (!voxel_valid(x, d0, ext)) {
            g1[i] = g1[i + n1] = g1[i + 2 * n1] = NAN;
            continue;
        }
        setup3(ax, x, bnd, dp, d0);
        g1[i]          = patch_sum(ax, f0, d0, 1, 0, 0);
        g1[i + n1]     = patch_sum(ax, f0, d0, 0, 1, 0);
        g1[i + 2 * n1] = patch_sum(ax, f0, d0, 0, 0, 1);
    }
}

void ora_pullh(double *h1, const float *phi, const float *f0, const pp_usize *d0,
               pp_usize n1, const int *bnd, const pp_usize *dp, int ext)
{
    pp_usize i;
    int c;
    for (i = 0; i < n1; ++i) {
        float  x[3];
        axis64 ax[3];
        double xx, yy, zz, xy, xz, yz;
        load_x(x, phi, i, n1);
        if (!voxel_valid(x, d0, ext)) {
            for (c = 0; c < 9; ++c) h1[i + (pp_usize)c * n1] = NAN;
            continue;
        }
        setup3(ax, x, bnd, dp, d0);
        xx = patch_sum(ax, f0, d0, 2, 0, 0);
        yy = patch_sum(ax, f0, d0, 0, 2, 0);
        zz = patch_sum(ax, f0, d0, 0, 0, 2);
        xy = patch_sum(ax, f0, d0, 1, 1, 0);
        xz = patch_sum(ax, f0, d0, 1, 0, 1);
        yz = patch_sum(ax, f0, d0, 0, 1, 1);
        /* column-major 3x3: entry (a,b) at component a + 3b */
        h1[i]          = xx;
        h1[i + 4 * n1] = yy;
        h1[i + 8 * n1] = zz;
        h1[i + 1 * n1] = h1[i + 3 * n1] = xy;
        h1[i + 2 * n1] = h1[i + 6 * n1] = xz;
        h1[i + 5 * n1] = h1[i + 7 * n1] = yz;
    }
}

void ora_push(double *f0, const float *phi, const float *f1, const pp_usize *d0,
              pp_usize n1, const int *bnd, const pp_usize *dp, int ext)
{
    pp_usize i;
    for (i = 0; i < n1; ++i) {
        float  x[3];
        axis64 ax[3];
        double g[3];
        if (!isfinite(f1[i])) continue;
        load_x(x, phi, i, n1);
        if (!voxel_valid(x, d0, ext)) continue;
        setup3(ax, x, bnd, dp, d0);
        g[0] = (double)f1[i];
        g[1] = g[2] = 0.0;
        patch_scatter(ax, f0, d0, g, 0);
    }
}

void ora_pushg(double *g0, const float *phi, const float *g1, const pp_usize *d0,
               pp_usize n1, const int *bnd, const pp_usize *dp, int ext)
{
    pp_usize i;
    for (i = 0; i < n1; ++i) {
        float  x[3];
        axis64 ax[3];
        double g[3];
        load_x(x, phi, i, n1);
        if (!voxel_valid(x, d0, ext)) continue;
        if (!isfinite(g1[i]) || !isfinite(g1[i + n1]) || !isfinite(g1[i + 2 * n1])) continue;
        setup3(ax, x, bnd, dp, d0);
        g[0] = (double)g1[i];
        g[1] = (double)g1[i + n1];
        g[2] = (double)g1[i + 2 * n1];
        patch_scatter(ax, g0, d0, g, 1);
    }
}

/* affine position of output voxel (i,j,k), float ops in the reference order
 * (pushpull.c:190-200) */
static void affine_x(float x[3], const float *A, pp_usize i, pp_usize j, pp_usize k)
{
    int c;
    for (c = 0; c < 3; ++c) {
        float xj = A[3 + c] * (float)j + A[6 + c] * (float)k + A[9 + c];
        x[c] = xj + A[c] * (float)i;
    }
}

void ora_pull_affine(double *f1, const float *f0, const pp_usize *d0, pp_usize n1,
                     const pp_usize *d1, const float *A, const int *bnd,
                     const pp_usize *dp, int ext)
{
    pp_usize i, j, k, ijk = 0;
    (void)n1;
    for (k = 0; k < d1[2]; ++k)
        for (j = 0; j < d1[1]; ++j)
            for (i = 0; i < d1[0]; ++i, ++ijk) {
                float  x[3];
                axis64 ax[3];
                affine_x(x, A, i, j, k);
                if (!voxel_valid(x, d0, ext)) { f1[ijk] = NAN; continue; }
                setup3(ax, x, bnd, dp, d0);
                f1[ijk] = patch_sum(ax, f0, d0, 0, 0, 0);
            }
}

void ora_push_affine(double *f0, const float *f1, const pp_usize *d0, pp_usize n1,
                     const pp_usize *d1, const float *A, const int *bnd,
                     const pp_usize *dp, int ext)
{
    pp_usize i, j, k, ijk = 0;
    (void)n1;
    for (k = 0; k < d1[2]; ++k)
        for (j = 0; j < d1[1]; ++j)
            for (i = 0; i < d1[0]; ++i, ++ijk) {
                float  x[3];
                axis64 ax[3];
                double g[3];
                if (!isfinite(f1[ijk])) continue;
                affine_x(x, A, i, j, k);
                if (!voxel_valid(x, d0, ext)) continue;
                setup3(ax, x, bnd, dp, d0);
                g[0] = (double)f1[ijk];
                g[1] = g[2] = 0.0;
                patch_scatter(ax, f0, d0, g, 0);
            }
}

/* ------------------------------------------------------------------------- */
/* FP32 port (CPU baseline)                                                   */
/* ------------------------------------------------------------------------- */

/* B-spline weights of degree dp-1 at the taps o..o+dp-1 for s = x - centre tap;
 * piecewise polynomials written out per tap, value (w) and derivative (dw). */
static pp_ssize port_weights(int dp, float x, float w[MAXDP], float dw[MAXDP])
{
    pp_ssize o = first_tap((pp_usize)dp, x);
    float    t = x - (float)o, s, a, b, p, q;
    switch (dp) {
    case 1:
        w[0] = 1.0f; dw[0] = 0.0f;
        break;
    case 2:
        w[0] = 1.0f - t; w[1] = t;
        dw[0] = -1.0f;   dw[1] = 1.0f;
        break;
    case 3:                      /* t in (1/2, 3/2] */
        s = t - 1.0f;
        a = 0.5f - s; b = 0.5f + s;
        w[0] = 0.5f * a * a; w[1] = 0.75f - s * s; w[2] = 0.5f * b * b;
        dw[0] = -a; dw[1] = -2.0f * s; dw[2] = b;
        break;
    case 4:                      /* t in (1, 2] */
        s = t - 1.0f; a = 1.0f - s;
        w[0] = a * a * a * (1.0f / 6.0f);
        w[1] = (2.0f / 3.0f) - s * s * (1.0f - 0.5f * s);
        w[2] = (2.0f / 3.0f) - a * a * (1.0f - 0.5f * a);
        w[3] = s * s * s * (1.0f / 6.0f);
        dw[0] = -0.5f * a * a;
        dw[1] = s * (1.5f * s - 2.0f);
        dw[2] = -a * (1.5f * a - 2.0f);
        dw[3] = 0.5f * s * s;
        break;
    default:                     /* dp == 5, t in (3/2, 5/2] */
        s = t - 2.0f;
        a = 0.5f - s; b = 0.5f + s;
        w[0] = a * a * a * a * (1.0f / 24.0f);
        w[4] = b * b * b * b * (1.0f / 24.0f);
        w[2] = (115.0f / 192.0f) + s * s * (s * s * 0.25f - 0.625f);
        p = 1.0f + s; q = 1.0f - s;
        w[1] = (55.0f / 96.0f) + p * ((5.0f / 24.0f) + p * (-1.25f + p * ((5.0f / 6.0f) - p * (1.0f / 6.0f))));
        w[3] = (55.0f / 96.0f) + q * ((5.0f / 24.0f) + q * (-1.25f + q * ((5.0f / 6.0f) - q * (1.0f / 6.0f))));
        dw[0] = -a * a * a * (1.0f / 6.0f);
        dw[4] = b * b * b * (1.0f / 6.0f);
        dw[2] = s * (s * s - 1.25f);
        dw[1] =  ((5.0f / 24.0f) + p * (-2.5f + p * (2.5f - p * (2.0f / 3.0f))));
        dw[3] = -((5.0f / 24.0f) + q * (-2.5f + q * (2.5f - q * (2.0f / 3.0f))));
        break;
    }
    return o;
}

static void port_fold(int bnd, pp_ssize o, int dp, pp_usize d, pp_usize idx[MAXDP], int sg[MAXDP])
{
    int k;
    for (k = 0; k < dp; ++k) idx[k] = fold_index(bnd, o + k, d, &sg[k]);
}

typedef struct {
    int      dp[3];
    float    w[3][MAXDP], dw[3][MAXDP];
    pp_usize idx[3][MAXDP];
    int      sg[3][MAXDP];
} port_patch;

static void port_setup(port_patch *p, const float x[3], const int *bnd,
                       const pp_usize *dp, const pp_usize *d0)
{
    int k;
    for (k = 0; k < 3; ++k) {
        pp_ssize o;
        p->dp[k] = (int)dp[k];
        o = port_weights(p->dp[k], x[k], p->w[k], p->dw[k]);
        port_fold(bnd[k], o, p->dp[k], d0[k], p->idx[k], p->sg[k]);
    }
}

/* gathers the patch into a local array first, like get_patch (patch.cu:62-83) */
static int port_gather(const port_patch *p, const float *f0, const pp_usize *d0,
                       float fp[MAXDP * MAXDP * MAXDP])
{
    int i, j, k, n = 0;
    for (k = 0; k < p->dp[2]; ++k)
        for (j = 0; j < p->dp[1]; ++j) {
            pp_usize row = d0[0] * (p->idx[1][j] + d0[1] * p->idx[2][k]);
            int      s   = p->sg[1][j] * p->sg[2][k];
            for (i = 0; i < p->dp[0]; ++i)
                fp[n++] = f0[row + p->idx[0][i]] * (float)(s * p->sg[0][i]);
        }
    return n;
}

void port_pull(float *f1, const float *phi, const float *f0, const pp_usize *d0,
               pp_usize n1, const int *bnd, const pp_usize *dp, int ext)
{
    pp_usize v;
    for (v = 0; v < n1; ++v) {
        float      x[3], fp[MAXDP * MAXDP * MAXDP], acc = 0.0f;
        port_patch p;
        int        i, j, k, n = 0;
        load_x(x, phi, v, n1);
        if (!voxel_valid(x, d0, ext)) { f1[v] = NAN; continue; }
        port_setup(&p, x, bnd, dp, d0);
        port_gather(&p, f0, d0, fp);
        for (k = 0; k < p.dp[2]; ++k)
            for (j = 0; j < p.dp[1]; ++j) {
                float wjk = p.w[2][k] * p.w[1][j];
                for (i = 0; i < p.dp[0]; ++i) acc += p.w[0][i] * wjk * fp[n++];
            }
        f1[v] = acc;
    }
}

void port_pullg(float *g1, const float *phi, const float *f0, const pp_usize *d0,
                pp_usize n1, const int *bnd, const pp_usize *dp, int ext)
{
    pp_usize v;
    for (v = 0; v < n1; ++v) {
        float      x[3], fp[MAXDP * MAXDP * MAXDP], gx = 0.0f, gy = 0.0f, gz = 0.0f;
        port_patch p;
        int        i, j, k, n = 0;
        load_x(x, phi, v, n1);
        if (!voxel_valid(x, d0, ext)) {
            g1[v] = g1[v + n1] = g1[v + 2 * n1] = NAN;
            continue;
        }
        port_setup(&p, x, bnd, dp, d0);
        port_gather(&p, f0, d0, fp);
        for (k = 0; k < p.dp[2]; ++k)
            for (j = 0; j < p.dp[1]; ++j) {
                float ax = p.w[2][k] * p.w[1][j], ay = p.w[2][k] * p.dw[1][j],
                      az = p.dw[2][k] * p.w[1][j];
                for (i = 0; i < p.dp[0]; ++i) {
                    float f = fp[n++];
                    gx += p.dw[0][i] * ax * f;
                    f *= p.w[0][i];
                    gy += ay * f;
                    gz += az * f;
                }
            }
        g1[v] = gx;
        g1[v + n1] = gy;
        g1[v + 2 * n1] = gz;
    }
}

static void port_scatter(const port_patch *p, float *f0, const pp_usize *d0,
                         const float g[3], int gradient)
{
    int i, j, k;
    for (k = 0; k < p->dp[2]; ++k)
        for (j = 0; j < p->dp[1]; ++j) {
            pp_usize row = d0[0] * (p->idx[1][j] + d0[1] * p->idx[2][k]);
            int      s   = p->sg[1][j] * p->sg[2][k];
            float    a, b;
            if (gradient) {
                a = g[0] * p->w[1][j] * p->w[2][k];
                b = g[1] * p->dw[1][j] * p->w[2][k] + g[2] * p->w[1][j] * p->dw[2][k];
            } else {
                a = 0.0f;
                b = g[0] * p->w[1][j] * p->w[2][k];
            }
            for (i = 0; i < p->dp[0]; ++i) {
                float v = a * p->dw[0][i] + b * p->w[0][i];
                f0[row + p->idx[0][i]] += v * (float)(s * p->sg[0][i]);
            }
        }
}

void port_push(float *f0, const float *phi, const float *f1, const pp_usize *d0,
               pp_usize n1, const int *bnd, const pp_usize *dp, int ext)
{
    pp_usize v;
    for (v = 0; v < n1; ++v) {
        float      x[3], g[3];
        port_patch p;
        if (!isfinite(f1[v])) continue;
        load_x(x, phi, v, n1);
        if (!voxel_valid(x, d0, ext)) continue;
        port_setup(&p, x, bnd, dp, d0);
        g[0] = f1[v];
        g[1] = g[2] = 0.0f;
        port_scatter(&p, f0, d0, g, 0);
    }
}

void port_pushg(float *g0, const float *phi, const float *g1, const pp_usize *d0,
                pp_usize n1, const int *bnd, const pp_usize *dp, int ext)
{
    pp_usize v;
    for (v = 0; v < n1; ++v) {
        float      x[3], g[3];
        port_patch p;
        load_x(x, phi, v, n1);
        if (!voxel_valid(x, d0, ext)) continue;
        g[0] = g1[v];
        g[1] = g1[v + n1];
        g[2] = g1[v + 2 * n1];
        if (!isfinite(g[0]) || !isfinite(g[1]) || !isfinite(g[2])) continue;
        port_setup(&p, x, bnd, dp, d0);
        port_scatter(&p, g0, d0, g, 1);
    }
}
