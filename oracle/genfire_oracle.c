/*
 * genfire_oracle.c -- CPU restatement of the GENFIRE v2 reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the genfire_gb300 package,
 * libgenfire.so) links, loads or calls this file.  It is the checker that the
 * tests, the smoke check and the CPU-baseline leg of bench.py compare against.
 *
 * PARITY UNPINNED: the reference (MATLAB, 19 .m files) ships no golden outputs
 * and cannot run here (no MATLAB/Octave, and its CPU gridding calls the
 * un-vendored CMCL nufft2d2).  This file restates the reference's algorithm
 * and is pinned instead by known-answer tests derived from the mathematics
 * (Dirichlet-kernel DFTs, on-axis planes, FFT identities, analytic line
 * integrals) and by an independent numpy restatement; see tests/.
 *
 * Precision model (restating what the reference does, file:line cited at each
 * function):
 *   - geometry (rotation matrices) in FP64, stored FP32 as the reference does;
 *   - K-point selection, closest point, 3x3 solve and the in-plane box filter in
 *     FP32 with a fixed operation order and no FMA contraction (build with
 *     -ffp-contract=off) so index sets are reproducible bit for bit;
 *   - the DFT as the exact direct sum in FP64 (the quantity nufft2d2
 *     approximates at eps 1e-6 and the reference GPU path evaluates in FP32);
 *   - weighted averaging, the Fourier-constraint loop, FFTs, projector and
 *     R-factors in FP64.
 *
 * Array layout: MATLAB column-major (dimension 1 fastest), complex values
 * interleaved (re, im) as doubles.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct { double re, im; } zc;

static inline zc zmul(zc a, zc b) { zc r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline zc zadd(zc a, zc b) { zc r = {a.re + b.re, a.im + b.im}; return r; }

/* Parameters mirroring the GENFIRE_Reconstructor properties used on the path
 * (GENFIRE_Reconstructor.m:30-70). */
typedef struct {
    int    Dim1, Dim2, NumProjs;
    double oversamplingRatio;
    double interpolationCutoffDistance;
    int    DFT_CentroSymmetricity;
    double vector1[3], vector2[3], vector3[3];
    int    numIterations;
    int    constraintEnforcementMode;
    int    constraintPositivity;
    int    constraintSupport;
    int    monitor_R;
    int    monitorR_loopLength;
} orc_params;

/* ------------------------------------------------------------------------ */
/* integer helpers                                                            */
/* ------------------------------------------------------------------------ */

/* MATLAB round(): half away from zero. */
static double mround(double x) { return x < 0 ? -floor(-x + 0.5) : floor(x + 0.5); }

static int imod(int64_t a, int64_t n) { int64_t r = a % n; return (int)(r < 0 ? r + n : r); }

/* n1_oversampled = round(Dim1 * oversamplingRatio)  (GENFIRE_Reconstructor.m:168-169) */
int orc_oversampled_size(int dim, double ratio) { return (int)mround((double)dim * ratio); }

/* Start offset (0-based) of a centred crop of length ori inside length big.
 * My_volumn_index.m:11-28 / My_stripzero.m:29-46 / My_paddzero.m:32-49 all use
 * the same four parity cases; they reduce to floor(big/2) - floor(ori/2). */
static int crop_start(int big, int ori)
{
    if (big % 2 == 0) {
        if (ori % 2 == 0) return (big - ori) / 2;
        return (big - ori + 1) / 2;
    } else {
        if (ori % 2 == 0) return (big - ori - 1) / 2;
        return (big - ori) / 2;
    }
}

/* My_volumn_index.m:3-34.  out is 3x2 column-major, 1-based [start end]. */
void orc_volumn_index(const int big[3], const int ori[3], int out[6])
{
    for (int i = 0; i < 3; ++i) {
        int s = crop_start(big[i], ori[i]);
        out[i] = s + 1;
        out[i + 3] = s + ori[i];
    }
}

/* My_iffshift3_ind.m:1-7: centred 1-based linear index -> ifftshifted one. */
void orc_iffshift3_ind(const int sz[3], int64_t count, const int64_t *ind, int64_t *out)
{
    for (int64_t t = 0; t < count; ++t) {
        int64_t i = ind[t] - 1;
        int64_t i1 = i % sz[0], i2 = (i / sz[0]) % sz[1], i3 = i / ((int64_t)sz[0] * sz[1]);
        i1 = (i1 + (sz[0] + 1) / 2) % sz[0];
        i2 = (i2 + (sz[1] + 1) / 2) % sz[1];
        i3 = (i3 + (sz[2] + 1) / 2) % sz[2];
        out[t] = i1 + (int64_t)sz[0] * (i2 + (int64_t)sz[1] * i3) + 1;
    }
}

/* My_paddzero.m:24-59 (real data). */
void orc_paddzero(const double *vol, const int vs[3], const int ps[3], double *out)
{
    int s0 = crop_start(ps[0], vs[0]), s1 = crop_start(ps[1], vs[1]), s2 = crop_start(ps[2], vs[2]);
    memset(out, 0, sizeof(double) * (size_t)ps[0] * ps[1] * ps[2]);
    for (int k = 0; k < vs[2]; ++k)
        for (int j = 0; j < vs[1]; ++j)
            for (int i = 0; i < vs[0]; ++i)
                out[(size_t)(i + s0) + (size_t)ps[0] * ((j + s1) + (size_t)ps[1] * (k + s2))] =
                    vol[(size_t)i + (size_t)vs[0] * (j + (size_t)vs[1] * k)];
}

/* My_stripzero.m:22-55 (real data). */
void orc_stripzero(const double *pad, const int ps[3], const int os[3], double *out)
{
    int s0 = crop_start(ps[0], os[0]), s1 = crop_start(ps[1], os[1]), s2 = crop_start(ps[2], os[2]);
    for (int k = 0; k < os[2]; ++k)
        for (int j = 0; j < os[1]; ++j)
            for (int i = 0; i < os[0]; ++i)
                out[(size_t)i + (size_t)os[0] * (j + (size_t)os[1] * k)] =
                    pad[(size_t)(i + s0) + (size_t)ps[0] * ((j + s1) + (size_t)ps[1] * (k + s2))];
}

/* make_Kspace_indices.m:16-62: Q = |k|/(n/2) on a centred grid, Q = sqrt(Kx^2+Ky^2+Kz^2)
 * with Kx along dim 2, Ky along dim 1 (meshgrid(vec2,vec1,vec3)). */
static double kvec(int n, int i)
{
    if (n == 1) return 0.0;
    int r = (n % 2 == 0) ? n / 2 : (n - 1) / 2;      /* n2K */
    return (double)(i - r) / (double)r;
}
void orc_make_kspace_indices(const int sz[3], double *Q)
{
    for (int k = 0; k < sz[2]; ++k)
        for (int j = 0; j < sz[1]; ++j)
            for (int i = 0; i < sz[0]; ++i) {
                double kx = kvec(sz[1], j), ky = kvec(sz[0], i), kz = kvec(sz[2], k);
                Q[(size_t)i + (size_t)sz[0] * (j + (size_t)sz[1] * k)] = sqrt(kx * kx + ky * ky + kz * kz);
            }
}

/* ------------------------------------------------------------------------ */
/* geometry                                                                   */
/* ------------------------------------------------------------------------ */

/* MatrixQuaternionRot: fillInFourierGrid_DFT.m:353-363 and src/MatrixQuaternionRot.m:1-12.
 * R is column-major. */
void orc_quat_rot(const double v[3], double theta_deg, double R[9])
{
    double th = theta_deg * M_PI / 180.0;
    double nv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double a = v[0] / nv, b = v[1] / nv, c = v[2] / nv;
    double w = cos(th / 2), s = -sin(th / 2);
    double x = s * a, y = s * b, z = s * c;
    /* rows as written in the reference; R[i + 3*j] */
    R[0] = 1 - 2 * y * y - 2 * z * z; R[3] = 2 * x * y + 2 * w * z;     R[6] = 2 * x * z - 2 * w * y;
    R[1] = 2 * x * y - 2 * w * z;     R[4] = 1 - 2 * x * x - 2 * z * z; R[7] = 2 * y * z + 2 * w * x;
    R[2] = 2 * x * z + 2 * w * y;     R[5] = 2 * y * z - 2 * w * x;     R[8] = 1 - 2 * x * x - 2 * y * y;
}

static void matmul3(const double A[9], const double B[9], double C[9])
{
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i)
            C[i + 3 * j] = A[i] * B[3 * j] + A[i + 3] * B[3 * j + 1] + A[i + 6] * B[3 * j + 2];
}

/* R = Q(v1,phi) Q(v2,theta) Q(v3,psi): fillInFourierGrid_DFT.m:110-114,
 * calculate3Dprojection_RealSpaceinterp_general.m:3-7. */
void orc_euler_rot(const double v1[3], const double v2[3], const double v3[3],
                   double phi, double theta, double psi, double R[9])
{
    double A[9], B[9], C[9], T[9];
    orc_quat_rot(v1, phi, A);
    orc_quat_rot(v2, theta, B);
    orc_quat_rot(v3, psi, C);
    matmul3(A, B, T);
    matmul3(T, C, R);
}

/* sind/cosd with exact reduction in degrees (MATLAB's sind/cosd are exact at
 * multiples of 90). */
static void sincosd(double x, double *s, double *c)
{
    double r = remainder(x, 360.0);
    double q = nearbyint(r / 90.0);
    double t = (r - 90.0 * q) * (M_PI / 180.0);
    double st = sin(t), ct = cos(t);
    int qi = ((int)q % 4 + 4) % 4;
    switch (qi) {
    case 0: *s = st; *c = ct; break;
    case 1: *s = ct; *c = -st; break;
    case 2: *s = -st; *c = -ct; break;
    default: *s = -ct; *c = st; break;
    }
}

/* Closed-form ZYZ matrix of calculate3Dprojection_RealSpaceinterp.m:13-15. */
void orc_rot_zyz(double phi, double theta, double psi, double R[9])
{
    double sf, cf, st, ct, sp, cp;
    sincosd(phi, &sf, &cf); sincosd(theta, &st, &ct); sincosd(psi, &sp, &cp);
    R[0] = cp * ct * cf - sp * sf;  R[3] = -sp * ct * cf - cp * sf; R[6] = st * cf;
    R[1] = cp * ct * sf + sp * cf;  R[4] = -sp * ct * sf + cp * cf; R[7] = st * sf;
    R[2] = -cp * st;                R[5] = sp * st;                 R[8] = ct;
}

/* Per-projection FP32 geometry (fillInFourierGrid_DFT.m:100-118): rotMATs(:,:,p) as
 * single, normVECs(p,:) = rotMATs(:,:,p) * [0 0 1]' = third column. */
void orc_proj_geometry(const orc_params *prm, double phi, double theta, double psi,
                       float Rf[9], float nrm[3])
{
    double R[9];
    orc_euler_rot(prm->vector1, prm->vector2, prm->vector3, phi, theta, psi, R);
    for (int i = 0; i < 9; ++i) Rf[i] = (float)R[i];
    nrm[0] = Rf[6]; nrm[1] = Rf[7]; nrm[2] = Rf[8];
}

/* ------------------------------------------------------------------------ */
/* FP32 3x3 LU solve (mldivide for a full 3x3 matrix: LU, partial pivoting)   */
/* ------------------------------------------------------------------------ */

typedef struct { float a[9]; int piv[3]; } lu3f;

/* Row-pivoted LU in LAPACK getf2 order: pick the first largest |a(i,k)|,
 * scale the column by the reciprocal pivot, rank-1 update. */
static void lu3f_factor(const float R[9], lu3f *f)
{
    memcpy(f->a, R, sizeof(float) * 9);
    float *A = f->a;
    for (int k = 0; k < 3; ++k) {
        int p = k;
        float best = fabsf(A[k + 3 * k]);
        for (int i = k + 1; i < 3; ++i)
            if (fabsf(A[i + 3 * k]) > best) { best = fabsf(A[i + 3 * k]); p = i; }
        f->piv[k] = p;
        if (p != k)
            for (int j = 0; j < 3; ++j) { float t = A[k + 3 * j]; A[k + 3 * j] = A[p + 3 * j]; A[p + 3 * j] = t; }
        if (A[k + 3 * k] != 0.0f && k < 2) {
            float r = 1.0f / A[k + 3 * k];
            for (int i = k + 1; i < 3; ++i) A[i + 3 * k] = A[i + 3 * k] * r;
        }
        for (int j = k + 1; j < 3; ++j)
            for (int i = k + 1; i < 3; ++i)
                A[i + 3 * j] = A[i + 3 * j] - A[i + 3 * k] * A[k + 3 * j];
    }
}

/* getrs: apply row swaps, unit-lower forward, upper back substitution
 * (trsm column order). */
static void lu3f_solve(const lu3f *f, float b[3])
{
    const float *A = f->a;
    for (int k = 0; k < 3; ++k)
        if (f->piv[k] != k) { float t = b[k]; b[k] = b[f->piv[k]]; b[f->piv[k]] = t; }
    for (int k = 0; k < 3; ++k)
        for (int i = k + 1; i < 3; ++i) b[i] = b[i] - b[k] * A[i + 3 * k];
    for (int k = 2; k >= 0; --k) {
        b[k] = b[k] / A[k + 3 * k];
        for (int i = 0; i < k; ++i) b[i] = b[i] - b[k] * A[i + 3 * k];
    }
}

/* ------------------------------------------------------------------------ */
/* half-grid index space (fillInFourierGrid_DFT.m:122-144)                   */
/* ------------------------------------------------------------------------ */

typedef struct { int lo1, lo2, lo3, l1, l2, l3; } gridspec;

static gridspec make_grid(int n1, int n2, int centro)
{
    gridspec g;
    if (centro) {
        g.lo1 = -(n1 / 2); g.l1 = n1 / 2 + 1;
        g.lo2 = -(n2 / 2); g.l2 = 2 * (n2 / 2) + 1;
        g.lo3 = -(n1 / 2); g.l3 = 2 * (n1 / 2) + 1;
    } else {
        g.lo1 = -((n1) / 2); g.l1 = n1;       /* -ceil((n-1)/2) == -(n/2) for integers */
        g.lo2 = -((n2) / 2); g.l2 = n2;
        g.lo3 = g.lo1;       g.l3 = n1;
    }
    return g;
}

void orc_grid_extent(int n1, int n2, int centro, int out[6])
{
    gridspec g = make_grid(n1, n2, centro);
    out[0] = g.lo1; out[1] = g.lo2; out[2] = g.lo3; out[3] = g.l1; out[4] = g.l2; out[5] = g.l3;
}

/* ------------------------------------------------------------------------ */
/* K-point selection, one projection (fillInFourierGrid_DFT.m:175-192)       */
/* ------------------------------------------------------------------------ */

/* Returns the number of selected points written (ascending linear index, the
 * order of MATLAB's find), or -1 when cap is too small.  ind is the 0-based
 * linear index into the l1 x l2 x l3 grid; dist is D (FP32); u, v are
 * CP_plane(1,:), CP_plane(2,:).  *offplane counts |CP_plane(3,:)| > 1e-4
 * (the reference prints "something wrong!" when it is non-zero). */
/* one point of the selection; returns 1 when selected */
static int select_point(const gridspec *g, int64_t li, float h0, float h1, float h2, const float nrm[3], float nsq,
                        const lu3f *lu, double cutoff, double half1, double half2,
                        float *D_, float *u_, float *v_, int *off_)
{
    int i1 = (int)(li % g->l1), i2 = (int)((li / g->l1) % g->l2), i3 = (int)(li / ((int64_t)g->l1 * g->l2));
    float K1 = (float)(g->lo1 + i1), K2 = (float)(g->lo2 + i2), K3 = (float)(g->lo3 + i3);
    float D = fabsf(K1 * h0 + K2 * h1 + K3 * h2);
    *off_ = 0;
    if (!((double)D < cutoff)) return 0;
    float s = K1 * nrm[0] + K2 * nrm[1] + K3 * nrm[2];
    float t = (0.0f - s) / nsq;
    float b[3] = {K1 + t * nrm[0], K2 + t * nrm[1], K3 + t * nrm[2]};
    lu3f_solve(lu, b);
    if (fabsf(b[2]) > 0.0001f) *off_ = 1;
    if (!(fabs((double)b[0]) <= half1 && fabs((double)b[1]) <= half2)) return 0;
    *D_ = D; *u_ = b[0]; *v_ = b[1];
    return 1;
}

/* Returns the number of selected points written (ascending linear index, the
 * order of MATLAB's find), or -1 when cap is too small.  ind is the 0-based
 * linear index into the l1 x l2 x l3 grid; dist is D (FP32); u, v are
 * CP_plane(1,:), CP_plane(2,:).  *offplane counts |CP_plane(3,:)| > 1e-4
 * (the reference prints "something wrong!" when it is non-zero).  The grid is
 * scanned in chunks in parallel; the chunk counts are prefix-summed so the
 * output order is the serial order. */
int64_t orc_select(int n1, int n2, int centro, double cutoff, const float Rf[9], const float nrm[3],
                   int64_t cap, int64_t *ind, float *dist, float *u, float *v, int64_t *offplane)
{
    gridspec g = make_grid(n1, n2, centro);
    /* distancePointsPlane_YY (:331-333): normvec / norm(normvec) in single */
    float nn = sqrtf(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    float h0 = nrm[0] / nn, h1 = nrm[1] / nn, h2 = nrm[2] / nn;
    /* closestpoint (:338-350) uses the un-normalised normal */
    float nsq = nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2];
    lu3f lu;
    lu3f_factor(Rf, &lu);
    double half1 = n1 / 2.0, half2 = n2 / 2.0;
    int64_t total = (int64_t)g.l1 * g.l2 * g.l3;
    const int64_t CH = 1 << 16;
    int64_t nch = (total + CH - 1) / CH;
    int64_t *cnt = (int64_t *)calloc((size_t)nch + 1, sizeof(int64_t));
    int64_t off = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : off)
    for (int64_t c = 0; c < nch; ++c) {
        int64_t e = (c + 1) * CH < total ? (c + 1) * CH : total, k = 0;
        for (int64_t li = c * CH; li < e; ++li) {
            float D, uu, vv;
            int o;
            k += select_point(&g, li, h0, h1, h2, nrm, nsq, &lu, cutoff, half1, half2, &D, &uu, &vv, &o);
            off += o;
        }
        cnt[c + 1] = k;
    }
    for (int64_t c = 0; c < nch; ++c) cnt[c + 1] += cnt[c];
    if (cnt[nch] > cap) { free(cnt); return -1; }
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t c = 0; c < nch; ++c) {
        int64_t e = (c + 1) * CH < total ? (c + 1) * CH : total, k = cnt[c];
        for (int64_t li = c * CH; li < e; ++li) {
            float D, uu, vv;
            int o;
            if (select_point(&g, li, h0, h1, h2, nrm, nsq, &lu, cutoff, half1, half2, &D, &uu, &vv, &o)) {
                ind[k] = li; dist[k] = D; u[k] = uu; v[k] = vv;
                ++k;
            }
        }
    }
    int64_t n = cnt[nch];
    free(cnt);
    if (offplane) *offplane = off;
    return n;
}

/* ------------------------------------------------------------------------ */
/* the DFT at off-grid points, exact direct sum in FP64                       */
/* (fillInFourierGrid_DFT.m:243; nufft2d2 at :253 approximates the same sum)  */
/* ------------------------------------------------------------------------ */

/* exp(-2 pi i * a * w / n) with the phase reduced exactly: a*w is exact in
 * FP64 (w is an FP32 value, |a| < 2^20), remainder() is exact. */
static inline zc phase(double a, double w, double n)
{
    double t = remainder(a * w, n) / n;
    double ang = -2.0 * M_PI * t;
    zc r = {cos(ang), sin(ang)};
    return r;
}

/* F[j] = sum_{a,b} P(a,b) exp(-2 pi i (K10(a) u_j / n1 + K20(b) v_j / n2)),
 * K10 = -ceil((D1-1)/2) .. floor((D1-1)/2) along dim 1 (:147-150). */
void orc_dft(const double *proj, int D1, int D2, int n1, int n2, int64_t nk,
             const float *u, const float *v, double *F)
{
    int a0 = -(D1 / 2), b0 = -(D2 / 2);
#pragma omp parallel
    {
        zc *eu = (zc *)malloc(sizeof(zc) * D1);
#pragma omp for schedule(dynamic, 16)
        for (int64_t j = 0; j < nk; ++j) {
            for (int a = 0; a < D1; ++a) eu[a] = phase((double)(a0 + a), (double)u[j], (double)n1);
            zc acc = {0, 0};
            for (int b = 0; b < D2; ++b) {
                zc q = {0, 0};
                const double *col = proj + (size_t)D1 * b;
                for (int a = 0; a < D1; ++a) { q.re += eu[a].re * col[a]; q.im += eu[a].im * col[a]; }
                acc = zadd(acc, zmul(q, phase((double)(b0 + b), (double)v[j], (double)n2)));
            }
            F[2 * j] = acc.re; F[2 * j + 1] = acc.im;
        }
        free(eu);
    }
}

/* ------------------------------------------------------------------------ */
/* CentroSymmetricity.m:2-72 and hermitianSymmetrize.m:22-65                  */
/* ------------------------------------------------------------------------ */

/* FS: (n_k1+1) x L2 x L3 half grid with k1 <= 0 (L2 = 2*floor(n2/2)+1,
 * L3 = 2*floor(n1/2)+1).  M: n1 x n2 x n1 centred full grid.  All four parity
 * branches of the reference reduce to M(k) = FS(k) for k1 <= 0 and
 * M(k) = conj(FS(-k)) for k1 > 0. */
void orc_centro(const double *FS, int n1, int n_k1, int n2, double *M)
{
    int L1 = n_k1 + 1, L2 = 2 * (n2 / 2) + 1, L3 = 2 * (n1 / 2) + 1;
    int c1 = n1 / 2, c2 = n2 / 2, c3 = n1 / 2;
    for (int i3 = 0; i3 < n1; ++i3)
        for (int i2 = 0; i2 < n2; ++i2)
            for (int i1 = 0; i1 < n1; ++i1) {
                int k1 = i1 - c1, k2 = i2 - c2, k3 = i3 - c3;
                size_t o = (size_t)i1 + (size_t)n1 * (i2 + (size_t)n2 * i3);
                int s = 1;
                if (k1 > 0) { k1 = -k1; k2 = -k2; k3 = -k3; s = -1; }
                size_t src = (size_t)(k1 + n_k1) + (size_t)L1 * ((k2 + n2 / 2) + (size_t)L2 * (k3 + n1 / 2));
                (void)L3;
                M[2 * o] = FS[2 * src];
                M[2 * o + 1] = s * FS[2 * src + 1];
            }
}

void orc_hermitian_symmetrize(const double *in, int d1, int d2, int d3, double *out)
{
    int e1 = d1 + (d1 % 2 == 0), e2 = d2 + (d2 % 2 == 0), e3 = d3 + (d3 % 2 == 0);
#define IN(i, j, k) (((i) < d1 && (j) < d2 && (k) < d3) ? (size_t)(i) + (size_t)d1 * ((j) + (size_t)d2 * (k)) : (size_t)-1)
    for (int k = 0; k < d3; ++k)
        for (int j = 0; j < d2; ++j)
            for (int i = 0; i < d1; ++i) {
                size_t a = IN(i, j, k), b = IN(e1 - 1 - i, e2 - 1 - j, e3 - 1 - k);
                double ar = in[2 * a], ai = in[2 * a + 1];
                double br = 0, bi = 0;
                if (b != (size_t)-1) { br = in[2 * b]; bi = in[2 * b + 1]; }
                double re = ar + br, im = ai - bi;
                int cnt = (ar != 0 || ai != 0) + (br != 0 || bi != 0);
                if (cnt) { re /= cnt; im /= cnt; }
                out[2 * a] = re; out[2 * a + 1] = im;
            }
#undef IN
}

/* ------------------------------------------------------------------------ */
/* FFT (mixed radix, FP64).  fftn: unnormalised forward, 1/N inverse.        */
/* ------------------------------------------------------------------------ */

typedef struct { int n; int nf; int f[64]; zc *w; } fftplan;

static void plan_init(fftplan *p, int n)
{
    p->n = n; p->nf = 0;
    int m = n;
    while (m % 4 == 0) { p->f[p->nf++] = 4; m /= 4; }
    while (m % 2 == 0) { p->f[p->nf++] = 2; m /= 2; }
    for (int q = 3; m > 1; q += 2)
        while (m % q == 0) { p->f[p->nf++] = q; m /= q; }
    p->w = (zc *)malloc(sizeof(zc) * (n > 0 ? n : 1));
    for (int t = 0; t < n; ++t) {
        double ang = -2.0 * M_PI * (double)t / (double)n;
        p->w[t].re = cos(ang); p->w[t].im = sin(ang);
    }
}
static void plan_free(fftplan *p) { free(p->w); }

/* Out-of-place Stockham passes; returns the buffer holding the result. */
static zc *fft1(const fftplan *p, zc *x, zc *y, int sign)
{
    int n = p->n, Ns = 1;
    zc v[64], o[64];
    for (int s = 0; s < p->nf; ++s) {
        int R = p->f[s], m = n / R;
        for (int j = 0; j < m; ++j) {
            int k = j % Ns;
            for (int r = 0; r < R; ++r) {
                zc a = x[j + r * m];
                int t = (int)(((int64_t)k * r * (n / (Ns * R))) % n);
                zc w = p->w[t];
                if (sign > 0) w.im = -w.im;
                v[r] = zmul(a, w);
            }
            for (int q = 0; q < R; ++q) {
                zc acc = {0, 0};
                for (int r = 0; r < R; ++r) {
                    zc w = p->w[(int)(((int64_t)q * r % R) * (n / R))];
                    if (sign > 0) w.im = -w.im;
                    acc = zadd(acc, zmul(v[r], w));
                }
                o[q] = acc;
            }
            int base = (j / Ns) * Ns * R + k;
            for (int q = 0; q < R; ++q) y[base + q * Ns] = o[q];
        }
        Ns *= R;
        zc *t = x; x = y; y = t;
    }
    return x;
}

/* In-place 3-D FFT of an n1 x n2 x n3 complex array (interleaved). */
void orc_fftn(double *data, int n1, int n2, int n3, int inverse)
{
    zc *d = (zc *)data;
    int dims[3] = {n1, n2, n3};
    size_t strides[3] = {1, (size_t)n1, (size_t)n1 * n2};
    size_t N = (size_t)n1 * n2 * n3;
    int sign = inverse ? +1 : -1;
    for (int ax = 0; ax < 3; ++ax) {
        int n = dims[ax];
        if (n == 1) continue;
        fftplan p; plan_init(&p, n);
        size_t nl = N / n, st = strides[ax];
#pragma omp parallel
        {
            zc *a = (zc *)malloc(sizeof(zc) * n), *b = (zc *)malloc(sizeof(zc) * n);
#pragma omp for schedule(static)
            for (int64_t l = 0; l < (int64_t)nl; ++l) {
                size_t base;
                if (ax == 0) base = (size_t)l * n;
                else if (ax == 1) base = (size_t)(l % n1) + (size_t)(l / n1) * n1 * n2;
                else base = (size_t)l;
                for (int i = 0; i < n; ++i) a[i] = d[base + i * st];
                zc *r = fft1(&p, a, b, sign);
                for (int i = 0; i < n; ++i) d[base + i * st] = r[i];
            }
            free(a); free(b);
        }
        plan_free(&p);
    }
    if (inverse) {
        double s = 1.0 / (double)N;
#pragma omp parallel for
        for (int64_t i = 0; i < (int64_t)N; ++i) { d[i].re *= s; d[i].im *= s; }
    }
}

/* ------------------------------------------------------------------------ */
/* fillInFourierGrid_DFT.m:85-304 end to end                                 */
/* ------------------------------------------------------------------------ */

/* Fourier-grid average for one grid: fills FS (2*l1*l2*l3) from the
 * per-projection selections in projection order, with the exact-hit
 * override (:268-291; last occurrence wins). */
static int64_t grid_fill(const orc_params *prm, const double *projs, const double *angles,
                         double *FS, int64_t *stats_nk)
{
    int D1 = prm->Dim1, D2 = prm->Dim2, P = prm->NumProjs;
    int n1 = orc_oversampled_size(D1, prm->oversamplingRatio);
    int n2 = orc_oversampled_size(D2, prm->oversamplingRatio);
    gridspec g = make_grid(n1, n2, prm->DFT_CentroSymmetricity);
    size_t total = (size_t)g.l1 * g.l2 * g.l3;
    double *W = (double *)calloc(total, sizeof(double));
    double *EX = (double *)calloc(2 * total, sizeof(double));
    unsigned char *hasx = (unsigned char *)calloc(total, 1);
    memset(FS, 0, sizeof(double) * 2 * total);
    int64_t cap = (int64_t)total;
    int64_t *ind = (int64_t *)malloc(sizeof(int64_t) * cap);
    float *dist = (float *)malloc(sizeof(float) * cap), *u = (float *)malloc(sizeof(float) * cap),
          *v = (float *)malloc(sizeof(float) * cap);
    double *F = (double *)malloc(sizeof(double) * 2 * cap);
    int64_t totsel = 0, offplane_total = 0;
    for (int p = 0; p < P; ++p) {
        float Rf[9], nrm[3];
        orc_proj_geometry(prm, angles[p], angles[p + P], angles[p + 2 * P], Rf, nrm);
        int64_t off = 0;
        int64_t nk = orc_select(n1, n2, prm->DFT_CentroSymmetricity, prm->interpolationCutoffDistance,
                                Rf, nrm, cap, ind, dist, u, v, &off);
        offplane_total += off;
        if (stats_nk) stats_nk[p] = nk;
        orc_dft(projs + (size_t)D1 * D2 * p, D1, D2, n1, n2, nk, u, v, F);
        for (int64_t j = 0; j < nk; ++j) {
            size_t li = (size_t)ind[j];
            if ((double)dist[j] < 1e-7) {
                EX[2 * li] = F[2 * j]; EX[2 * li + 1] = F[2 * j + 1]; hasx[li] = 1;
            } else {
                double w = 1.0 / (double)dist[j];
                FS[2 * li] += F[2 * j] * w; FS[2 * li + 1] += F[2 * j + 1] * w;
                W[li] += w;
            }
        }
        totsel += nk;
    }
    for (size_t li = 0; li < total; ++li) {
        if (W[li] > 0) { FS[2 * li] /= W[li]; FS[2 * li + 1] /= W[li]; }
        if (hasx[li]) { FS[2 * li] = EX[2 * li]; FS[2 * li + 1] = EX[2 * li + 1]; }
    }
    free(W); free(EX); free(hasx); free(ind); free(dist); free(u); free(v); free(F);
    (void)offplane_total;
    return totsel;
}

/* The half/full grid FS before CentroSymmetricity (2*l1*l2*l3 doubles). */
int64_t orc_grid_fs(const orc_params *prm, const double *projs, const double *angles, double *FS, int64_t *nk)
{
    return grid_fill(prm, projs, angles, FS, nk);
}

/* recIFFT = My_stripzero(real(my_ifft(M)), [D1 D2 D1]) (fillInFourierGrid_DFT.m:304). */
void orc_rec_ifft(const double *M, int n1, int n2, int D1, int D2, double *rec)
{
    size_t N = (size_t)n1 * n2 * n1;
    double *k = (double *)malloc(sizeof(double) * 2 * N);
    /* ifftshift (centred -> FFT order) */
    for (int i3 = 0; i3 < n1; ++i3)
        for (int i2 = 0; i2 < n2; ++i2)
            for (int i1 = 0; i1 < n1; ++i1) {
                size_t src = (size_t)((i1 + n1 / 2) % n1) + (size_t)n1 * (((i2 + n2 / 2) % n2) + (size_t)n2 * ((i3 + n1 / 2) % n1));
                size_t dst = (size_t)i1 + (size_t)n1 * (i2 + (size_t)n2 * i3);
                k[2 * dst] = M[2 * src]; k[2 * dst + 1] = M[2 * src + 1];
            }
    orc_fftn(k, n1, n2, n1, 1);
    int s1 = D1 / 2, s2 = D2 / 2;
    for (int i3 = 0; i3 < D1; ++i3)
        for (int i2 = 0; i2 < D2; ++i2)
            for (int i1 = 0; i1 < D1; ++i1) {
                size_t src = (size_t)imod(i1 - s1, n1) + (size_t)n1 * (imod(i2 - s2, n2) + (size_t)n2 * imod(i3 - s1, n1));
                rec[(size_t)i1 + (size_t)D1 * (i2 + (size_t)D2 * i3)] = k[2 * src];
            }
    free(k);
}

/* fillInFourierGrid_DFT end to end: measuredK (2*n1*n2*n1, centred) and,
 * if rec != NULL, recIFFT (D1*D2*D1).  nk (NumProjs entries) receives the
 * per-projection selected counts. Returns the total selected count. */
int64_t orc_grid_dft(const orc_params *prm, const double *projs, const double *angles,
                     double *measuredK, double *rec, int64_t *nk)
{
    int n1 = orc_oversampled_size(prm->Dim1, prm->oversamplingRatio);
    int n2 = orc_oversampled_size(prm->Dim2, prm->oversamplingRatio);
    gridspec g = make_grid(n1, n2, prm->DFT_CentroSymmetricity);
    size_t total = (size_t)g.l1 * g.l2 * g.l3;
    double *FS = (double *)malloc(sizeof(double) * 2 * total);
    int64_t tot = grid_fill(prm, projs, angles, FS, nk);
    if (prm->DFT_CentroSymmetricity) orc_centro(FS, n1, n1 / 2, n2, measuredK);
    else memcpy(measuredK, FS, sizeof(double) * 2 * total);
    free(FS);
    if (rec) orc_rec_ifft(measuredK, n1, n2, prm->Dim1, prm->Dim2, rec);
    return tot;
}

/* ------------------------------------------------------------------------ */
/* FFT gridding: fillInFourierGrid (griddingMethod = 1)                       */
/* ------------------------------------------------------------------------ */

/* Cube size of fillInFourierGrid.m:38-42 (particleWindowSize = Dim2,
 * GENFIRE_Reconstructor.m:121): Dim2*ratio for even Dim2, else
 * 1 + (Dim2-1)*ratio; -1 when that is not an integer (MATLAB's zeros() would
 * reject it). */
int orc_fft_grid_size(int Dim2, double ratio)
{
    double m = (Dim2 % 2 == 0) ? (double)Dim2 * ratio : 1.0 + (double)(Dim2 - 1) * ratio;
    double r = mround(m);
    if (fabs(m - r) > 1e-9 || r < 1) return -1;
    return (int)r;
}

/* fillInFourierGrid.m:27-168 in FP64 (the reference FFTs single-precision
 * padded projections and sums single-precision products; this restatement
 * keeps every value in double except the FP32 geometry and weights):
 *   kMeasured(:,:,p) = my_fft(My_paddzero(proj_p, [m m])) (:59-61), my_fft =
 *     fftshift(fftn(ifftshift(.))) (src/my_fft.m);
 *   slice coordinates kx = i - nc (dim 1), ky = j - nc (dim 2), nc = floor(m/2)+1
 *     (:47-54, meshgrid order);
 *   rotkCoords = R' [kx; ky; 0] (:80-89) in FP32 with R of :80-82 (= the ZYZ
 *     matrix of the projector transposed), products left to right without
 *     FMA, the kz = 0 column dropped;
 *   values exactly -999 are dropped (:97-101);
 *   for Yshift, Xshift, Zshift in [-s, s] (outer to inner; s = round(cutoff)
 *     when allowMultipleGridMatches, else 0, :108-139): voxel round(coords) +
 *     shift (half away from zero), FP32 distance sqrt(dx^2 + dy^2 + dz^2),
 *     kept when inside the m^3 cube and distance <= cutoff (compared in double);
 *   weight 1/(d + 1e-5) in FP32 (:155-157); sums of w*F and w in FP64 in the
 *     list order (shift, projection, pixel), FS = sum(wF)/sum(w) where
 *     sum(w) > 0 (:159-161); measuredK = hermitianSymmetrize(FS) (:163);
 *   recIFFT = My_stripzero(real(my_ifft(measuredK)), [Dim1 Dim2 Dim1]) (:165).
 * measuredK: 2*m^3 doubles (centred, complex interleaved); rec (optional):
 * Dim1*Dim2*Dim1.  Returns the number of (voxel, value) pairs gridded, or -1
 * when m is not an integer or smaller than Dim1/Dim2. */
int64_t orc_grid_fft(const orc_params *prm, int allowMultipleGridMatches, const double *projs,
                     const double *angles, double *measuredK, double *rec)
{
    const int D1 = prm->Dim1, D2 = prm->Dim2, P = prm->NumProjs;
    const int m = orc_fft_grid_size(D2, prm->oversamplingRatio);
    if (m < 0 || m < D1 || m < D2) return -1;
    const size_t mm = (size_t)m * m, N = mm * m;
    const int h = m / 2;
    /* per-projection centred spectra */
    double *K = (double *)calloc(2 * mm * (size_t)P, sizeof(double));
    double *buf = (double *)malloc(sizeof(double) * 2 * mm);
    for (int p = 0; p < P; ++p) {
        memset(buf, 0, sizeof(double) * 2 * mm);
        /* padded position x + (h - D1/2), then ifftshift: index (x - D1/2) mod m */
        for (int y = 0; y < D2; ++y)
            for (int x = 0; x < D1; ++x) {
                size_t d = (size_t)imod(x - D1 / 2, m) + (size_t)m * imod(y - D2 / 2, m);
                buf[2 * d] = projs[(size_t)p * D1 * D2 + x + (size_t)D1 * y];
            }
        orc_fftn(buf, m, m, 1, 0);
        double *kp = K + 2 * mm * (size_t)p;
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) { /* fftshift: centred (i, j) <- FFT index (i - h, j - h) mod m */
                size_t s = (size_t)imod(i - h, m) + (size_t)m * imod(j - h, m);
                size_t d = (size_t)i + (size_t)m * j;
                kp[2 * d] = buf[2 * s];
                kp[2 * d + 1] = buf[2 * s + 1];
            }
    }
    free(buf);
    /* rotated slice coordinates, FP32 */
    float *cx = (float *)malloc(sizeof(float) * mm * (size_t)P);
    float *cy = (float *)malloc(sizeof(float) * mm * (size_t)P);
    float *cz = (float *)malloc(sizeof(float) * mm * (size_t)P);
    for (int p = 0; p < P; ++p) {
        double R[9];
        orc_rot_zyz(angles[p], angles[p + P], angles[p + 2 * P], R);
        /* rotkCoords = R_fft' k = R_zyz k: X = R[0] kx + R[3] ky, Y = R[1] kx + R[4] ky, Z = R[2] kx + R[5] ky */
        const float a0 = (float)R[0], a3 = (float)R[3], a1 = (float)R[1], a4 = (float)R[4];
        const float a2 = (float)R[2], a5 = (float)R[5];
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) {
                const float kx = (float)(i - h), ky = (float)(j - h);
                const size_t o = (size_t)p * mm + i + (size_t)m * j;
                cx[o] = a0 * kx + a3 * ky;
                cy[o] = a1 * kx + a4 * ky;
                cz[o] = a2 * kx + a5 * ky;
            }
    }
    const int s = allowMultipleGridMatches ? (int)mround(prm->interpolationCutoffDistance) : 0;
    const double cut = prm->interpolationCutoffDistance;
    double *num = (double *)calloc(2 * N, sizeof(double));
    double *ws = (double *)calloc(N, sizeof(double));
    int64_t pairs = 0;
    for (int ys = -s; ys <= s; ++ys)
        for (int xs = -s; xs <= s; ++xs)
            for (int zs = -s; zs <= s; ++zs)
                for (size_t o = 0; o < mm * (size_t)P; ++o) {
                    const double vr = K[2 * o], vi = K[2 * o + 1];
                    if (vr == -999.0 && vi == 0.0) continue;
                    const float tx = roundf(cx[o]) + (float)xs, ty = roundf(cy[o]) + (float)ys,
                                tz = roundf(cz[o]) + (float)zs;
                    const float dx = cx[o] - tx, dy = cy[o] - ty, dz = cz[o] - tz;
                    const float d = sqrtf(dx * dx + dy * dy + dz * dz);
                    const int ix = (int)tx + h, iy = (int)ty + h, iz = (int)tz + h;
                    if (ix < 0 || ix >= m || iy < 0 || iy >= m || iz < 0 || iz >= m) continue;
                    if (!((double)d <= cut)) continue;
                    const float w = 1.0f / (d + 1e-5f);
                    const size_t v = (size_t)ix + (size_t)m * (iy + (size_t)m * iz);
                    num[2 * v] += vr * (double)w;
                    num[2 * v + 1] += vi * (double)w;
                    ws[v] += (double)w;
                    ++pairs;
                }
    free(cx); free(cy); free(cz); free(K);
    for (size_t v = 0; v < N; ++v)
        if (ws[v] > 0) { num[2 * v] /= ws[v]; num[2 * v + 1] /= ws[v]; }
    free(ws);
    orc_hermitian_symmetrize(num, m, m, m, measuredK);
    free(num);
    if (rec) orc_rec_ifft(measuredK, m, m, D1, D2, rec);
    return pairs;
}

/* ------------------------------------------------------------------------ */
/* real-space projector (calculate3Dprojection_RealSpaceinterp(_general).m)  */
/* interpolation is trilinear; out-of-volume samples are 0                    */
/* ------------------------------------------------------------------------ */

static inline double tri(const double *V, int n1, int n2, int n3, double x, double y, double z)
{
    if (!(x >= 0 && y >= 0 && z >= 0 && x <= n1 - 1 && y <= n2 - 1 && z <= n3 - 1)) return 0.0;
    int i = (int)floor(x), j = (int)floor(y), k = (int)floor(z);
    if (i > n1 - 2) i = n1 - 2;
    if (i < 0) i = 0;
    if (j > n2 - 2) j = n2 - 2;
    if (j < 0) j = 0;
    if (k > n3 - 2) k = n3 - 2;
    if (k < 0) k = 0;
    double fx = x - i, fy = y - j, fz = z - k;
    int i1 = (n1 > 1) ? i + 1 : i, j1 = (n2 > 1) ? j + 1 : j, k1 = (n3 > 1) ? k + 1 : k;
#define VV(a, b, c) V[(size_t)(a) + (size_t)n1 * ((b) + (size_t)n2 * (c))]
    double c00 = VV(i, j, k) * (1 - fx) + VV(i1, j, k) * fx;
    double c10 = VV(i, j1, k) * (1 - fx) + VV(i1, j1, k) * fx;
    double c01 = VV(i, j, k1) * (1 - fx) + VV(i1, j, k1) * fx;
    double c11 = VV(i, j1, k1) * (1 - fx) + VV(i1, j1, k1) * fx;
#undef VV
    double c0 = c00 * (1 - fy) + c10 * fy;
    double c1 = c01 * (1 - fy) + c11 * fy;
    return c0 * (1 - fz) + c1 * fz;
}

/* interp3(..., 'cubic', 0) restated as the published method it names:
 * cubic convolution with Keys' kernel (a = -1/2), samples beyond the grid
 * taken from Keys' boundary rule f(-1) = 3 f(0) - 3 f(1) + f(2) (mirrored at
 * the far end), 0 outside [0, n-1] in any dimension.  MATLAB's own code is
 * closed, so parity with it is unpinned.  Needs n >= 4 per dimension. */
static double keys_w(double s)
{
    s = fabs(s);
    if (s <= 1.0) return 1.5 * s * s * s - 2.5 * s * s + 1.0;
    if (s < 2.0) return -0.5 * s * s * s + 2.5 * s * s - 4.0 * s + 2.0;
    return 0.0;
}
static double keys_ext(const double *V, int n1, int n2, int n3, int a, int b, int c)
{
    if (a < 0) return 3 * keys_ext(V, n1, n2, n3, 0, b, c) - 3 * keys_ext(V, n1, n2, n3, 1, b, c) + keys_ext(V, n1, n2, n3, 2, b, c);
    if (a > n1 - 1) return 3 * keys_ext(V, n1, n2, n3, n1 - 1, b, c) - 3 * keys_ext(V, n1, n2, n3, n1 - 2, b, c) + keys_ext(V, n1, n2, n3, n1 - 3, b, c);
    if (b < 0) return 3 * keys_ext(V, n1, n2, n3, a, 0, c) - 3 * keys_ext(V, n1, n2, n3, a, 1, c) + keys_ext(V, n1, n2, n3, a, 2, c);
    if (b > n2 - 1) return 3 * keys_ext(V, n1, n2, n3, a, n2 - 1, c) - 3 * keys_ext(V, n1, n2, n3, a, n2 - 2, c) + keys_ext(V, n1, n2, n3, a, n2 - 3, c);
    if (c < 0) return 3 * keys_ext(V, n1, n2, n3, a, b, 0) - 3 * keys_ext(V, n1, n2, n3, a, b, 1) + keys_ext(V, n1, n2, n3, a, b, 2);
    if (c > n3 - 1) return 3 * keys_ext(V, n1, n2, n3, a, b, n3 - 1) - 3 * keys_ext(V, n1, n2, n3, a, b, n3 - 2) + keys_ext(V, n1, n2, n3, a, b, n3 - 3);
    return V[(size_t)a + (size_t)n1 * (b + (size_t)n2 * c)];
}
static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static double cub(const double *V, int n1, int n2, int n3, double x, double y, double z)
{
    if (!(x >= 0 && y >= 0 && z >= 0 && x <= n1 - 1 && y <= n2 - 1 && z <= n3 - 1)) return 0.0;
    const int i = clampi((int)floor(x), 0, n1 - 2), j = clampi((int)floor(y), 0, n2 - 2), k = clampi((int)floor(z), 0, n3 - 2);
    double s = 0.0;
    for (int c = k - 1; c <= k + 2; ++c) {
        const double wz = keys_w(z - c);
        for (int b = j - 1; b <= j + 2; ++b) {
            const double wy = keys_w(y - b);
            for (int a = i - 1; a <= i + 2; ++a) s += keys_w(x - a) * wy * wz * keys_ext(V, n1, n2, n3, a, b, c);
        }
    }
    return s;
}

/* Proj(i,j) = sum_k Vol(R * [X_i; Y_j; Z_k]) with centred coordinates
 * -ceil((n-1)/2)..floor((n-1)/2) (…RealSpaceinterp.m:17-31, 55); interp 0
 * trilinear, 1 cubic. */
static void project_R_interp(const double *vol, int n1, int n2, int n3, const double R[9], int interp, double *proj)
{
    int c1 = n1 / 2, c2 = n2 / 2, c3 = n3 / 2;
#pragma omp parallel for collapse(2) schedule(static)
    for (int j = 0; j < n2; ++j)
        for (int i = 0; i < n1; ++i) {
            double X = i - c1, Y = j - c2, s = 0.0;
            for (int k = 0; k < n3; ++k) {
                double Z = k - c3;
                double rx = R[0] * X + R[3] * Y + R[6] * Z;
                double ry = R[1] * X + R[4] * Y + R[7] * Z;
                double rz = R[2] * X + R[5] * Y + R[8] * Z;
                s += interp ? cub(vol, n1, n2, n3, rx + c1, ry + c2, rz + c3)
                            : tri(vol, n1, n2, n3, rx + c1, ry + c2, rz + c3);
            }
            proj[(size_t)i + (size_t)n1 * j] = s;
        }
}

void orc_project_R(const double *vol, int n1, int n2, int n3, const double R[9], double *proj)
{
    project_R_interp(vol, n1, n2, n3, R, 0, proj);
}

/* vecs == NULL: the ZYZ closed form of calculate3Dprojection_RealSpaceinterp;
 * otherwise vecs = [v1 v2 v3] as in …_general. */
void orc_project(const double *vol, int n1, int n2, int n3, double phi, double theta, double psi,
                 const double *vecs, double *proj)
{
    double R[9];
    if (vecs) orc_euler_rot(vecs, vecs + 3, vecs + 6, phi, theta, psi, R);
    else orc_rot_zyz(phi, theta, psi, R);
    project_R_interp(vol, n1, n2, n3, R, 0, proj);
}

void orc_project_interp(const double *vol, int n1, int n2, int n3, double phi, double theta, double psi,
                        const double *vecs, int interp, double *proj)
{
    double R[9];
    if (vecs) orc_euler_rot(vecs, vecs + 3, vecs + 6, phi, theta, psi, R);
    else orc_rot_zyz(phi, theta, psi, R);
    project_R_interp(vol, n1, n2, n3, R, interp, proj);
}

/* Tian_calc_Rfactor_realspace.m:1-24: projections with the Z, Y, X axes
 * (calculate3Dprojection_RealSpaceinterpZYX, absent from the reference tree,
 * taken as the general projector with vectors [0 0 1], [0 1 0], [1 0 0]),
 * cropped to p1 x p2 by My_stripzero, Rarr = sum| |bp| - |pj| | / sum|pj|,
 * returns mean(Rarr); simu (p1*p2*P, optional) receives the cropped
 * projections. */
double orc_rfactor_realspace(const double *model, int m1, int m2, int m3, const double *projs, int p1, int p2,
                             int P, const double *angles, int interp, double *Rarr, double *simu)
{
    const double v[9] = {0, 0, 1, 0, 1, 0, 1, 0, 0};
    double *bp = (double *)malloc(sizeof(double) * (size_t)m1 * m2);
    double *cr = (double *)malloc(sizeof(double) * (size_t)p1 * p2);
    int ps[3] = {m1, m2, 1}, os[3] = {p1, p2, 1};
    double tot = 0.0;
    for (int q = 0; q < P; ++q) {
        orc_project_interp(model, m1, m2, m3, angles[q], angles[q + P], angles[q + 2 * P], v, interp, bp);
        orc_stripzero(bp, ps, os, cr);
        const double *pj = projs + (size_t)q * p1 * p2;
        double a = 0.0, b = 0.0;
        for (size_t t = 0; t < (size_t)p1 * p2; ++t) {
            a += fabs(fabs(cr[t]) - fabs(pj[t]));
            b += fabs(pj[t]);
        }
        Rarr[q] = a / b;
        tot += Rarr[q];
        if (simu) memcpy(simu + (size_t)q * p1 * p2, cr, sizeof(double) * (size_t)p1 * p2);
    }
    free(bp);
    free(cr);
    return tot / P;
}

/* R-factors of reconstruct.m:176-177: sum|bp-pj|/sum|pj| and the Frobenius ratio. */
void orc_rfactor(const double *bp, const double *pj, int64_t n, double *R1, double *R2)
{
    double a = 0, b = 0, c = 0, d = 0;
    for (int64_t i = 0; i < n; ++i) {
        double e = bp[i] - pj[i];
        a += fabs(e); b += fabs(pj[i]); c += e * e; d += pj[i] * pj[i];
    }
    *R1 = a / b; *R2 = sqrt(c) / sqrt(d);
}

/* ------------------------------------------------------------------------ */
/* reconstruct.m:28-194                                                        */
/* ------------------------------------------------------------------------ */

/* constraintEnforcementDelayIndicators (GENFIRE_Reconstructor.m:156-165).
 * Colon ranges a:s:b are materialised as a + k*s. Returns the count or -1. */
int orc_delay_indicators(int mode, double *out)
{
    int m = 0;
    if (mode == 1 || mode == 2) {
        for (int k = 0; k < 12; ++k) out[m++] = 0.95 + k * -0.1;
        out[m++] = -10; out[m++] = -10;
        if (mode == 1) {
            out[m++] = -10;
            for (int k = 0; k < 12; ++k) out[m++] = -0.15 + k * 0.1;
        }
        return m;
    }
    if (mode == 3) { for (int k = 0; k < 5; ++k) out[m++] = -999; return m; }
    return -1;
}

/* round(linspace(1, N, m)) (reconstruct.m:103) */
void orc_change_points(int N, int m, int *out)
{
    for (int i = 0; i < m; ++i) {
        double y = (m == 1) ? (double)N : 1.0 + ((double)i * (double)(N - 1)) / (double)(m - 1);
        if (i == m - 1) y = N;
        out[i] = (int)mround(y);
    }
}

/* measuredK: centred n1 x n2 x n1 complex; mask (same size, nullable: then
 * measuredK ~= 0); support D1 x D2 x D1 (nullable: ones); initial D1 x D2 x D1
 * (nullable: zeros).  projs/angles are needed only when monitor_R.
 * rec_out: D1 x D2 x D1.  errK: numIterations.  errR/Rarr/Rarr2: per monitor
 * point (floor(N/loopLength), Rarr/Rarr2 NumProjs per point). */
static double g_loop_seconds = 0.0;
static double *g_iter_start = NULL;  /* wall time at the start of each iteration */
static int g_iter_count = 0;
static double g_loop_end = 0.0;

/* Wall time of the iteration loop of the last orc_reconstruct call (the
 * setup before reconstruct.m:117 excluded). */
double orc_last_loop_seconds(void) { return g_loop_seconds; }

/* Wall time of iterations first+1 .. numIterations of the last
 * orc_reconstruct call (the first `first` iterations as a warm-up); 0 when
 * first is out of range. */
double orc_last_loop_seconds_from(int first)
{
    if (first < 0 || first >= g_iter_count || !g_iter_start) return 0.0;
    return g_loop_end - g_iter_start[first];
}

static double wall(void)
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

/* Rfree candidate points of shell s (0-based) of nbins (reconstruct.m:47-50):
 * find(measuredK ~= 0 & Q >= edge(s) + resRange & Q < edge(s+1)) with
 * edge = linspace(0, 1, nbins + 1) (edge(i) = i / nbins), resRange = -0.05 and
 * Q = make_Kspace_indices of the measuredK-sized grid.  Writes the ascending
 * 0-based linear indices to out (if not NULL) and returns their count. */
int64_t orc_rfree_candidates(int n1, int n2, const double *measuredK, int nbins, int s, int64_t *out)
{
    int sz[3] = {n1, n2, n1};
    size_t N = (size_t)n1 * n2 * n1;
    double *Q = (double *)malloc(sizeof(double) * N);
    orc_make_kspace_indices(sz, Q);
    const double lo = (double)s / (double)nbins + -0.05, hi = (double)(s + 1) / (double)nbins;
    int64_t cnt = 0;
    for (size_t i = 0; i < N; ++i) {
        int nz = measuredK[2 * i] != 0 || measuredK[2 * i + 1] != 0;
        if (nz && Q[i] >= lo && Q[i] < hi) {
            if (out) out[cnt] = (int64_t)i;
            ++cnt;
        }
    }
    free(Q);
    return cnt;
}

int orc_reconstruct_rfree(const orc_params *prm, const double *measuredK, const unsigned char *mask,
                          const unsigned char *support, const double *initial,
                          const double *projs, const double *angles,
                          double *rec_out, double *errK, double *errR, double *Rarr, double *Rarr2,
                          int nshells, const int64_t *rcounts, const int64_t *rind, double *rfree);

int orc_reconstruct(const orc_params *prm, const double *measuredK, const unsigned char *mask,
                    const unsigned char *support, const double *initial,
                    const double *projs, const double *angles,
                    double *rec_out, double *errK, double *errR, double *Rarr, double *Rarr2)
{
    return orc_reconstruct_rfree(prm, measuredK, mask, support, initial, projs, angles, rec_out, errK, errR,
                                 Rarr, Rarr2, 0, NULL, NULL, NULL);
}

/* reconstruct.m with the Rfree monitor (:137-146): rind holds the withheld
 * 0-based centred linear indices of nshells shells (rcounts[s] each,
 * concatenated); the caller has removed them from mask (:65).  Each iteration
 * writes rfree[s + nshells * (it - 1)] = sum |k(shifted) - M| / sum |M| over
 * shell s, with k = fftn of the object before the Fourier constraint. */
int orc_reconstruct_rfree(const orc_params *prm, const double *measuredK, const unsigned char *mask,
                          const unsigned char *support, const double *initial,
                          const double *projs, const double *angles,
                          double *rec_out, double *errK, double *errR, double *Rarr, double *Rarr2,
                          int nshells, const int64_t *rcounts, const int64_t *rind, double *rfree)
{
    int D1 = prm->Dim1, D2 = prm->Dim2;
    int n1 = orc_oversampled_size(D1, prm->oversamplingRatio);
    int n2 = orc_oversampled_size(D2, prm->oversamplingRatio);
    int sz[3] = {n1, n2, n1}, vs[3] = {D1, D2, D1};
    size_t N = (size_t)n1 * n2 * n1, NV = (size_t)D1 * D2 * D1;
    double delay[64];
    int m = orc_delay_indicators(prm->constraintEnforcementMode, delay);
    if (m < 0) return -1;
    int *changes = (int *)malloc(sizeof(int) * m);
    orc_change_points(prm->numIterations, m, changes);

    /* padded support (My_paddzero.m, single in the reference: 0/1 here) and
     * the initial object, both moved to FFT order (ifftshift, :109-110) */
    double *tmp = (double *)malloc(sizeof(double) * NV);
    double *padc = (double *)malloc(sizeof(double) * N);
    double *S = (double *)malloc(sizeof(double) * N);
    double *x = (double *)malloc(sizeof(double) * N);
    double *best = (double *)calloc(N, sizeof(double));
    for (size_t i = 0; i < NV; ++i) tmp[i] = support ? (support[i] ? 1.0 : 0.0) : 1.0;
    orc_paddzero(tmp, vs, sz, padc);
    /* FFT-order index of a centred index: (c + ceil(n/2)) mod n */
#define TOFFT(c1, c2, c3) ((size_t)(((c1) + (n1 + 1) / 2) % n1) + (size_t)n1 * ((((c2) + (n2 + 1) / 2) % n2) + (size_t)n2 * (((c3) + (n1 + 1) / 2) % n1)))
    for (int c3 = 0; c3 < n1; ++c3)
        for (int c2 = 0; c2 < n2; ++c2)
            for (int c1 = 0; c1 < n1; ++c1)
                S[TOFFT(c1, c2, c3)] = padc[(size_t)c1 + (size_t)n1 * (c2 + (size_t)n2 * c3)];
    if (initial) { for (size_t i = 0; i < NV; ++i) tmp[i] = initial[i]; }
    else memset(tmp, 0, sizeof(double) * NV);
    orc_paddzero(tmp, vs, sz, padc);
    for (int c3 = 0; c3 < n1; ++c3)
        for (int c2 = 0; c2 < n2; ++c2)
            for (int c1 = 0; c1 < n1; ++c1)
                x[TOFFT(c1, c2, c3)] = padc[(size_t)c1 + (size_t)n1 * (c2 + (size_t)n2 * c3)];

    /* E = find(measuredK ~= 0 & mask) (:99-100), indicators 1 - Q (:36-42) */
    double *Q = (double *)malloc(sizeof(double) * N);
    orc_make_kspace_indices(sz, Q);
    int64_t nE = 0;
    for (size_t i = 0; i < N; ++i) {
        int nz = measuredK[2 * i] != 0 || measuredK[2 * i + 1] != 0;
        if (nz && (mask ? mask[i] != 0 : 1)) ++nE;
    }
    int64_t *E = (int64_t *)malloc(sizeof(int64_t) * (nE ? nE : 1));
    int64_t *Esh = (int64_t *)malloc(sizeof(int64_t) * (nE ? nE : 1));
    double *ci = (double *)malloc(sizeof(double) * (nE ? nE : 1));
    double denom = 0;
    nE = 0;
    for (size_t i = 0; i < N; ++i) {
        int nz = measuredK[2 * i] != 0 || measuredK[2 * i + 1] != 0;
        if (nz && (mask ? mask[i] != 0 : 1)) {
            int c1 = (int)(i % n1), c2 = (int)((i / n1) % n2), c3 = (int)(i / ((size_t)n1 * n2));
            E[nE] = (int64_t)i; Esh[nE] = (int64_t)TOFFT(c1, c2, c3); ci[nE] = 1.0 - Q[i];
            denom += hypot(measuredK[2 * i], measuredK[2 * i + 1]);
            ++nE;
        }
    }
#undef TOFFT
    unsigned char *inC = (unsigned char *)calloc(nE ? nE : 1, 1);
    double *k = (double *)malloc(sizeof(double) * 2 * N);
    double bestErr = 1e30;
    int cur = 0;          /* 0-based currentCutoffNum */
    int nmon = 0;
    int P = prm->NumProjs;
    int *vi = (int *)malloc(sizeof(int) * 6);
    { int b[3] = {n1, n2, n1}; orc_volumn_index(b, vs, vi); }
    double *model = (double *)malloc(sizeof(double) * NV);
    double *bp = (double *)malloc(sizeof(double) * (size_t)D1 * D2);

    free(g_iter_start);
    g_iter_count = prm->numIterations > 0 ? prm->numIterations : 0;
    g_iter_start = (double *)malloc(sizeof(double) * (g_iter_count ? g_iter_count : 1));
    double t_loop = wall();
    for (int it = 1; it <= prm->numIterations; ++it) {
        if (g_iter_start) g_iter_start[it - 1] = wall();
        if (cur < m && it == changes[cur]) {
            int last = cur;
            for (int c = 0; c < m; ++c) if (changes[c] == it) last = c;
            for (int64_t e = 0; e < nE; ++e) inC[e] = ci[e] > delay[last];
            cur = last + 1;
            bestErr = 1e30;
        }
        if (prm->constraintPositivity) {
#pragma omp parallel for
            for (int64_t i = 0; i < (int64_t)N; ++i) if (x[i] < 0) x[i] = 0;
        }
        if (prm->constraintSupport) {
#pragma omp parallel for
            for (int64_t i = 0; i < (int64_t)N; ++i) x[i] *= S[i];
        }
#pragma omp parallel for
        for (int64_t i = 0; i < (int64_t)N; ++i) { k[2 * i] = x[i]; k[2 * i + 1] = 0; }
        orc_fftn(k, n1, n2, n1, 0);
        double num = 0;
        for (int64_t e = 0; e < nE; ++e) {
            size_t a = (size_t)Esh[e], b = (size_t)E[e];
            num += fabs(hypot(k[2 * a], k[2 * a + 1]) - hypot(measuredK[2 * b], measuredK[2 * b + 1]));
        }
        double err = num / denom;
        errK[it - 1] = err;
        if (nshells > 0 && rfree) {
            int64_t o = 0;
            for (int sh = 0; sh < nshells; ++sh) {
                double rn = 0, rd = 0;
                for (int64_t e = 0; e < rcounts[sh]; ++e, ++o) {
                    size_t b = (size_t)rind[o];
                    int c1 = (int)(b % n1), c2 = (int)((b / n1) % n2), c3 = (int)(b / ((size_t)n1 * n2));
                    size_t a = (size_t)((c1 + (n1 + 1) / 2) % n1) + (size_t)n1 * (((c2 + (n2 + 1) / 2) % n2) + (size_t)n2 * ((c3 + (n1 + 1) / 2) % n1));
                    rn += hypot(k[2 * a] - measuredK[2 * b], k[2 * a + 1] - measuredK[2 * b + 1]);
                    rd += hypot(measuredK[2 * b], measuredK[2 * b + 1]);
                }
                rfree[(size_t)sh + (size_t)nshells * (it - 1)] = rn / rd;
            }
        }
        if (err < bestErr) { bestErr = err; memcpy(best, x, sizeof(double) * N); }
        for (int64_t e = 0; e < nE; ++e)
            if (inC[e]) {
                size_t a = (size_t)Esh[e], b = (size_t)E[e];
                k[2 * a] = measuredK[2 * b]; k[2 * a + 1] = measuredK[2 * b + 1];
            }
        orc_fftn(k, n1, n2, n1, 1);
#pragma omp parallel for
        for (int64_t i = 0; i < (int64_t)N; ++i) x[i] = k[2 * i];

        if (prm->monitor_R == 1 && prm->monitorR_loopLength > 0 && it % prm->monitorR_loopLength == 0) {
            /* model = fftshift(x)(Vol_ind) (:173-174) */
            for (int i3 = 0; i3 < D1; ++i3)
                for (int i2 = 0; i2 < D2; ++i2)
                    for (int i1 = 0; i1 < D1; ++i1) {
                        int c1 = vi[0] - 1 + i1, c2 = vi[1] - 1 + i2, c3 = vi[2] - 1 + i3;
                        size_t src = (size_t)imod(c1 - n1 / 2, n1) + (size_t)n1 * (imod(c2 - n2 / 2, n2) + (size_t)n2 * imod(c3 - n1 / 2, n1));
                        model[(size_t)i1 + (size_t)D1 * (i2 + (size_t)D2 * i3)] = x[src];
                    }
            double s1 = 0, s2 = 0;
            for (int p = 0; p < P; ++p) {
                double r1, r2;
                orc_project(model, D1, D2, D1, angles[p], angles[p + P], angles[p + 2 * P], NULL, bp);
                orc_rfactor(bp, projs + (size_t)D1 * D2 * p, (int64_t)D1 * D2, &r1, &r2);
                if (Rarr) Rarr[(size_t)nmon * P + p] = r1;
                if (Rarr2) Rarr2[(size_t)nmon * P + p] = r2;
                s1 += r1; s2 += r2;
            }
            if (errR) errR[nmon] = s1 / P;
            ++nmon;
        }
    }
    g_loop_end = wall();
    g_loop_seconds = g_loop_end - t_loop;
    /* reconstruction = My_stripzero(fftshift(best), [D1 D2 D1]) (:192) */
    for (int i3 = 0; i3 < D1; ++i3)
        for (int i2 = 0; i2 < D2; ++i2)
            for (int i1 = 0; i1 < D1; ++i1) {
                size_t src = (size_t)imod(i1 - D1 / 2, n1) + (size_t)n1 * (imod(i2 - D2 / 2, n2) + (size_t)n2 * imod(i3 - D1 / 2, n1));
                rec_out[(size_t)i1 + (size_t)D1 * (i2 + (size_t)D2 * i3)] = best[src];
            }
    free(changes); free(tmp); free(padc); free(S); free(x); free(best); free(Q); free(E); free(Esh);
    free(ci); free(inC); free(k); free(vi); free(model); free(bp);
    return 0;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
