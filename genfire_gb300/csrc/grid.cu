// grid.cu -- DFT gridding (fillInFourierGrid_DFT) and the index/symmetry kernels.
//
// Pipeline for P projections (all on the context stream):
//   1. k_sel_count   per row (k2, k3) of the gridded space and projection: the
//                    k1 interval near the plane, FP32 plane test of its
//                    points; the row's count
//   2. CUB           exclusive scan of the row counts (the rows' output
//                    offsets) and the list of rows that hold points
//   3. k_sel_write   per listed row: (index, D, u, v) at its offset, so each
//                    projection's points are in ascending index order, the
//                    order of find()
//   4. k_dft         F_j = sum_b E_v(j,b) sum_a E_u(j,a) P(a,b) per point
//                    (k_dft_tcgen05 in grid_mma.cu for MIXED / FP16_SCALED)
//   5. k_fill_grid   the output grid's zero pattern (CentroSymmetricity's
//                    -0 imaginary parts on the mirrored half)
//   6. k_accum_runs  the entries (projection-major) sorted stably by grid
//                    index; each run of one grid point sums its contributions
//                    in FP64 in projection order and keeps the last exact hit,
//                    the reference's accumulation order
//                    (fillInFourierGrid_DFT.m:268-291), then writes
//                    FS = sum(w F) / sum(w) (or the exact hit), cast to the
//                    output precision, at the point and at its centro mirror
#include "fft.cuh"
#include "internal.h"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <cstring>

namespace gf {

// ===========================================================================
// host geometry
// ===========================================================================
int oversampled(int dim, double ratio) { return (int)mround((double)dim * ratio); }

// MatrixQuaternionRot (fillInFourierGrid_DFT.m:353-363, src/MatrixQuaternionRot.m:1-12)
void quat_rot(const double v[3], double theta_deg, double R[9])
{
    const double pi = 3.14159265358979323846;
    double th = theta_deg * pi / 180.0;
    double nv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double a = v[0] / nv, b = v[1] / nv, c = v[2] / nv;
    double w = std::cos(th / 2), s = -std::sin(th / 2);
    double x = s * a, y = s * b, z = s * c;
    R[0] = 1 - 2 * y * y - 2 * z * z; R[3] = 2 * x * y + 2 * w * z;     R[6] = 2 * x * z - 2 * w * y;
    R[1] = 2 * x * y - 2 * w * z;     R[4] = 1 - 2 * x * x - 2 * z * z; R[7] = 2 * y * z + 2 * w * x;
    R[2] = 2 * x * z + 2 * w * y;     R[5] = 2 * y * z - 2 * w * x;     R[8] = 1 - 2 * x * x - 2 * y * y;
}

static void mat3(const double A[9], const double B[9], double C[9])
{
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i)
            C[i + 3 * j] = A[i] * B[3 * j] + A[i + 3] * B[3 * j + 1] + A[i + 6] * B[3 * j + 2];
}

void euler_rot(const double v1[3], const double v2[3], const double v3[3], double phi, double theta,
               double psi, double R[9])
{
    double A[9], B[9], Cm[9], T[9];
    quat_rot(v1, phi, A);
    quat_rot(v2, theta, B);
    quat_rot(v3, psi, Cm);
    mat3(A, B, T);
    mat3(T, Cm, R);
}

// sind / cosd with exact reduction in degrees
static void sincosd(double x, double *s, double *c)
{
    const double pi = 3.14159265358979323846;
    double r = std::remainder(x, 360.0);
    double q = std::nearbyint(r / 90.0);
    double t = (r - 90.0 * q) * (pi / 180.0);
    double st = std::sin(t), ct = std::cos(t);
    int qi = (((int)q) % 4 + 4) % 4;
    switch (qi) {
    case 0: *s = st; *c = ct; break;
    case 1: *s = ct; *c = -st; break;
    case 2: *s = -st; *c = -ct; break;
    default: *s = -ct; *c = st; break;
    }
}

// closed-form ZYZ matrix (src/calculate3Dprojection_RealSpaceinterp.m:13-15)
void rot_zyz(double phi, double theta, double psi, double R[9])
{
    double sf, cf, st, ct, sp, cp;
    sincosd(phi, &sf, &cf);
    sincosd(theta, &st, &ct);
    sincosd(psi, &sp, &cp);
    R[0] = cp * ct * cf - sp * sf;  R[3] = -sp * ct * cf - cp * sf; R[6] = st * cf;
    R[1] = cp * ct * sf + sp * cf;  R[4] = -sp * ct * sf + cp * cf; R[7] = st * sf;
    R[2] = -cp * st;                R[5] = sp * st;                 R[8] = ct;
}

void proj_geometry(const genfire_params &p, double phi, double theta, double psi, ProjGeom &g)
{
    double R[9];
    euler_rot(p.vector1, p.vector2, p.vector3, phi, theta, psi, R);
    for (int i = 0; i < 9; ++i) g.R[i] = (float)R[i];
    g.nrm[0] = g.R[6]; g.nrm[1] = g.R[7]; g.nrm[2] = g.R[8];
    float nn = std::sqrt(g.nrm[0] * g.nrm[0] + g.nrm[1] * g.nrm[1] + g.nrm[2] * g.nrm[2]);
    g.h[0] = g.nrm[0] / nn; g.h[1] = g.nrm[1] / nn; g.h[2] = g.nrm[2] / nn;
    g.nsq = g.nrm[0] * g.nrm[0] + g.nrm[1] * g.nrm[1] + g.nrm[2] * g.nrm[2];
    g.ih = 1.0f / g.h[0];
    // LU with partial pivoting (first largest pivot), reciprocal column scaling
    float *A = g.lu;
    std::memcpy(A, g.R, sizeof(float) * 9);
    for (int k = 0; k < 3; ++k) {
        int pv = k;
        float best = std::fabs(A[k + 3 * k]);
        for (int i = k + 1; i < 3; ++i)
            if (std::fabs(A[i + 3 * k]) > best) { best = std::fabs(A[i + 3 * k]); pv = i; }
        g.piv[k] = pv;
        if (pv != k)
            for (int j = 0; j < 3; ++j) std::swap(A[k + 3 * j], A[pv + 3 * j]);
        if (A[k + 3 * k] != 0.0f && k < 2) {
            float r = 1.0f / A[k + 3 * k];
            for (int i = k + 1; i < 3; ++i) A[i + 3 * k] = A[i + 3 * k] * r;
        }
        for (int j = k + 1; j < 3; ++j)
            for (int i = k + 1; i < 3; ++i) A[i + 3 * j] = A[i + 3 * j] - A[i + 3 * k] * A[k + 3 * j];
    }
}

GridSpec make_grid(int n1, int n2, int centro)
{
    GridSpec g;
    if (centro) {
        g.lo1 = -(n1 / 2); g.l1 = n1 / 2 + 1;
        g.lo2 = -(n2 / 2); g.l2 = 2 * (n2 / 2) + 1;
        g.lo3 = -(n1 / 2); g.l3 = 2 * (n1 / 2) + 1;
    } else {
        g.lo1 = -(n1 / 2); g.l1 = n1;
        g.lo2 = -(n2 / 2); g.l2 = n2;
        g.lo3 = -(n1 / 2); g.l3 = n1;
    }
    g.total = (long long)g.l1 * g.l2 * g.l3;
    return g;
}

void check_params(const genfire_params &p, bool need_projs)
{
    if (p.Dim1 < 2 || p.Dim2 < 2) fail(GENFIRE_ERR_ARG, "Dim1 and Dim2 must be at least 2.");
    if (need_projs && p.NumProjs < 1) fail(GENFIRE_ERR_ARG, "NumProjs must be positive.");
    if (!(p.oversamplingRatio >= 1.0) || p.oversamplingRatio > 64.0)
        fail(GENFIRE_ERR_ARG, "oversamplingRatio must be in [1, 64].");
    if (!(p.interpolationCutoffDistance > 0.0)) fail(GENFIRE_ERR_ARG, "interpolationCutoffDistance must be positive.");
    if (p.precision != GENFIRE_PREC_FP64 && p.precision != GENFIRE_PREC_MIXED && p.precision != GENFIRE_PREC_FP16_SCALED)
        fail(GENFIRE_ERR_ARG, "precision must be GENFIRE_PREC_FP64, GENFIRE_PREC_MIXED or GENFIRE_PREC_FP16_SCALED.");
    for (const double *v : {p.vector1, p.vector2, p.vector3})
        if (v[0] == 0 && v[1] == 0 && v[2] == 0) fail(GENFIRE_ERR_ARG, "rotation axis vectors must be non-zero.");
    int n1 = oversampled(p.Dim1, p.oversamplingRatio), n2 = oversampled(p.Dim2, p.oversamplingRatio);
    GridSpec g = make_grid(n1, n2, p.DFT_CentroSymmetricity);
    if ((long long)n1 * n2 * n1 >= (1LL << 31) || g.total >= (1LL << 31) - 8192)
        fail(GENFIRE_ERR_ARG, "oversampled grid too large (n1*n2*n1 must stay below 2^31).");
    if (n1 > 65535 || n2 > 65535) fail(GENFIRE_ERR_ARG, "oversampled size too large.");
}

// ===========================================================================
// selection kernels
// ===========================================================================
// The thresholds are FP32 values chosen so the FP32 comparisons decide
// exactly as the reference's comparisons in double do (this part's FP64 pipe
// issues 2 operations per clock per SM, and a double comparison per candidate
// would bound the selection): for a float D, D < cutoff in double holds iff
// D < cut_lt, the smallest float not below cutoff; n/2 is exact in FP32.
struct SelParams {
    int lo1, lo2, lo3, l1, l2, l3;
    int nrows;    // l2 * l3 rows of the gridded index space
    float cut_lt;      // D < cutoff  <=>  D < cut_lt
    float cut_margin;  // cutoff + 0.01 in FP32: the candidate-interval half width
    float half1, half2;
};

// Rows (k2, k3) of the gridded index space are the work units: the points of
// a row that can lie within the cutoff of the plane form one interval of k1,
// found with conservative FP32 bounds; only those candidates get the exact
// test.  Row ri = i2 + l2 i3 holds the linear indices (k1 - lo1) + l1 ri, so
// rows in ascending ri and k1 ascending within a row give the ascending order
// of find().  The count pass runs one thread per row: a CTA is 8 warps, each
// 32 consecutive rows (i2) of one i3.
constexpr int kSelThreads = 256;
constexpr int kSelRowsX = 32, kSelRowsY = kSelThreads / kSelRowsX;

// FP32 plane test of grid point (K1, K2, K3) (distancePointsPlane_YY,
// closestpoint, R \ CP, box filter), with every rounding step explicit.
__device__ __forceinline__ bool sel_test(const ProjGeom &g, const SelParams &sp, float K1, float K2, float K3,
                                         float &D, float &u, float &v)
{
    D = fabsf(__fadd_rn(__fadd_rn(__fmul_rn(K1, g.h[0]), __fmul_rn(K2, g.h[1])), __fmul_rn(K3, g.h[2])));
    if (!(D < sp.cut_lt)) return false;
    const float s = __fadd_rn(__fadd_rn(__fmul_rn(K1, g.nrm[0]), __fmul_rn(K2, g.nrm[1])), __fmul_rn(K3, g.nrm[2]));
    const float t = __fdiv_rn(__fsub_rn(0.0f, s), g.nsq);
    float b[3] = {__fadd_rn(K1, __fmul_rn(t, g.nrm[0])), __fadd_rn(K2, __fmul_rn(t, g.nrm[1])),
                  __fadd_rn(K3, __fmul_rn(t, g.nrm[2]))};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int pv = g.piv[k];
        if (pv != k) { float tmp = b[k]; b[k] = b[pv]; b[pv] = tmp; }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int i = k + 1; i < 3; ++i) b[i] = __fsub_rn(b[i], __fmul_rn(b[k], g.lu[i + 3 * k]));
#pragma unroll
    for (int k = 2; k >= 0; --k) {
        b[k] = __fdiv_rn(b[k], g.lu[k + 3 * k]);
#pragma unroll
        for (int i = 0; i < k; ++i) b[i] = __fsub_rn(b[i], __fmul_rn(b[k], g.lu[i + 3 * k]));
    }
    u = b[0];
    v = b[1];
    return fabsf(b[0]) <= sp.half1 && fabsf(b[1]) <= sp.half2;
}

// Candidate k1 range [k1a, k1b] of row (K2, K3): every k1 with
// |k1 h1 + K2 h2 + K3 h3| below the cutoff, widened by a margin that covers the
// FP32 rounding of D (|error| < 1e-3 for grids up to 2^16) and of the bounds.
// g.ih = 1 / h1 (IEEE division), formed once per projection on the host.
__device__ __forceinline__ void row_range(const ProjGeom &g, const SelParams &sp, float K2, float K3, int &k1a,
                                          int &k1b)
{
    const int lo = sp.lo1, hi = sp.lo1 + sp.l1 - 1;
    const float x = -(K2 * g.h[1] + K3 * g.h[2]);
    const float c = sp.cut_margin;
    const float h1 = g.h[0];
    k1a = lo;
    k1b = hi;
    if (fabsf(h1) >= 0.01f) {
        // bounds through the reciprocal: within a few ulps of the quotients,
        // which the one-point padding below covers
        const float ih = g.ih;
        float b0 = (x - c) * ih, b1 = (x + c) * ih;
        if (b0 > b1) { const float t = b0; b0 = b1; b1 = t; }
        b0 = fmaxf(b0, (float)lo - 4.f);
        b1 = fminf(b1, (float)hi + 4.f);
        k1a = max(lo, (int)floorf(b0) - 1);
        k1b = min(hi, (int)ceilf(b1) + 1);
    } else {
        const float reach = fabsf(h1) * (float)max(-lo, hi);
        if (fabsf(x) > c + reach) { k1a = 1; k1b = 0; }  // empty
    }
}

// Rows whose candidate interval is longer than this are shared by the whole
// warp (lanes take consecutive k1), instead of one lane looping over them:
// planes nearly parallel to k1 give rows of a few hundred candidates, most of
// which pass, and one lane per such row left the passes waiting on a tail.
constexpr int kSelLongRow = 64;

// Points per row (uint16: a row holds at most l1 <= 32769 points).  Grid:
// x = 32-row group along i2, y = group of 32 values of i3 (each thread takes
// i3, i3 + 8, i3 + 16, i3 + 24), z = projection of the batch (p0 + z).
constexpr int kSelI3PerThread = 4;
__global__ void __launch_bounds__(kSelThreads) k_sel_count(const ProjGeom *__restrict__ geo, int p0, SelParams sp,
                                                          uint16_t *__restrict__ rowcnt)
{
    static_assert(sizeof(ProjGeom) % 4 == 0 && sizeof(ProjGeom) / 4 <= kSelThreads, "geometry words");
    __shared__ ProjGeom sg;
    if (threadIdx.x < sizeof(ProjGeom) / 4)
        reinterpret_cast<uint32_t *>(&sg)[threadIdx.x] =
            reinterpret_cast<const uint32_t *>(geo + p0 + blockIdx.z)[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int i2 = blockIdx.x * kSelRowsX + lane;
    const bool valid = i2 < sp.l2;  // the warp stays whole for its ballots
    const float K2 = (float)(sp.lo2 + i2);
    uint16_t *out = rowcnt + (long long)blockIdx.z * sp.nrows + i2;
#pragma unroll 1
    for (int it = 0; it < kSelI3PerThread; ++it) {
        const int i3 = (blockIdx.y * kSelI3PerThread + it) * kSelRowsY + threadIdx.x / kSelRowsX;  // warp-uniform
        if (i3 >= sp.l3) break;
        const float K3 = (float)(sp.lo3 + i3);
        int a0 = 1, a1 = 0;
        if (valid) row_range(sg, sp, K2, K3, a0, a1);
        const bool longrow = a1 - a0 + 1 > kSelLongRow;
        int cnt = 0;
        if (!longrow)
            for (int k1 = a0; k1 <= a1; ++k1) {
                float D, u, v;
                cnt += sel_test(sg, sp, (float)k1, K2, K3, D, u, v) ? 1 : 0;
            }
        for (unsigned lm = __ballot_sync(0xffffffffu, longrow); lm; lm &= lm - 1) {
            const int src = __ffs(lm) - 1;
            const int sa0 = __shfl_sync(0xffffffffu, a0, src), sa1 = __shfl_sync(0xffffffffu, a1, src);
            const float sK2 = __shfl_sync(0xffffffffu, K2, src);
            int c = 0;
            for (int k0 = sa0; k0 <= sa1; k0 += 32) {
                const int k1 = k0 + lane;
                float D, u, v;
                c += __popc(__ballot_sync(0xffffffffu, k1 <= sa1 && sel_test(sg, sp, (float)k1, sK2, K3, D, u, v)));
            }
            if (lane == src) cnt = c;
        }
        if (valid) out[(long long)sp.l2 * i3] = (uint16_t)cnt;
    }
}

// uint32 sum (wraps modulo 2^32) for the offset scan
struct AddU32 {
    __host__ __device__ uint32_t operator()(uint32_t a, uint32_t b) const { return a + b; }
};

// nonzero row count (the rows the write pass visits)
struct RowHolds {
    const uint16_t *cnt;
    __host__ __device__ bool operator()(uint32_t r) const { return cnt[r] != 0; }
};

// Per projection of the batch (one thread each): its point count, from the
// rows' exclusive offsets (rowoff, modulo 2^32) and counts.
__global__ void k_sel_totals(const uint32_t *__restrict__ rowoff, const uint16_t *__restrict__ rowcnt, int np,
                             long long nrows, long long *__restrict__ nk)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const long long last = np * nrows - 1;
    const uint32_t b = rowoff[q * nrows];
    const uint32_t e = q + 1 < np ? rowoff[(q + 1) * nrows] : rowoff[last] + (uint32_t)rowcnt[last];
    nk[q] = (long long)(uint32_t)(e - b);
}

// The row's placement: projection q of the batch, row ri, the candidate
// interval [a0, a1] and the output offset of its first point.
struct SelRow {
    int q, ri, a0, a1;
    float K2, K3;
    long long o;
};
__device__ __forceinline__ SelRow sel_row(const ProjGeom *__restrict__ geo, int p0, const SelParams &sp, uint32_t r,
                                          const uint32_t *__restrict__ rowoff, const long long *__restrict__ doff)
{
    SelRow w;
    w.q = (int)(r / (uint32_t)sp.nrows);
    w.ri = (int)(r - (uint32_t)w.q * (uint32_t)sp.nrows);
    const int i3 = w.ri / sp.l2, i2 = w.ri - i3 * sp.l2;
    w.K2 = (float)(sp.lo2 + i2);
    w.K3 = (float)(sp.lo3 + i3);
    row_range(geo[p0 + w.q], sp, w.K2, w.K3, w.a0, w.a1);
    w.o = doff[p0 + w.q] + (uint32_t)(rowoff[r] - rowoff[(uint32_t)w.q * (uint32_t)sp.nrows]);
    return w;
}

// The listed rows (each holds points), 32 per warp and step of a grid-stride
// loop over the count the list's selection left on the device: the row's
// points at the projection's first output offset (doff) plus the row's offset
// within the projection, in ascending k1.  Rows with more than kSelLongRow
// candidates are queued for k_sel_write_long instead: they are consecutive in
// the list (the rows of planes nearly parallel to k1), and one warp taking 32
// of them in turn was the pass's tail.
__global__ void __launch_bounds__(kSelThreads) k_sel_write(const ProjGeom *__restrict__ geo, int p0, SelParams sp,
                                                          const uint32_t *__restrict__ rows,
                                                          const int *__restrict__ nrows_listed,
                                                          const uint32_t *__restrict__ rowoff,
                                                          const long long *__restrict__ doff,
                                                          uint32_t *__restrict__ ind, float *__restrict__ dist,
                                                          float *__restrict__ uu, float *__restrict__ vv,
                                                          uint32_t *__restrict__ longq, int *__restrict__ nlong)
{
    const int n = *nrows_listed;
    const int lane = threadIdx.x & 31;
    const long long nwarps = (long long)gridDim.x * (kSelThreads / 32);
    for (long long base = ((long long)blockIdx.x * (kSelThreads / 32) + (threadIdx.x >> 5)) * 32; base < n;
         base += nwarps * 32) {
        const long long i = base + lane;
        SelRow w{0, 0, 1, 0, 0.f, 0.f, 0};
        if (i < n) w = sel_row(geo, p0, sp, rows[i], rowoff, doff);
        const bool longrow = w.a1 - w.a0 + 1 > kSelLongRow;
        const unsigned lm = __ballot_sync(0xffffffffu, longrow);
        if (lm) {  // one queue slot per long row, taken by the warp at once
            int at = 0;
            if (lane == 0) at = atomicAdd(nlong, __popc(lm));
            at = __shfl_sync(0xffffffffu, at, 0);
            if (longrow) longq[at + __popc(lm & ((1u << lane) - 1u))] = rows[i];
        }
        if (longrow) continue;
        const ProjGeom &g = geo[p0 + w.q];
        long long o = w.o;
        for (int k1 = w.a0; k1 <= w.a1; ++k1) {
            float D, u, v;
            if (sel_test(g, sp, (float)k1, w.K2, w.K3, D, u, v)) {
                ind[o] = (uint32_t)((k1 - sp.lo1) + sp.l1 * w.ri);
                dist[o] = D;
                uu[o] = u;
                vv[o] = v;
                ++o;
            }
        }
    }
}

// The queued long rows, one per warp (grid-stride): lanes test consecutive k1
// and place their points by the ballot's prefix count, so the row's points
// stay in ascending k1.
__global__ void __launch_bounds__(kSelThreads) k_sel_write_long(const ProjGeom *__restrict__ geo, int p0,
                                                               SelParams sp, const uint32_t *__restrict__ longq,
                                                               const int *__restrict__ nlong,
                                                               const uint32_t *__restrict__ rowoff,
                                                               const long long *__restrict__ doff,
                                                               uint32_t *__restrict__ ind, float *__restrict__ dist,
                                                               float *__restrict__ uu, float *__restrict__ vv)
{
    const int n = *nlong;
    const int lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * (kSelThreads / 32);
    for (int j = blockIdx.x * (kSelThreads / 32) + (threadIdx.x >> 5); j < n; j += nwarps) {
        const SelRow w = sel_row(geo, p0, sp, longq[j], rowoff, doff);
        const ProjGeom &g = geo[p0 + w.q];
        long long o = w.o;
        for (int k0 = w.a0; k0 <= w.a1; k0 += 32) {
            const int k1 = k0 + lane;
            float D = 0.f, u = 0.f, v = 0.f;
            const bool pass = k1 <= w.a1 && sel_test(g, sp, (float)k1, w.K2, w.K3, D, u, v);
            const unsigned bm = __ballot_sync(0xffffffffu, pass);
            if (pass) {
                const long long oo = o + __popc(bm & ((1u << lane) - 1u));
                ind[oo] = (uint32_t)((k1 - sp.lo1) + sp.l1 * w.ri);
                dist[oo] = D;
                uu[oo] = u;
                vv[oo] = v;
            }
            o += __popc(bm);
        }
    }
}

// ===========================================================================
// DFT at the selected points
// ===========================================================================
// exp(-2 pi i a w / n) with the phase reduced in FP64: a*w is exact (w is
// FP32, |a| < 2^20), r = frac(a*w/n) in [-1/2, 1/2].
template <typename T> __device__ __forceinline__ cplx<T> phase(int a, float w, double inv_n);
template <> __device__ __forceinline__ double2 phase<double>(int a, float w, double inv_n)
{
    double t = (double)a * (double)w * inv_n;
    t -= rint(t);
    double s, c;
    sincospi(-2.0 * t, &s, &c);
    return make_double2(c, s);
}
template <> __device__ __forceinline__ float2 phase<float>(int a, float w, double inv_n)
{
    double t = (double)a * (double)w * inv_n;
    t -= rint(t);
    float s, c;
    sincospif((float)(-2.0 * t), &s, &c);
    return make_float2(c, s);
}

constexpr int kDftJ = 8;      // points per CTA (one warp each)
constexpr int kDftA = 16;     // projection rows per shared-memory chunk
constexpr int kDftB = 256;    // projection columns per pass (8 per lane)
constexpr int kDftPitch = kDftB + 1;

struct DftTile {
    int proj;
    int nj;
    long long j0;
};

// One CTA: kDftJ points of one projection.  Warp w owns point j0 + w and
// accumulates Q(b) = sum_a E_u(a) P(a,b) for its lane's 8 columns b, then
// contracts with E_v(b) and reduces across the warp.
template <typename T>
__global__ void __launch_bounds__(256) k_dft(const T *__restrict__ proj, int D1, int D2, int n1, int n2,
                                            const DftTile *__restrict__ tiles, const float *__restrict__ uu,
                                            const float *__restrict__ vv, cplx<T> *__restrict__ F)
{
    __shared__ T Ps[kDftA * kDftPitch];
    __shared__ cplx<T> Eu[kDftJ * kDftA];
    const DftTile tl = tiles[blockIdx.x];
    const T *P = proj + (long long)tl.proj * D1 * D2;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int amin = -(D1 / 2), bmin = -(D2 / 2);
    const double inv1 = 1.0 / (double)n1, inv2 = 1.0 / (double)n2;
    const bool active = w < tl.nj;
    const float my_v = active ? vv[tl.j0 + w] : 0.f;
    cplx<T> acc = mk((T)0, (T)0);
    for (int b0 = 0; b0 < D2; b0 += kDftB) {
        const int nb = min(kDftB, D2 - b0);
        cplx<T> q[kDftB / 32];
#pragma unroll
        for (int m = 0; m < kDftB / 32; ++m) q[m] = mk((T)0, (T)0);
        for (int a0 = 0; a0 < D1; a0 += kDftA) {
            const int na = min(kDftA, D1 - a0);
            __syncthreads();
            for (int idx = threadIdx.x; idx < kDftA * kDftB; idx += blockDim.x) {
                const int a = idx % kDftA, b = idx / kDftA;
                Ps[a * kDftPitch + b] = (a < na && b < nb) ? P[(a0 + a) + (long long)D1 * (b0 + b)] : (T)0;
            }
            if (threadIdx.x < kDftJ * kDftA) {
                const int j = threadIdx.x / kDftA, a = threadIdx.x % kDftA;
                Eu[threadIdx.x] = (j < tl.nj && a < na) ? phase<T>(amin + a0 + a, uu[tl.j0 + j], inv1)
                                                        : mk((T)0, (T)0);
            }
            __syncthreads();
            for (int a = 0; a < na; ++a) {
                const cplx<T> e = Eu[w * kDftA + a];
#pragma unroll
                for (int m = 0; m < kDftB / 32; ++m) {
                    const T pv = Ps[a * kDftPitch + lane + 32 * m];
                    q[m].x += e.x * pv;
                    q[m].y += e.y * pv;
                }
            }
        }
        if (active) {
#pragma unroll
            for (int m = 0; m < kDftB / 32; ++m) {
                const int b = lane + 32 * m;
                if (b < nb) acc = cadd(acc, cmul(q[m], phase<T>(bmin + b0 + b, my_v, inv2)));
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
    }
    if (active && lane == 0) F[tl.j0 + w] = acc;
}

// ===========================================================================
// accumulation, average, mirror
// ===========================================================================
// One pass over the entries sorted (stably) by grid index: the first entry of
// each run sums the run's contributions in their order -- projection order --
// keeps the last exact hit and writes the point's final value into the output
// grid, which k_fill_grid has set to its zero pattern; nothing of the gridded
// space is stored in between.
__global__ void k_iota(uint32_t *__restrict__ v, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[i] = (uint32_t)i;
}

// The output grid (n1 x n2 x n1, dim 1 fastest) before the touched points are
// written: zero, with the imaginary part -0 where CentroSymmetricity mirrors
// (k1 > 0: M(k) = conj(FS(-k)) of an untouched FS(-k) = 0 is (0, -0)), the
// reference's conj of its zero fill.  Grid: x over pairs of c1 (one 16-byte
// store for two complex64 when vec: n1 even and M 16-byte aligned, checked by
// the host), y = c2, z = c3.
template <typename TO>
__global__ void __launch_bounds__(256) k_fill_grid(int n1, int n2, int centro, bool vec, cplx<TO> *__restrict__ M)
{
    const int c1 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (c1 >= n1) return;
    cplx<TO> *row = M + (long long)n1 * (blockIdx.y + (long long)n2 * blockIdx.z);
    const int h = n1 / 2;  // k1 = c1 - h
    const TO z0 = (centro && c1 > h) ? -(TO)0 : (TO)0, z1 = (centro && c1 + 1 > h) ? -(TO)0 : (TO)0;
    if (sizeof(TO) == 4 && vec) {
        *reinterpret_cast<float4 *>(row + c1) = make_float4(0.f, (float)z0, 0.f, (float)z1);
    } else {
        row[c1] = mk((TO)0, z0);
        if (c1 + 1 < n1) row[c1 + 1] = mk((TO)0, z1);
    }
}

// Each run of one grid point (the entries sorted stably by gridded-space
// index, projection-major within a run) sums its contributions in FP64 in
// projection order (fillInFourierGrid_DFT.m:268-291): weight 1/D, except an
// exact hit (D < 1e-7), the last of which replaces the average.  The FP64 path
// forms 1/D in FP64; the reduced-precision paths form it in FP32, as the
// reference forms 1./master_dist in single (:275), and sum in FP64 (the
// products of FP32 values are exact in FP64), which takes the FP64 division
// off a pipe that issues 2 operations per clock per SM.  exact_lt is the
// smallest float not below 1e-7, so dist < exact_lt decides as the double
// comparison does.  The point's
// value is written straight into the output grid: at its own position, and
// conjugated at -k when CentroSymmetricity mirrors it there (k1 < 0, -k inside
// the grid).  FP32 output averages in FP32 from the FP64 sums; FP64 output
// divides in FP64.
template <typename T, typename TO>
__global__ void k_accum_runs(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ order,
                             const float *__restrict__ dist, const cplx<T> *__restrict__ F, long long n,
                             float exact_lt, GridSpec g, int n1, int n2, int centro, cplx<TO> *__restrict__ M)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint32_t li = keys[i];
        if (i > 0 && keys[i - 1] == li) continue;  // not the start of a run
        double2 a = make_double2(0.0, 0.0), e = a;
        double w = 0.0;
        bool hit = false;
        for (long long t = i; t < n && keys[t] == li; ++t) {
            const uint32_t o = order[t];
            const float df = dist[o];
            const cplx<T> f = F[o];
            if (df < exact_lt) {
                e = make_double2((double)f.x, (double)f.y);
                hit = true;
            } else if constexpr (sizeof(T) == 8) {
                const double wgt = 1.0 / (double)df;
                a.x += (double)f.x * wgt;
                a.y += (double)f.y * wgt;
                w += wgt;
            } else {
                const double wgt = (double)(1.0f / df);
                a.x = fma((double)f.x, wgt, a.x);
                a.y = fma((double)f.y, wgt, a.y);
                w += wgt;
            }
        }
        TO x, y;
        if (hit) {
            x = (TO)e.x;
            y = (TO)e.y;
        } else if constexpr (sizeof(TO) == 8) {
            x = a.x / w;
            y = a.y / w;
        } else {
            const float ws = (float)w;
            x = __fdiv_rn((float)a.x, ws);
            y = __fdiv_rn((float)a.y, ws);
        }
        // gridded-space coordinates of li
        const int k1 = g.lo1 + (int)(li % (uint32_t)g.l1);
        const uint32_t r = li / (uint32_t)g.l1;
        const int k2 = g.lo2 + (int)(r % (uint32_t)g.l2), k3 = g.lo3 + (int)(r / (uint32_t)g.l2);
        const int h1 = n1 / 2, h2 = n2 / 2;
        auto inside = [&](int a1, int a2, int a3) {
            return a1 + h1 >= 0 && a1 + h1 < n1 && a2 + h2 >= 0 && a2 + h2 < n2 && a3 + h1 >= 0 && a3 + h1 < n1;
        };
        auto at = [&](int a1, int a2, int a3) {
            return (long long)(a1 + h1) + (long long)n1 * ((a2 + h2) + (long long)n2 * (a3 + h1));
        };
        if (inside(k1, k2, k3) && !(centro && k1 > 0)) M[at(k1, k2, k3)] = mk(x, y);
        if (centro && k1 < 0 && inside(-k1, -k2, -k3)) M[at(-k1, -k2, -k3)] = mk(x, -y);
    }
}

// Linear index into the gridded space of the centred full-grid position
// (c1, c2, c3); conj is set when CentroSymmetricity mirrors k1 > 0 onto -k
// (CentroSymmetricity.m:2-72 reduces to M(k) = conj(FS(-k)) for k1 > 0).
__device__ __forceinline__ long long src_index(const GridSpec &g, int n1, int n2, int centro, int c1, int c2,
                                               int c3, bool &conj)
{
    int k1 = c1 - n1 / 2, k2 = c2 - n2 / 2, k3 = c3 - n1 / 2;
    conj = false;
    if (centro && k1 > 0) { k1 = -k1; k2 = -k2; k3 = -k3; conj = true; }
    return (long long)(k1 - g.lo1) + (long long)g.l1 * ((k2 - g.lo2) + (long long)g.l2 * (k3 - g.lo3));
}

__global__ void k_centro(const double2 *__restrict__ FS, GridSpec g, int n1, int n2, double2 *__restrict__ M)
{
    const int c2 = blockIdx.y, c3 = blockIdx.z;
    const long long row = (long long)n1 * (c2 + (long long)n2 * c3);
    for (int c1 = blockIdx.x * blockDim.x + threadIdx.x; c1 < n1; c1 += gridDim.x * blockDim.x) {
        bool cj;
        const long long li = src_index(g, n1, n2, 1, c1, c2, c3, cj);
        const double2 v = FS[li];
        M[row + c1] = make_double2(v.x, cj ? -v.y : v.y);
    }
}

// hermitianSymmetrize (src/hermitianSymmetrize.m:22-65): mate of (i,j,k) is
// (e1-1-i, e2-1-j, e3-1-k) on the odd-extended grid; values beyond the input
// are zero.
__global__ void k_hermitian(const double2 *__restrict__ in, int d1, int d2, int d3, double2 *__restrict__ out)
{
    const long long N = (long long)d1 * d2 * d3;
    const int e1 = d1 + (d1 % 2 == 0), e2 = d2 + (d2 % 2 == 0), e3 = d3 + (d3 % 2 == 0);
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < N; o += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(o % d1);
        const long long r = o / d1;
        const int j = (int)(r % d2), k = (int)(r / d2);
        const int mi = e1 - 1 - i, mj = e2 - 1 - j, mk_ = e3 - 1 - k;
        const double2 a = in[o];
        double2 b = make_double2(0.0, 0.0);
        if (mi < d1 && mj < d2 && mk_ < d3) b = in[mi + (long long)d1 * (mj + (long long)d2 * mk_)];
        double re = a.x + b.x, im = a.y - b.y;
        const int cnt = (a.x != 0 || a.y != 0) + (b.x != 0 || b.y != 0);
        if (cnt) { re /= cnt; im /= cnt; }
        out[o] = make_double2(re, im);
    }
}

// make_Kspace_indices (src/make_Kspace_indices.m:16-62)
__device__ __forceinline__ double kvec(int n, int i)
{
    if (n == 1) return 0.0;
    const int r = (n % 2 == 0) ? n / 2 : (n - 1) / 2;
    return (double)(i - r) / (double)r;
}

// sqrt(Kx.^2 + Ky.^2 + Kz.^2) rounded step by step (no contraction), so the
// constraint thresholds 1 - Q > delay resolve exactly as in the oracle
__device__ __forceinline__ double q_radius(double kx, double ky, double kz)
{
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz)));
}

__global__ void k_kspace(int d1, int d2, int d3, double *__restrict__ Q)
{
    const long long N = (long long)d1 * d2 * d3;
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < N; o += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(o % d1);
        const long long r = o / d1;
        const int j = (int)(r % d2), k = (int)(r / d2);
        Q[o] = q_radius(kvec(d2, j), kvec(d1, i), kvec(d3, k));
    }
}

// My_iffshift3_ind (src/My_iffshift3_ind.m:1-7), 1-based in and out
__global__ void k_iffshift(int s1, int s2, int s3, long long count, const long long *__restrict__ in,
                           long long *__restrict__ out)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < count; t += (long long)gridDim.x * blockDim.x) {
        const long long i = in[t] - 1;
        long long i1 = i % s1, i2 = (i / s1) % s2, i3 = i / ((long long)s1 * s2);
        i1 = (i1 + (s1 + 1) / 2) % s1;
        i2 = (i2 + (s2 + 1) / 2) % s2;
        i3 = (i3 + (s3 + 1) / 2) % s3;
        out[t] = i1 + (long long)s1 * (i2 + (long long)s2 * i3) + 1;
    }
}

static unsigned grid_for(genfire_ctx *ctx, long long n, int threads)
{
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)ctx->sm_count * 8;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (unsigned)b;
}

// ===========================================================================
// host orchestration
// ===========================================================================
struct Selection {
    DevBuf ind, dist, u, v;
    DevBuf doff;  // off on the device (P + 1 entries)
    std::vector<long long> nk, off;
    long long total = 0;
};

// off[0] = 0, off[p + 1] = off[p] + nk[p]: one CTA of 1024 threads, a block
// scan per 1024 projections with the running total carried
__global__ void __launch_bounds__(1024) k_sel_offsets(const long long *__restrict__ nk, int P, long long *__restrict__ off)
{
    __shared__ long long wsum[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long carry = 0;
    if (threadIdx.x == 0) off[0] = 0;
    for (int base = 0; base < P; base += 1024) {
        const int i = base + threadIdx.x;
        const long long x = i < P ? nk[i] : 0;
        long long inc = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsum[w] = inc;
        __syncthreads();
        long long before = 0, tot = 0;
        for (int k = 0; k < 32; ++k) {
            before += k < w ? wsum[k] : 0;
            tot += wsum[k];
        }
        if (i < P) off[i + 1] = carry + before + inc;
        carry += tot;
        __syncthreads();
    }
}

static void select_points(genfire_ctx *ctx, const GridSpec &g, double cutoff, int n1, int n2,
                          const std::vector<ProjGeom> &geo, Selection &sel)
{
    cudaStream_t st = ctx->stream;
    const int P = (int)geo.size();
    SelParams sp;
    sp.lo1 = g.lo1; sp.lo2 = g.lo2; sp.lo3 = g.lo3; sp.l1 = g.l1; sp.l2 = g.l2; sp.l3 = g.l3;
    sp.nrows = g.l2 * g.l3;
    sp.cut_lt = (float)cutoff;
    if ((double)sp.cut_lt < cutoff) sp.cut_lt = std::nextafter(sp.cut_lt, INFINITY);
    sp.cut_margin = (float)cutoff + 0.01f;
    sp.half1 = (float)(n1 / 2.0); sp.half2 = (float)(n2 / 2.0);
    DevBuf dgeo(sizeof(ProjGeom) * P, st);
    GF_CUDA(cudaMemcpyAsync(dgeo.p, geo.data(), sizeof(ProjGeom) * P, cudaMemcpyHostToDevice, st));

    // Batches of projections with at most 2^30 rows (CUB's item counts are
    // int) and 65535 projections (the count pass's grid z).  Row offsets are uint32 and may wrap across a batch; a projection's
    // own offsets are differences modulo 2^32, exact since it holds fewer than
    // 2^31 points.
    const long long nrows = sp.nrows;
    const int pb = (int)std::max<long long>(1, std::min<long long>(std::min(P, 65535), (1LL << 30) / nrows));
    struct Batch {
        int p0, np;
        DevBuf cnt, off, rows, nlisted;
    };
    std::vector<Batch> batches;
    DevBuf dnk(sizeof(long long) * P, st), tmp;
    for (int p0 = 0; p0 < P; p0 += pb) {
        batches.emplace_back();
        Batch &b = batches.back();
        b.p0 = p0;
        b.np = std::min(pb, P - p0);
        const long long nr = (long long)b.np * nrows;
        b.cnt.alloc(sizeof(uint16_t) * nr, st);
        b.off.alloc(sizeof(uint32_t) * nr, st);
        b.rows.alloc(sizeof(uint32_t) * nr, st);
        b.nlisted.alloc(sizeof(int), st);
        const dim3 grid((unsigned)cdiv(sp.l2, kSelRowsX), (unsigned)cdiv(sp.l3, kSelRowsY * kSelI3PerThread),
                        (unsigned)b.np);
        k_sel_count<<<grid, kSelThreads, 0, st>>>(dgeo.as<ProjGeom>(), p0, sp, b.cnt.as<uint16_t>());
        GF_CHECK_LAUNCH();
        const thrust::counting_iterator<uint32_t> ids(0);
        const RowHolds holds{b.cnt.as<uint16_t>()};
        size_t t1 = 0, t2 = 0;
        GF_CUDA(cub::DeviceScan::ExclusiveScan(nullptr, t1, b.cnt.as<uint16_t>(), b.off.as<uint32_t>(), AddU32(),
                                               (uint32_t)0, (int)nr, st));
        GF_CUDA(cub::DeviceSelect::If(nullptr, t2, ids, b.rows.as<uint32_t>(), b.nlisted.as<int>(), (int)nr, holds, st));
        if (std::max(t1, t2) > tmp.bytes) tmp.alloc(std::max(t1, t2), st);
        GF_CUDA(cub::DeviceScan::ExclusiveScan(tmp.p, t1, b.cnt.as<uint16_t>(), b.off.as<uint32_t>(), AddU32(),
                                               (uint32_t)0, (int)nr, st));
        GF_CUDA(cub::DeviceSelect::If(tmp.p, t2, ids, b.rows.as<uint32_t>(), b.nlisted.as<int>(), (int)nr, holds, st));
        k_sel_totals<<<(unsigned)cdiv(b.np, 128), 128, 0, st>>>(b.off.as<uint32_t>(), b.cnt.as<uint16_t>(), b.np,
                                                                 nrows, dnk.as<long long>() + p0);
        GF_CHECK_LAUNCH();
    }
    sel.doff.alloc(sizeof(long long) * (P + 1), st);
    k_sel_offsets<<<1, 1024, 0, st>>>(dnk.as<long long>(), P, sel.doff.as<long long>());
    GF_CHECK_LAUNCH();
    sel.nk.assign(P, 0);
    GF_CUDA(cudaMemcpyAsync(sel.nk.data(), dnk.p, sizeof(long long) * P, cudaMemcpyDeviceToHost, st));
    GF_CUDA(cudaStreamSynchronize(st));
    sel.off.assign(P + 1, 0);
    for (int p = 0; p < P; ++p) sel.off[p + 1] = sel.off[p] + sel.nk[p];
    sel.total = sel.off[P];
    if (sel.total >= (1LL << 31)) fail(GENFIRE_ERR_ARG, "more than 2^31 selected points in one gridding call.");
    const size_t nt = (size_t)std::max<long long>(sel.total, 1);
    sel.ind.alloc(nt * sizeof(uint32_t), st);
    sel.dist.alloc(nt * sizeof(float), st);
    sel.u.alloc(nt * sizeof(float), st);
    sel.v.alloc(nt * sizeof(float), st);
    // one full wave of resident CTAs for each grid-stride write pass
    int per_sm = 0, per_sm_long = 0;
    GF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sel_write, kSelThreads, 0));
    GF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_long, k_sel_write_long, kSelThreads, 0));
    const unsigned wgrid = (unsigned)std::max(1, per_sm) * (unsigned)ctx->sm_count;
    const unsigned lgrid = (unsigned)std::max(1, per_sm_long) * (unsigned)ctx->sm_count;
    for (Batch &b : batches) {
        // the long-row queue: at most one entry per row of the batch
        DevBuf lq(sizeof(uint32_t) * (size_t)b.np * (size_t)nrows, st), nlong(sizeof(int), st);
        GF_CUDA(cudaMemsetAsync(nlong.p, 0, sizeof(int), st));
        k_sel_write<<<wgrid, kSelThreads, 0, st>>>(
            dgeo.as<ProjGeom>(), b.p0, sp, b.rows.as<uint32_t>(), b.nlisted.as<int>(), b.off.as<uint32_t>(),
            sel.doff.as<long long>(), sel.ind.as<uint32_t>(), sel.dist.as<float>(), sel.u.as<float>(),
            sel.v.as<float>(), lq.as<uint32_t>(), nlong.as<int>());
        GF_CHECK_LAUNCH();
        k_sel_write_long<<<lgrid, kSelThreads, 0, st>>>(
            dgeo.as<ProjGeom>(), b.p0, sp, lq.as<uint32_t>(), nlong.as<int>(), b.off.as<uint32_t>(),
            sel.doff.as<long long>(), sel.ind.as<uint32_t>(), sel.dist.as<float>(), sel.u.as<float>(),
            sel.v.as<float>());
        GF_CHECK_LAUNCH();
    }
}

// CUDA events on the context stream between the stages of a gridding call
struct StageEvents {
    std::vector<cudaEvent_t> ev;
    StageEvents(int n, bool on)
    {
        if (!on) return;
        ev.resize(n);
        for (auto &e : ev) GF_CUDA(cudaEventCreate(&e));
    }
    ~StageEvents()
    {
        for (auto &e : ev) cudaEventDestroy(e);
    }
    void mark(int i, cudaStream_t st)
    {
        if (!ev.empty()) GF_CUDA(cudaEventRecord(ev[i], st));
    }
    cudaEvent_t event(int i) const { return ev.empty() ? nullptr : ev[i]; }
    double ms(int a, int b)
    {
        float t = 0;
        GF_CUDA(cudaEventElapsedTime(&t, ev[a], ev[b]));
        return t;
    }
};

template <typename T>
static void grid_dft_t(genfire_ctx *ctx, const genfire_params &p, const double *d_proj, const double *angles,
                       void *d_M, void *d_rec, int64_t *nk_out, double *stage_ms)
{
    cudaStream_t st = ctx->stream;
    StageEvents se(9, stage_ms != nullptr);
    se.mark(0, st);
    const int D1 = p.Dim1, D2 = p.Dim2, P = p.NumProjs;
    const int n1 = oversampled(D1, p.oversamplingRatio), n2 = oversampled(D2, p.oversamplingRatio);
    const GridSpec g = make_grid(n1, n2, p.DFT_CentroSymmetricity);
    std::vector<ProjGeom> geo(P);
    for (int i = 0; i < P; ++i) proj_geometry(p, angles[i], angles[i + P], angles[i + 2 * P], geo[i]);

    Selection sel;
    select_points(ctx, g, p.interpolationCutoffDistance, n1, n2, geo, sel);
    if (nk_out)
        for (int i = 0; i < P; ++i) nk_out[i] = sel.nk[i];
    se.mark(1, st);

    DevBuf F(sizeof(cplx<T>) * (size_t)std::max<long long>(sel.total, 1), st);
    double dft_kernel_ms = 0;
    DevBuf dft_err(sizeof(int), st);  // set by the tensor-core DFT when a bounded wait expired
    GF_CUDA(cudaMemsetAsync(dft_err.p, 0, sizeof(int), st));
    if (sizeof(T) == sizeof(float)) {
        // MIXED / FP16_SCALED: split-BF16 / split-FP16 tensor-core DFT (grid_mma.cu)
        dft_tcgen05(ctx, d_proj, D1, D2, n1, n2, P, sel.nk, sel.doff.as<long long>(), sel.u.as<float>(),
                    sel.v.as<float>(), reinterpret_cast<float2 *>(F.p), dft_err.as<int>(), se.event(6), se.event(7),
                    p.precision == GENFIRE_PREC_FP16_SCALED);
    } else {
        // FP64: kDftJ consecutive points of one projection per CTA
        std::vector<DftTile> tiles;
        tiles.reserve((size_t)(sel.total / kDftJ + P));
        for (int i = 0; i < P; ++i)
            for (long long j = 0; j < sel.nk[i]; j += kDftJ)
                tiles.push_back(DftTile{i, (int)std::min<long long>(kDftJ, sel.nk[i] - j), sel.off[i] + j});
        if (!tiles.empty()) {
            DevBuf dt(sizeof(DftTile) * tiles.size(), st);
            GF_CUDA(cudaMemcpyAsync(dt.p, tiles.data(), sizeof(DftTile) * tiles.size(), cudaMemcpyHostToDevice, st));
            se.mark(6, st);
            k_dft<double><<<(unsigned)tiles.size(), 256, 0, st>>>(d_proj, D1, D2, n1, n2, dt.as<DftTile>(),
                                                                   sel.u.as<float>(), sel.v.as<float>(),
                                                                   reinterpret_cast<double2 *>(F.p));
            GF_CHECK_LAUNCH();
            se.mark(7, st);
        }
    }
    se.mark(2, st);

    // weighted average in FP64, projection by projection
    const size_t G = (size_t)g.total;
    // the output grid's zero pattern, then the touched points written over it
    const bool vec = (n1 % 2 == 0) && (reinterpret_cast<uintptr_t>(d_M) % 16 == 0);
    k_fill_grid<T><<<dim3(cdiv(n1, 512), n2, n1), 256, 0, st>>>(n1, n2, p.DFT_CentroSymmetricity, vec,
                                                                reinterpret_cast<cplx<T> *>(d_M));
    GF_CHECK_LAUNCH();
    se.mark(8, st);
    if (sel.total > 0) {
        // stable radix sort of (grid index, entry) keeps projection order within a grid point
        const long long n = sel.total;
        int bits = 1;
        while (bits < 32 && (1ull << bits) < (unsigned long long)G) ++bits;
        DevBuf keys(sizeof(uint32_t) * n, st), vin(sizeof(uint32_t) * n, st), vout(sizeof(uint32_t) * n, st);
        k_iota<<<grid_for(ctx, n, 256), 256, 0, st>>>(vin.as<uint32_t>(), n);
        GF_CHECK_LAUNCH();
        size_t tb = 0;
        GF_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, sel.ind.as<uint32_t>(), keys.as<uint32_t>(),
                                                vin.as<uint32_t>(), vout.as<uint32_t>(), n, 0, bits, st));
        DevBuf tmp(std::max<size_t>(tb, 1), st);
        GF_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, sel.ind.as<uint32_t>(), keys.as<uint32_t>(),
                                                vin.as<uint32_t>(), vout.as<uint32_t>(), n, 0, bits, st));
        float exact_lt = 1e-7f;  // the smallest float not below 1e-7
        if ((double)exact_lt < 1e-7) exact_lt = std::nextafter(exact_lt, INFINITY);
        k_accum_runs<T, T><<<grid_for(ctx, n, 256), 256, 0, st>>>(keys.as<uint32_t>(), vout.as<uint32_t>(),
                                                                   sel.dist.as<float>(), F.as<cplx<T>>(), n,
                                                                   exact_lt, g, n1,
                                                                   n2, p.DFT_CentroSymmetricity,
                                                                   reinterpret_cast<cplx<T> *>(d_M));
        GF_CHECK_LAUNCH();
    }
    se.mark(3, st);
    se.mark(4, st);
    if (d_rec) rec_ifft(ctx, p.precision, d_M, n1, n2, D1, D2, d_rec);
    se.mark(5, st);
    int herr = 0;
    GF_CUDA(cudaMemcpyAsync(&herr, dft_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GF_CUDA(cudaStreamSynchronize(st));
    if (herr) fail(GENFIRE_ERR_TIMEOUT, "tensor-core gridding: a bounded wait for the tensor core or a bulk copy expired.");
    if (stage_ms) {
        dft_kernel_ms = sel.total > 0 ? se.ms(6, 7) : 0.0;
        stage_ms[0] = se.ms(0, 1);  // selection
        stage_ms[1] = se.ms(1, 2);  // DFT stage (operand preparation and the DFT kernel)
        stage_ms[2] = dft_kernel_ms;  // the DFT kernel alone
        stage_ms[3] = se.ms(8, 3);  // sort, weighted sums, average, centro mirror, cast (written into the grid)
        stage_ms[4] = se.ms(2, 8);  // the output grid's zero pattern
        stage_ms[5] = se.ms(4, 5);  // recIFFT
    }
}

void grid_dft(genfire_ctx *ctx, const genfire_params &p, const double *d_proj, const double *angles, void *d_M,
              void *d_rec, int64_t *nk, double *stage_ms)
{
    if (p.precision == GENFIRE_PREC_FP64) grid_dft_t<double>(ctx, p, d_proj, angles, d_M, d_rec, nk, stage_ms);
    else grid_dft_t<float>(ctx, p, d_proj, angles, d_M, d_rec, nk, stage_ms);
}

long long select_one(genfire_ctx *ctx, const genfire_params &p, double phi, double theta, double psi,
                     long long cap, int64_t *ind, float *dist, float *u, float *v)
{
    const int n1 = oversampled(p.Dim1, p.oversamplingRatio), n2 = oversampled(p.Dim2, p.oversamplingRatio);
    const GridSpec g = make_grid(n1, n2, p.DFT_CentroSymmetricity);
    std::vector<ProjGeom> geo(1);
    proj_geometry(p, phi, theta, psi, geo[0]);
    Selection sel;
    select_points(ctx, g, p.interpolationCutoffDistance, n1, n2, geo, sel);
    const long long n = sel.total;
    if (n > cap) fail(GENFIRE_ERR_ARG, "select: cap smaller than the number of selected points.");
    std::vector<uint32_t> hi(n);
    cudaStream_t st = ctx->stream;
    if (n) {
        GF_CUDA(cudaMemcpyAsync(hi.data(), sel.ind.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaMemcpyAsync(dist, sel.dist.p, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaMemcpyAsync(u, sel.u.p, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaMemcpyAsync(v, sel.v.p, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
    }
    for (long long i = 0; i < n; ++i) ind[i] = hi[i];
    return n;
}

void centro_device(genfire_ctx *ctx, const double2 *d_FS, int n1, int n_k1, int n2, double2 *d_M)
{
    (void)n_k1;
    const GridSpec g = make_grid(n1, n2, 1);
    k_centro<<<dim3(cdiv(n1, 256), n2, n1), 256, 0, ctx->stream>>>(d_FS, g, n1, n2, d_M);
    GF_CHECK_LAUNCH();
}

void hermitian_device(genfire_ctx *ctx, const double2 *d_in, int d1, int d2, int d3, double2 *d_out)
{
    const long long N = (long long)d1 * d2 * d3;
    k_hermitian<<<grid_for(ctx, N, 256), 256, 0, ctx->stream>>>(d_in, d1, d2, d3, d_out);
    GF_CHECK_LAUNCH();
}

void kspace_device(genfire_ctx *ctx, int d1, int d2, int d3, double *d_Q)
{
    const long long N = (long long)d1 * d2 * d3;
    k_kspace<<<grid_for(ctx, N, 256), 256, 0, ctx->stream>>>(d1, d2, d3, d_Q);
    GF_CHECK_LAUNCH();
}

void iffshift_device(genfire_ctx *ctx, const int sz[3], long long count, const long long *d_in, long long *d_out)
{
    k_iffshift<<<grid_for(ctx, count, 256), 256, 0, ctx->stream>>>(sz[0], sz[1], sz[2], count, d_in, d_out);
    GF_CHECK_LAUNCH();
}

}  // namespace gf
