// project.cu -- the real-space projector and the R-factor reductions.
//
// calculate3Dprojection_RealSpaceinterp(_general) rotates the centred voxel
// grid by R, samples the volume there and sums along dimension 3
// (src/calculate3Dprojection_RealSpaceinterp.m:17-55).  Here one thread owns
// one output pixel and walks the rotated line through the volume with
// trilinear interpolation (the default) or the cubic convolution of interp3
// 'cubic' (:45), both 0 outside the volume; the volume of a 256^3
// reconstruction (67 MB in FP32) stays resident in the 129 MB L2.  The
// R-factor sums of reconstruct.m:176-177 are fused into the same kernel
// and reduced with warp shuffles, per projection, in a fixed order.
#include "internal.h"

#include <map>
#include <mutex>

namespace gf {

template <typename T> struct Coord;

// FP64: coordinates and weights in double with explicit rounding steps.
template <> struct Coord<double> {
    static __device__ __forceinline__ double lin(double a, double x, double b, double y, double c, double z)
    {
        return __dadd_rn(__dadd_rn(__dmul_rn(a, x), __dmul_rn(b, y)), __dmul_rn(c, z));
    }
};

// floor in the argument's own precision (the float path must not round through FP64)
__device__ __forceinline__ float floor_t(float x) { return floorf(x); }
__device__ __forceinline__ double floor_t(double x) { return floor(x); }

template <typename T>
__device__ __forceinline__ T trilinear(const T *__restrict__ V, int n1, int n2, int n3, long long vs1, long long vs2,
                                       T x, T y, T z)
{
    if (!(x >= (T)0 && y >= (T)0 && z >= (T)0 && x <= (T)(n1 - 1) && y <= (T)(n2 - 1) && z <= (T)(n3 - 1)))
        return (T)0;
    int i = (int)floor_t(x), j = (int)floor_t(y), k = (int)floor_t(z);
    i = min(i, n1 - 2); j = min(j, n2 - 2); k = min(k, n3 - 2);
    i = max(i, 0); j = max(j, 0); k = max(k, 0);
    const T fx = x - (T)i, fy = y - (T)j, fz = z - (T)k;
    const int i1 = n1 > 1 ? i + 1 : i;
    const long long j0o = (long long)j * vs1, j1o = (long long)(n2 > 1 ? j + 1 : j) * vs1;
    const long long k0o = (long long)k * vs2, k1o = (long long)(n3 > 1 ? k + 1 : k) * vs2;
    const T v000 = V[i + j0o + k0o], v100 = V[i1 + j0o + k0o];
    const T v010 = V[i + j1o + k0o], v110 = V[i1 + j1o + k0o];
    const T v001 = V[i + j0o + k1o], v101 = V[i1 + j0o + k1o];
    const T v011 = V[i + j1o + k1o], v111 = V[i1 + j1o + k1o];
    const T c00 = v000 * ((T)1 - fx) + v100 * fx;
    const T c10 = v010 * ((T)1 - fx) + v110 * fx;
    const T c01 = v001 * ((T)1 - fx) + v101 * fx;
    const T c11 = v011 * ((T)1 - fx) + v111 * fx;
    const T c0 = c00 * ((T)1 - fy) + c10 * fy;
    const T c1 = c01 * ((T)1 - fy) + c11 * fy;
    return c0 * ((T)1 - fz) + c1 * fz;
}

// interp3(..., 'cubic', 0) on a uniform grid: separable cubic convolution
// with Keys' kernel (a = -1/2) and Keys' boundary rule f(-1) = 3 f(0) - 3 f(1)
// + f(2) (and its mirror at the far end), 0 outside [0, n-1] in any
// dimension.  MATLAB's own implementation is closed; this is the published
// method it names (cubic convolution), restated.  Needs n >= 4 per dimension.
// Per dimension: the 4 consecutive indices from s and their weights, with the
// boundary rule folded in.
template <typename T> __device__ __forceinline__ void keys_taps(T x, int n, int &s, T (&e)[4])
{
    int i = (int)floor_t(x);
    i = min(max(i, 0), n - 2);
    const T t = x - (T)i, t2 = t * t, t3 = t2 * t;
    const T wm = (T)0.5 * (-t3 + (T)2 * t2 - t);            // index i - 1
    const T w0 = (T)0.5 * ((T)3 * t3 - (T)5 * t2 + (T)2);   // i
    const T w1 = (T)0.5 * ((T)-3 * t3 + (T)4 * t2 + t);     // i + 1
    const T w2 = (T)0.5 * (t3 - t2);                        // i + 2
    if (i == 0) {            // f(-1) = 3 f(0) - 3 f(1) + f(2)
        s = 0;
        e[0] = w0 + (T)3 * wm; e[1] = w1 - (T)3 * wm; e[2] = w2 + wm; e[3] = (T)0;
    } else if (i == n - 2) { // f(n) = 3 f(n-1) - 3 f(n-2) + f(n-3)
        s = n - 4;
        e[0] = (T)0; e[1] = wm + w2; e[2] = w0 - (T)3 * w2; e[3] = w1 + (T)3 * w2;
    } else {
        s = i - 1;
        e[0] = wm; e[1] = w0; e[2] = w1; e[3] = w2;
    }
}

template <typename T>
__device__ __forceinline__ T tricubic(const T *__restrict__ V, int n1, int n2, int n3, long long vs1, long long vs2,
                                      T x, T y, T z)
{
    if (!(x >= (T)0 && y >= (T)0 && z >= (T)0 && x <= (T)(n1 - 1) && y <= (T)(n2 - 1) && z <= (T)(n3 - 1)))
        return (T)0;
    int si, sj, sk;
    T ex[4], ey[4], ez[4];
    keys_taps<T>(x, n1, si, ex);
    keys_taps<T>(y, n2, sj, ey);
    keys_taps<T>(z, n3, sk, ez);
    T acc = (T)0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        T accy = (T)0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const T *row = V + si + (long long)(sj + b) * vs1 + (long long)(sk + c) * vs2;
            const T ax = ex[0] * row[0] + ex[1] * row[1] + ex[2] * row[2] + ex[3] * row[3];
            accy += ey[b] * ax;
        }
        acc += ez[c] * accy;
    }
    return acc;
}

// Trilinear sample of a float volume with no conversion instructions (this
// part routes float<->int conversions and rounding to a narrow pipe): for
// 0 <= x < 2^22, t = x + 1.5*2^23 holds round-to-nearest(x) in its low mantissa
// bits, one step down where that exceeds x gives floor(x) and its integer; the
// result equals trilinear<float> bit for bit.
__device__ __forceinline__ void floor_split(float x, float hi, int &i, float &f)
{
    const float t = __fadd_rn(x, 12582912.0f);
    float fl = __fsub_rn(t, 12582912.0f);
    int n = __float_as_int(t) - 0x4B400000;
    if (fl > x) { fl -= 1.0f; n -= 1; }
    if (fl > hi) { fl = hi; n = __float_as_int(__fadd_rn(hi, 12582912.0f)) - 0x4B400000; }  // clamp to n - 2
    i = n;
    f = x - fl;
}
__device__ __forceinline__ float trilinear_f(const float *__restrict__ V, float e1, float e2, float e3, float h1,
                                             float h2, float h3, long long vs1, long long vs2, float x, float y,
                                             float z)
{
    if (!(x >= 0.f && y >= 0.f && z >= 0.f && x <= e1 && y <= e2 && z <= e3)) return 0.f;
    int i, j, k;
    float fx, fy, fz;
    floor_split(x, h1, i, fx);
    floor_split(y, h2, j, fy);
    floor_split(z, h3, k, fz);
    const long long j0o = (long long)j * vs1, j1o = j0o + vs1, k0o = (long long)k * vs2, k1o = k0o + vs2;
    const float v000 = V[i + j0o + k0o], v100 = V[i + 1 + j0o + k0o];
    const float v010 = V[i + j1o + k0o], v110 = V[i + 1 + j1o + k0o];
    const float v001 = V[i + j0o + k1o], v101 = V[i + 1 + j0o + k1o];
    const float v011 = V[i + j1o + k1o], v111 = V[i + 1 + j1o + k1o];
    const float c00 = v000 * (1.f - fx) + v100 * fx;
    const float c10 = v010 * (1.f - fx) + v110 * fx;
    const float c01 = v001 * (1.f - fx) + v101 * fx;
    const float c11 = v011 * (1.f - fx) + v111 * fx;
    const float c0 = c00 * (1.f - fy) + c10 * fy;
    const float c1 = c01 * (1.f - fy) + c11 * fy;
    return c0 * (1.f - fz) + c1 * fz;
}

template <typename T, bool CUBIC>
__device__ __forceinline__ T sample(const T *__restrict__ V, int n1, int n2, int n3, long long vs1, long long vs2,
                                    T x, T y, T z)
{
    if constexpr (CUBIC) return tricubic<T>(V, n1, n2, n3, vs1, vs2, x, y, z);
    else return trilinear<T>(V, n1, n2, n3, vs1, vs2, x, y, z);
}

constexpr int kProjThreads = 256;

template <typename T, bool CUBIC>
__global__ void __launch_bounds__(kProjThreads)
    k_project(const T *__restrict__ vol, int n1, int n2, int n3, long long vs1, long long vs2,
              const double *__restrict__ Rs, T *__restrict__ proj, const double *__restrict__ measured,
              double *__restrict__ part)
{
    const int p = blockIdx.y;
    const double *R = Rs + 9 * (long long)p;
    const long long npix = (long long)n1 * n2;
    const long long pix = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double s[4] = {0, 0, 0, 0};
    if (pix < npix) {
        const int i = (int)(pix % n1), j = (int)(pix / n1);
        const int c1 = n1 / 2, c2 = n2 / 2, c3 = n3 / 2;
        const double X = i - c1, Y = j - c2;
        double acc = 0;
        T part_acc = 0;
        if constexpr (sizeof(T) == sizeof(double)) {
            // FP64: the oracle's operation order, ((R0 X + R3 Y) + R6 Z), each rounded
            for (int k = 0; k < n3; ++k) {
                const double Z = k - c3;
                const T rx = Coord<T>::lin(R[0], X, R[3], Y, R[6], Z);
                const T ry = Coord<T>::lin(R[1], X, R[4], Y, R[7], Z);
                const T rz = Coord<T>::lin(R[2], X, R[5], Y, R[8], Z);
                part_acc += sample<T, CUBIC>(vol, n1, n2, n3, vs1, vs2, rx + (T)c1, ry + (T)c2, rz + (T)c3);
                if ((k & 15) == 15) { acc += (double)part_acc; part_acc = 0; }
            }
        } else {
            // FP32: the pixel's part R0 X + R3 Y (+ the centre) once in FP64, rounded
            // to float; per sample one FP32 fma with the third column (this part runs
            // FP64 at 2 operations per clock per SM, so the loop stays FP32)
            const float bx = (float)(R[0] * X + R[3] * Y + c1), by = (float)(R[1] * X + R[4] * Y + c2),
                        bz = (float)(R[2] * X + R[5] * Y + c3);
            const float r6 = (float)R[6], r7 = (float)R[7], r8 = (float)R[8];
            float Z = (float)(-c3);  // stepped by exact additions of 1
            if constexpr (CUBIC) {
                for (int k = 0; k < n3; ++k, Z += 1.f) {
                    part_acc += sample<T, CUBIC>(vol, n1, n2, n3, vs1, vs2, fmaf(Z, r6, bx), fmaf(Z, r7, by), fmaf(Z, r8, bz));
                    if ((k & 15) == 15) { acc += (double)part_acc; part_acc = 0; }
                }
            } else if (n1 >= 2 && n2 >= 2 && n3 >= 2) {
                const float e1 = (float)(n1 - 1), e2 = (float)(n2 - 1), e3 = (float)(n3 - 1);
                const float h1 = (float)(n1 - 2), h2 = (float)(n2 - 2), h3 = (float)(n3 - 2);
                for (int k = 0; k < n3; ++k, Z += 1.f) {
                    part_acc += trilinear_f(reinterpret_cast<const float *>(vol), e1, e2, e3, h1, h2, h3, vs1, vs2,
                                            fmaf(Z, r6, bx), fmaf(Z, r7, by), fmaf(Z, r8, bz));
                    if ((k & 15) == 15) { acc += (double)part_acc; part_acc = 0; }
                }
            } else {
                for (int k = 0; k < n3; ++k, Z += 1.f) {
                    part_acc += sample<T, CUBIC>(vol, n1, n2, n3, vs1, vs2, fmaf(Z, r6, bx), fmaf(Z, r7, by), fmaf(Z, r8, bz));
                    if ((k & 15) == 15) { acc += (double)part_acc; part_acc = 0; }
                }
            }
        }
        acc += (double)part_acc;
        if (proj) proj[(long long)p * npix + pix] = (T)acc;
        if (measured) {
            const double pj = measured[(long long)p * npix + pix];
            const double d = acc - pj;
            s[0] = fabs(d); s[1] = fabs(pj); s[2] = d * d; s[3] = pj * pj;
        }
    }
    if (!measured) return;
    __shared__ double red[4][kProjThreads / 32];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        double v = s[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0;
        for (int w = 0; w < kProjThreads / 32; ++w) v += red[threadIdx.x][w];
        part[((long long)p * gridDim.x + blockIdx.x) * 4 + threadIdx.x] = v;
    }
}

// per-projection sums over the block partials, in block order
__global__ void k_project_sums(const double *__restrict__ part, int nblk, double *__restrict__ sums)
{
    const int p = blockIdx.x;
    if (threadIdx.x >= 4) return;
    double v = 0;
    for (int b = 0; b < nblk; ++b) v += part[((long long)p * nblk + b) * 4 + threadIdx.x];
    sums[4 * p + threadIdx.x] = v;
}

template <typename T>
static void project_t(genfire_ctx *ctx, const T *vol, int n1, int n2, int n3, long long vs1, long long vs2, int P,
                      const double *d_R, T *d_proj, const double *d_meas, double *d_sums, cudaStream_t st)
{
    const long long npix = (long long)n1 * n2;
    const unsigned nblk = cdiv(npix, kProjThreads);
    DevBuf part;
    if (d_meas) part.alloc(sizeof(double) * 4 * (size_t)nblk * P, st);
    dim3 grid(nblk, P);
    if (ctx->interp == GENFIRE_INTERP_CUBIC)
        k_project<T, true><<<grid, kProjThreads, 0, st>>>(vol, n1, n2, n3, vs1, vs2, d_R, d_proj, d_meas,
                                                          part.as<double>());
    else
        k_project<T, false><<<grid, kProjThreads, 0, st>>>(vol, n1, n2, n3, vs1, vs2, d_R, d_proj, d_meas,
                                                           part.as<double>());
    GF_CHECK_LAUNCH();
    if (d_meas) {
        k_project_sums<<<P, 32, 0, st>>>(part.as<double>(), (int)nblk, d_sums);
        GF_CHECK_LAUNCH();
    }
}

void project_batch(genfire_ctx *ctx, int precision, const void *d_vol, int n1, int n2, int n3, long long vs1,
                   long long vs2, int P, const double *d_R, void *d_proj, const double *d_measured, double *d_sums,
                   cudaStream_t stream)
{
    if (n1 < 2 || n2 < 2 || n3 < 2) fail(GENFIRE_ERR_ARG, "projector: every volume dimension must be at least 2.");
    if (ctx->interp == GENFIRE_INTERP_CUBIC && (n1 < 4 || n2 < 4 || n3 < 4))
        fail(GENFIRE_ERR_ARG, "projector: cubic interpolation needs at least 4 samples in every dimension.");
    if (precision == GENFIRE_PREC_FP64)
        project_t<double>(ctx, (const double *)d_vol, n1, n2, n3, vs1, vs2, P, d_R, (double *)d_proj, d_measured,
                          d_sums, stream);
    else
        project_t<float>(ctx, (const float *)d_vol, n1, n2, n3, vs1, vs2, P, d_R, (float *)d_proj, d_measured,
                         d_sums, stream);
}

// ===========================================================================
// Tian_calc_Rfactor_realspace (src/Tian_calc_Rfactor_realspace.m:1-24): the
// ZYX projections of a model, cropped to the measured size (My_stripzero),
// Rarr = sum| |bp| - |pj| | / sum|pj| per projection, their mean, and the
// simulated projections in single precision.
// ===========================================================================
template <typename T>
__global__ void __launch_bounds__(256) k_rfactor_rs(const T *__restrict__ bp, int m1, int m2, int o1, int o2,
                                                    const double *__restrict__ pj, int p1, int p2,
                                                    float *__restrict__ simu, double *__restrict__ sums)
{
    const int p = blockIdx.x;
    const T *b = bp + (size_t)p * m1 * m2;
    const double *q = pj + (size_t)p * p1 * p2;
    double s0 = 0, s1 = 0;
    for (int t = threadIdx.x; t < p1 * p2; t += blockDim.x) {
        const int i = t % p1, j = t / p1;
        const T v = b[(o1 + i) + (size_t)m1 * (o2 + j)];
        const double x = q[t];
        s0 += fabs(fabs((double)v) - fabs(x));
        s1 += fabs(x);
        if (simu) simu[(size_t)p * p1 * p2 + t] = (float)v;
    }
    __shared__ double red[2][8];
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_down_sync(0xffffffffu, s0, o);
        s1 += __shfl_down_sync(0xffffffffu, s1, o);
    }
    if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = s0; red[1][threadIdx.x >> 5] = s1; }
    __syncthreads();
    if (threadIdx.x < 2) {
        double v = 0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) v += red[threadIdx.x][w];
        sums[2 * p + threadIdx.x] = v;
    }
}

// My_stripzero's crop start along a dimension of size big kept to size ori
static int strip_start(int big, int ori)
{
    if (big % 2 == 0) return ori % 2 == 0 ? (big - ori) / 2 : (big - ori + 1) / 2;
    return ori % 2 == 0 ? (big - ori - 1) / 2 : (big - ori) / 2;
}

void rfactor_realspace(genfire_ctx *ctx, int precision, const void *d_model, int m1, int m2, int m3, int P,
                       const double *angles, const double *d_projs, int p1, int p2, double *Rarr, double *Rtotal,
                       float *d_simu)
{
    if (p1 > m1 || p2 > m2) fail(GENFIRE_ERR_ARG, "rfactor_realspace: the projections are larger than the model.");
    cudaStream_t st = ctx->stream;
    // calculate3Dprojection_RealSpaceinterpZYX: the general projector with the
    // axes Z, Y, X for phi, theta, psi
    const double v[9] = {0, 0, 1, 0, 1, 0, 1, 0, 0};
    std::vector<double> Rs(9 * (size_t)P);
    for (int q = 0; q < P; ++q) euler_rot(v, v + 3, v + 6, angles[q], angles[q + P], angles[q + 2 * P], &Rs[9 * (size_t)q]);
    const size_t es = precision == GENFIRE_PREC_FP64 ? sizeof(double) : sizeof(float);
    DevBuf dR(sizeof(double) * Rs.size(), st), bp(es * (size_t)m1 * m2 * P, st), sums(sizeof(double) * 2 * P, st);
    GF_CUDA(cudaMemcpyAsync(dR.p, Rs.data(), sizeof(double) * Rs.size(), cudaMemcpyHostToDevice, st));
    project_batch(ctx, precision, d_model, m1, m2, m3, m1, (long long)m1 * m2, P, dR.as<double>(), bp.p, nullptr,
                  nullptr, st);
    const int o1 = strip_start(m1, p1), o2 = strip_start(m2, p2);
    if (precision == GENFIRE_PREC_FP64)
        k_rfactor_rs<double><<<P, 256, 0, st>>>(bp.as<double>(), m1, m2, o1, o2, d_projs, p1, p2, d_simu,
                                                sums.as<double>());
    else
        k_rfactor_rs<float><<<P, 256, 0, st>>>(bp.as<float>(), m1, m2, o1, o2, d_projs, p1, p2, d_simu,
                                               sums.as<double>());
    GF_CHECK_LAUNCH();
    std::vector<double> hs(2 * (size_t)P);
    GF_CUDA(cudaMemcpyAsync(hs.data(), sums.p, sizeof(double) * hs.size(), cudaMemcpyDeviceToHost, st));
    GF_CUDA(cudaStreamSynchronize(st));
    double tot = 0;
    for (int q = 0; q < P; ++q) {
        const double r = hs[2 * q] / hs[2 * q + 1];
        if (Rarr) Rarr[q] = r;
        tot += r;
    }
    if (Rtotal) *Rtotal = tot / P;
}

// ===========================================================================
// R-factors without allocation (genfire_rfactor_noalloc)
//
// For callers that hold their data in device memory they do not own and may
// not allocate more (for example a MEX function working on gpuArray data inside
// MATLAB's memory manager, or a service that reserves the device's memory for
// its own pool): the rotation matrices, the per-block partial sums and the
// per-projection sums live in this file-scope device array instead of
// cudaMalloc'd buffers.  Every GPU that loads the library holds the array until
// the process exits.  All calls share it: calls whose GPU work overlaps (two
// host threads, or two streams) race on it.  Nothing in it needs to start at
// zero: each call writes every value it reads before reading it.
// ===========================================================================
constexpr size_t kNoAllocScratchBytes = 4u << 20;  // 4 MiB
static __device__ __align__(256) unsigned char g_rfactor_scratch[kNoAllocScratchBytes];

// Device address of the array in the current context.  Looked up on every
// call (cudaGetSymbolAddress allocates nothing and is cheap once the module is
// loaded): an address cached across calls would go stale when the device is
// reset (MATLAB's reset(gpuDevice), cudaDeviceReset in another library), and a
// kernel given it would write to memory that is no longer mapped.
static unsigned char *noalloc_scratch()
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_rfactor_scratch);
    if (e != cudaSuccess || !p)
        fail(GENFIRE_ERR_CUDA, std::string("cudaGetSymbolAddress of the R-factor scratch array failed: ") +
                                   cudaGetErrorString(e));
    return static_cast<unsigned char *>(p);
}

size_t rfactor_noalloc_bytes(int n1, int n2, int P)
{
    const size_t nblk = cdiv((size_t)n1 * n2, kProjThreads);
    const size_t a = (sizeof(double) * 9 * (size_t)P + 255) / 256 * 256;     // rotation matrices
    const size_t b = (sizeof(double) * 4 * nblk * (size_t)P + 255) / 256 * 256;  // block partials
    return a + b + sizeof(double) * 4 * (size_t)P;                          // per-projection sums
}

// Rotation matrices go up and the per-projection sums come back through
// fixed-size chunks on the stack, so the call makes no heap allocation either.
void rfactor_noalloc(genfire_ctx *ctx, int precision, const void *d_vol, int n1, int n2, int n3, int P,
                     const double *angles, const double *vectors, const double *d_measured, double *Rarr,
                     double *Rarr2, double *errR)
{
    const size_t need = rfactor_noalloc_bytes(n1, n2, P);
    if (need > kNoAllocScratchBytes)
        fail(GENFIRE_ERR_ARG, "rfactor_noalloc: the inputs need more than the 4 MiB static scratch "
                              "(fewer projections per call, or genfire_rfactor).");
    cudaStream_t st = ctx->stream;
    unsigned char *base = noalloc_scratch();
    const unsigned nblk = cdiv((size_t)n1 * n2, kProjThreads);
    double *dR = reinterpret_cast<double *>(base);
    double *part = reinterpret_cast<double *>(base + (sizeof(double) * 9 * (size_t)P + 255) / 256 * 256);
    double *dsum = reinterpret_cast<double *>(reinterpret_cast<unsigned char *>(part) +
                                              (sizeof(double) * 4 * nblk * (size_t)P + 255) / 256 * 256);
    constexpr int CH = 64;
    double chunk[CH * 9];
    for (int c0 = 0; c0 < P; c0 += CH) {
        const int cn = P - c0 < CH ? P - c0 : CH;
        for (int i = 0; i < cn; ++i) {
            const int q = c0 + i;
            if (vectors) euler_rot(vectors, vectors + 3, vectors + 6, angles[q], angles[q + P], angles[q + 2 * P], chunk + 9 * i);
            else rot_zyz(angles[q], angles[q + P], angles[q + 2 * P], chunk + 9 * i);
        }
        // pageable source: the copy is staged before the call returns, so the chunk can be refilled
        GF_CUDA(cudaMemcpyAsync(dR + 9 * (size_t)c0, chunk, sizeof(double) * 9 * cn, cudaMemcpyHostToDevice, st));
    }
    dim3 grid(nblk, P);
    const bool cub = ctx->interp == GENFIRE_INTERP_CUBIC;
    if (cub && (n1 < 4 || n2 < 4 || n3 < 4))
        fail(GENFIRE_ERR_ARG, "projector: cubic interpolation needs at least 4 samples in every dimension.");
    const long long s1 = n1, s2 = (long long)n1 * n2;
    if (precision == GENFIRE_PREC_FP64) {
        const double *v = (const double *)d_vol;
        if (cub) k_project<double, true><<<grid, kProjThreads, 0, st>>>(v, n1, n2, n3, s1, s2, dR, nullptr, d_measured, part);
        else k_project<double, false><<<grid, kProjThreads, 0, st>>>(v, n1, n2, n3, s1, s2, dR, nullptr, d_measured, part);
    } else {
        const float *v = (const float *)d_vol;
        if (cub) k_project<float, true><<<grid, kProjThreads, 0, st>>>(v, n1, n2, n3, s1, s2, dR, nullptr, d_measured, part);
        else k_project<float, false><<<grid, kProjThreads, 0, st>>>(v, n1, n2, n3, s1, s2, dR, nullptr, d_measured, part);
    }
    GF_CHECK_LAUNCH();
    k_project_sums<<<P, 32, 0, st>>>(part, (int)nblk, dsum);
    GF_CHECK_LAUNCH();
    double tot = 0;
    for (int c0 = 0; c0 < P; c0 += CH) {
        const int cn = P - c0 < CH ? P - c0 : CH;
        GF_CUDA(cudaMemcpyAsync(chunk, dsum + 4 * (size_t)c0, sizeof(double) * 4 * cn, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
        for (int i = 0; i < cn; ++i) {
            const double *sm = chunk + 4 * i;
            const double r1 = sm[0] / sm[1], r2 = std::sqrt(sm[2]) / std::sqrt(sm[3]);
            if (Rarr) Rarr[c0 + i] = r1;
            if (Rarr2) Rarr2[c0 + i] = r2;
            tot += r1;
        }
    }
    if (errR) *errR = tot / P;
}

}  // namespace gf
