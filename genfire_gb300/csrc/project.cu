// project.cu -- the real-space projector and the R-factor reductions.
//
// calculate3Dprojection_RealSpaceinterp(_general) rotates the centred voxel
// grid by R, samples the volume there and sums along dimension 3
// (src/calculate3Dprojection_RealSpaceinterp.m:17-55).  Here one thread owns
// one output pixel and walks the rotated line through the volume with
// trilinear interpolation (0 outside the volume); the volume of a 256^3
// reconstruction (67 MB in FP32) stays resident in the 129 MB L2.  The
// R-factor sums of reconstruct.m:176-177 are fused into the same kernel
// and reduced with warp shuffles, per projection, in a fixed order.
#include "internal.h"

namespace gf {

template <typename T> struct Coord;

// FP64: coordinates and weights in double with explicit rounding steps.
template <> struct Coord<double> {
    static __device__ __forceinline__ double lin(double a, double x, double b, double y, double c, double z)
    {
        return __dadd_rn(__dadd_rn(__dmul_rn(a, x), __dmul_rn(b, y)), __dmul_rn(c, z));
    }
};
template <> struct Coord<float> {
    static __device__ __forceinline__ float lin(double a, double x, double b, double y, double c, double z)
    {
        return (float)fma(c, z, fma(b, y, a * x));
    }
};

template <typename T>
__device__ __forceinline__ T trilinear(const T *__restrict__ V, int n1, int n2, int n3, long long vs1, long long vs2,
                                       T x, T y, T z)
{
    if (!(x >= (T)0 && y >= (T)0 && z >= (T)0 && x <= (T)(n1 - 1) && y <= (T)(n2 - 1) && z <= (T)(n3 - 1)))
        return (T)0;
    int i = (int)floor(x), j = (int)floor(y), k = (int)floor(z);
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

constexpr int kProjThreads = 256;

template <typename T>
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
        for (int k = 0; k < n3; ++k) {
            const double Z = k - c3;
            const T rx = Coord<T>::lin(R[0], X, R[3], Y, R[6], Z);
            const T ry = Coord<T>::lin(R[1], X, R[4], Y, R[7], Z);
            const T rz = Coord<T>::lin(R[2], X, R[5], Y, R[8], Z);
            part_acc += trilinear<T>(vol, n1, n2, n3, vs1, vs2, rx + (T)c1, ry + (T)c2, rz + (T)c3);
            if ((k & 15) == 15) { acc += (double)part_acc; part_acc = 0; }
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
    k_project<T><<<grid, kProjThreads, 0, st>>>(vol, n1, n2, n3, vs1, vs2, d_R, d_proj, d_meas, part.as<double>());
    GF_CHECK_LAUNCH();
    if (d_meas) {
        k_project_sums<<<P, 32, 0, st>>>(part.as<double>(), (int)nblk, d_sums);
        GF_CHECK_LAUNCH();
    }
    (void)ctx;
}

void project_batch(genfire_ctx *ctx, int precision, const void *d_vol, int n1, int n2, int n3, long long vs1,
                   long long vs2, int P, const double *d_R, void *d_proj, const double *d_measured, double *d_sums,
                   cudaStream_t stream)
{
    if (n1 < 2 || n2 < 2 || n3 < 2) fail(GENFIRE_ERR_ARG, "projector: every volume dimension must be at least 2.");
    if (precision == GENFIRE_PREC_FP64)
        project_t<double>(ctx, (const double *)d_vol, n1, n2, n3, vs1, vs2, P, d_R, (double *)d_proj, d_measured,
                          d_sums, stream);
    else
        project_t<float>(ctx, (const float *)d_vol, n1, n2, n3, vs1, vs2, P, d_R, (float *)d_proj, d_measured,
                         d_sums, stream);
}

}  // namespace gf
