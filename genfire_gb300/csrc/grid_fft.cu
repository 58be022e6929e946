// grid_fft.cu -- FFT gridding, @GENFIRE_Reconstructor/fillInFourierGrid.m
// (griddingMethod = 1, the class default), on the GPU.
//
//   1. k_pad_ishift    each projection zero-padded to m x m with its centre kept
//                      (My_paddzero) and ifftshifted, in the pass precision
//   2. 2-D FFT         the column passes of fft.cuh along dims 1 and 2, batched
//                      over the projections (my_fft, fillInFourierGrid.m:59-61)
//   3. k_fft_scatter   one thread per (pixel, projection): slice coordinate
//                      R'(kx, ky, 0) in FP32 (:80-89), nearest voxel plus the
//                      shifts within round(cutoff) (:108-139), FP32 distance
//                      test, weight 1/(d + 1e-5) (:155-157), FP64 atomic sums of
//                      w*F and w (:159-160)
//   4. k_fft_finalize  FS = sum(w F) / sum(w) (:161) and hermitianSymmetrize
//                      (:163, src/hermitianSymmetrize.m:22-65) in one pass,
//                      cast to the output precision
//   5. recIFFT         rec_ifft (dr.cu): My_stripzero(real(my_ifft(K))) (:165)
//
// Differences from the reference, by design: the sums are FP64 (the reference
// accumulates single-precision products with accumarray), and they are atomic,
// so their order -- and the last bits of a sum with several terms -- does not
// follow the reference's list order.  The FP64 path also transforms the
// projections in FP64 (the reference pads to single precision); the MIXED
// path transforms in FP32 as the reference does.
#include "internal.h"

namespace gf {

int fft_grid_size(int Dim2, double ratio)
{
    const double m = (Dim2 % 2 == 0) ? (double)Dim2 * ratio : 1.0 + (double)(Dim2 - 1) * ratio;
    const double r = mround(m);
    if (std::fabs(m - r) > 1e-9 || r < 1 || r > 65535) return -1;
    return (int)r;
}

void grid_dims(const genfire_params &p, int &n1, int &n2)
{
    if (p.griddingMethod == 1) {
        const int m = fft_grid_size(p.Dim2, p.oversamplingRatio);
        if (m < 0)
            fail(GENFIRE_ERR_ARG, "FFT gridding: Dim2 * oversamplingRatio (1 + (Dim2-1) * oversamplingRatio for odd "
                                  "Dim2) must be an integer.");
        n1 = n2 = m;
    } else {
        n1 = oversampled(p.Dim1, p.oversamplingRatio);
        n2 = oversampled(p.Dim2, p.oversamplingRatio);
    }
}

__device__ __forceinline__ int wrap(int a, int n)
{
    a %= n;
    return a < 0 ? a + n : a;
}

// grid: x over dim 1 of the projection, y = dim-2 index, z = projection
template <typename T>
__global__ void k_pad_ishift(const double *__restrict__ proj, int D1, int D2, int m, cplx<T> *__restrict__ X)
{
    const int y = blockIdx.y, p = blockIdx.z;
    const int ty = wrap(y - D2 / 2, m);
    const double *src = proj + (size_t)p * D1 * D2 + (size_t)D1 * y;
    cplx<T> *dst = X + (size_t)p * m * m + (size_t)m * ty;
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < D1; x += gridDim.x * blockDim.x)
        dst[wrap(x - D1 / 2, m)] = mk((T)src[x], (T)0);
}

struct FftGridGeom {
    int m, s;           // cube size, shift range
    float cut_le;       // for a float d: d <= cutoff (in double) iff d <= cut_le, the largest float not above it
};

// grid: x over the centred dim-1 index i, y = j, z = projection
template <typename T>
__global__ void __launch_bounds__(128) k_fft_scatter(const cplx<T> *__restrict__ X, const float *__restrict__ rot,
                                                     FftGridGeom g, double2 *__restrict__ num,
                                                     double *__restrict__ ws, unsigned long long *__restrict__ pairs)
{
    const int m = g.m, h = m / 2;
    const int j = blockIdx.y, p = blockIdx.z;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned cnt = 0;
    if (i < m) {
        // centred (i, j) of my_fft = FFT index (i - h, j - h) mod m
        const cplx<T> val = X[(size_t)p * m * m + wrap(i - h, m) + (size_t)m * wrap(j - h, m)];
        if (!(val.x == (T)-999 && val.y == (T)0)) {
            const float *r = rot + 6 * p;
            const float kx = (float)(i - h), ky = (float)(j - h);
            const float cx = __fadd_rn(__fmul_rn(r[0], kx), __fmul_rn(r[1], ky));
            const float cy = __fadd_rn(__fmul_rn(r[2], kx), __fmul_rn(r[3], ky));
            const float cz = __fadd_rn(__fmul_rn(r[4], kx), __fmul_rn(r[5], ky));
            const float rx = roundf(cx), ry = roundf(cy), rz = roundf(cz);
            for (int ys = -g.s; ys <= g.s; ++ys)
                for (int xs = -g.s; xs <= g.s; ++xs)
                    for (int zs = -g.s; zs <= g.s; ++zs) {
                        const float tx = __fadd_rn(rx, (float)xs), ty = __fadd_rn(ry, (float)ys),
                                    tz = __fadd_rn(rz, (float)zs);
                        const int ix = (int)tx + h, iy = (int)ty + h, iz = (int)tz + h;
                        if (ix < 0 || ix >= m || iy < 0 || iy >= m || iz < 0 || iz >= m) continue;
                        const float dx = __fsub_rn(cx, tx), dy = __fsub_rn(cy, ty), dz = __fsub_rn(cz, tz);
                        const float d = __fsqrt_rn(
                            __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
                        if (!(d <= g.cut_le)) continue;
                        const double w = (double)__fdiv_rn(1.0f, __fadd_rn(d, 1e-5f));
                        const size_t v = (size_t)ix + (size_t)m * (iy + (size_t)m * iz);
                        atomicAdd(&num[v].x, (double)val.x * w);
                        atomicAdd(&num[v].y, (double)val.y * w);
                        atomicAdd(&ws[v], w);
                        ++cnt;
                    }
        }
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(pairs, (unsigned long long)cnt);
}

// sum(w F) / sum(w) where sum(w) > 0, else 0: in FP64 for the FP64 output,
// in FP32 from the FP64 sums for the single-precision output (no FP64
// arithmetic: this part's FP64 pipe issues 2 operations per clock per SM).
// The weight sum is >= 0, so it is positive iff its bits, as an integer, are.
template <typename TO>
__device__ __forceinline__ cplx<TO> fs_avg(const double2 *__restrict__ num, const double *__restrict__ ws, size_t v)
{
    cplx<TO> a = mk((TO)0, (TO)0);
    if (reinterpret_cast<const long long *>(ws)[v] > 0) {
        const double2 s = num[v];
        if constexpr (sizeof(TO) == 8) {
            const double w = ws[v];
            a = mk(s.x / w, s.y / w);
        } else {
            const float w = (float)ws[v];
            a = mk(__fdiv_rn((float)s.x, w), __fdiv_rn((float)s.y, w));
        }
    }
    return a;
}

// grid: x over dim 1, y = dim-2 index, z = dim-3 index of the m^3 cube.
// hermitianSymmetrize: mate of (i, j, k) is (e-1-i, e-1-j, e-1-k) on the
// odd-extended cube (e = m + 1 for even m), zero beyond the input; the two
// values are averaged over the number of non-zero ones.
template <typename TO>
__global__ void k_fft_finalize(const double2 *__restrict__ num, const double *__restrict__ ws, int m,
                               cplx<TO> *__restrict__ M)
{
    const int j = blockIdx.y, k = blockIdx.z;
    const int e = m + (m % 2 == 0);
    const int mj = e - 1 - j, mk_ = e - 1 - k;
    const size_t row = (size_t)m * (j + (size_t)m * k);
    const size_t mrow = (size_t)m * (mj + (size_t)m * mk_);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const int mi = e - 1 - i;
        const cplx<TO> a = fs_avg<TO>(num, ws, row + i);
        cplx<TO> b = mk((TO)0, (TO)0);
        if (mi < m && mj < m && mk_ < m) b = fs_avg<TO>(num, ws, mrow + mi);
        TO re = a.x + b.x, im = a.y - b.y;
        const int cnt = (a.x != 0 || a.y != 0) + (b.x != 0 || b.y != 0);
        if (cnt == 2) { re *= (TO)0.5; im *= (TO)0.5; }
        M[row + i] = mk(re, im);
    }
}

template <typename T>
static void grid_fft_t(genfire_ctx *ctx, const genfire_params &p, const double *d_proj, const double *angles,
                       void *d_M, void *d_rec, int64_t *npairs)
{
    cudaStream_t st = ctx->stream;
    const int D1 = p.Dim1, D2 = p.Dim2, P = p.NumProjs;
    const int m = fft_grid_size(D2, p.oversamplingRatio);
    const size_t mm = (size_t)m * m, N = mm * m;
    // 1-2: centred spectra of the padded projections (kept in FFT order)
    DevBuf X(sizeof(cplx<T>) * mm * P, st);
    GF_CUDA(cudaMemsetAsync(X.p, 0, X.bytes, st));
    k_pad_ishift<T><<<dim3(cdiv(D1, 128), D2, P), 128, 0, st>>>(d_proj, D1, D2, m, X.as<cplx<T>>());
    GF_CHECK_LAUNCH();
    fftn_device(ctx, sizeof(T) == 8 ? GENFIRE_PREC_FP64 : GENFIRE_PREC_MIXED, X.p, m, m, P, false, 3);
    // slice rotation: rotkCoords = R' [kx; ky; 0] with R of fillInFourierGrid.m:80-82,
    // which is the transpose of the projector's ZYZ matrix, so the rows are
    // (Rz(1,1), Rz(1,2)), (Rz(2,1), Rz(2,2)), (Rz(3,1), Rz(3,2)) in single precision
    std::vector<float> hr(6 * (size_t)P);
    for (int q = 0; q < P; ++q) {
        double R[9];
        rot_zyz(angles[q], angles[q + P], angles[q + 2 * P], R);
        float *r = &hr[6 * (size_t)q];
        r[0] = (float)R[0]; r[1] = (float)R[3];
        r[2] = (float)R[1]; r[3] = (float)R[4];
        r[4] = (float)R[2]; r[5] = (float)R[5];
    }
    DevBuf drot(sizeof(float) * hr.size(), st), dpairs(sizeof(unsigned long long), st);
    GF_CUDA(cudaMemcpyAsync(drot.p, hr.data(), sizeof(float) * hr.size(), cudaMemcpyHostToDevice, st));
    GF_CUDA(cudaMemsetAsync(dpairs.p, 0, sizeof(unsigned long long), st));
    // 3: weighted sums on the cube
    DevBuf num(sizeof(double2) * N, st), ws(sizeof(double) * N, st);
    GF_CUDA(cudaMemsetAsync(num.p, 0, num.bytes, st));
    GF_CUDA(cudaMemsetAsync(ws.p, 0, ws.bytes, st));
    FftGridGeom g;
    g.m = m;
    g.s = p.allowMultipleGridMatches ? (int)mround(p.interpolationCutoffDistance) : 0;
    g.cut_le = (float)p.interpolationCutoffDistance;
    if ((double)g.cut_le > p.interpolationCutoffDistance) g.cut_le = std::nextafter(g.cut_le, -INFINITY);
    k_fft_scatter<T><<<dim3(cdiv(m, 128), m, P), 128, 0, st>>>(X.as<cplx<T>>(), drot.as<float>(), g,
                                                               num.as<double2>(), ws.as<double>(),
                                                               dpairs.as<unsigned long long>());
    GF_CHECK_LAUNCH();
    X.release();
    // 4: average and Hermitian symmetry
    k_fft_finalize<T><<<dim3(cdiv(m, 256), m, m), 256, 0, st>>>(num.as<double2>(), ws.as<double>(), m,
                                                                 reinterpret_cast<cplx<T> *>(d_M));
    GF_CHECK_LAUNCH();
    num.release();
    ws.release();
    // 5: recIFFT
    if (d_rec) rec_ifft(ctx, p.precision, d_M, m, m, D1, D2, d_rec);
    unsigned long long hp = 0;
    GF_CUDA(cudaMemcpyAsync(&hp, dpairs.p, sizeof(hp), cudaMemcpyDeviceToHost, st));
    GF_CUDA(cudaStreamSynchronize(st));
    if (npairs) *npairs = (int64_t)hp;
}

void grid_fft(genfire_ctx *ctx, const genfire_params &p, const double *d_proj, const double *angles, void *d_M,
              void *d_rec, int64_t *npairs)
{
    const int m = fft_grid_size(p.Dim2, p.oversamplingRatio);
    if (m < 0)
        fail(GENFIRE_ERR_ARG, "FFT gridding: Dim2 * oversamplingRatio (1 + (Dim2-1) * oversamplingRatio for odd "
                              "Dim2) must be an integer.");
    if (m < p.Dim1 || m < p.Dim2) fail(GENFIRE_ERR_ARG, "FFT gridding: the grid is smaller than the projections.");
    if ((long long)m * m * m >= (1LL << 31)) fail(GENFIRE_ERR_ARG, "FFT gridding: grid too large (m^3 must stay below 2^31).");
    if (p.NumProjs > 65535) fail(GENFIRE_ERR_ARG, "FFT gridding: at most 65535 projections.");
    if (p.precision == GENFIRE_PREC_FP64) grid_fft_t<double>(ctx, p, d_proj, angles, d_M, d_rec, npairs);
    else grid_fft_t<float>(ctx, p, d_proj, angles, d_M, d_rec, npairs);
}

}  // namespace gf
