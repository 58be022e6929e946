// dr_mix.cu -- register-resident FFT passes for lengths N = N1 * N2 with N1 in
// {3, 5} and N2 a power of two (64 .. 512): the grids of oversampling ratios
// like 3 (n = 3 D, the class default) or 2.5, which the power-of-two engine
// of fft_reg.cuh does not cover.
//
// Decimation in time by N1: with n = n1 + N1 n2 and k = k2 + N2 k1,
//   X[k2 + N2 k1] = sum_{n1} W_N1^{n1 k1} W_N^{n1 k2} Y_{n1}[k2],
//   Y_{n1}[k2]    = sum_{n2} x[n1 + N1 n2] W_N2^{n2 k2}.
// Each thread carries its 8 registers of all N1 decimated sequences through
// the N2-point register engine (they are N1 adjacent "virtual columns" of the
// exchange layout, sharing twiddles and index arithmetic).  Afterwards
// register k of every sequence holds the same k2, so the twiddles W_N^{n1 k2}
// and the N1-point DFT are applied in registers and give X[k2 + N2 k1] with no
// further exchange.  The passes keep the contracts (and the tile widths) of
// k_colpass / k_rows_r2c / k_rows_c2r, so they are drop-in launch variants.
#include "fft_reg.cuh"
#include "internal.h"

#include <mutex>
#include <set>

namespace gf {

template <typename T> constexpr int mix_width(int n)  // tile_width<T>(n) as a constant
{
    int W = sizeof(T) == 4 ? 8 : 4;
    while (W > 1 && n * W > 8 * (sizeof(T) == 4 ? 512 : 256)) W /= 2;
    return W;
}
template <typename T, int N2, int N1> constexpr int mix_threads() { return N2 / 8 * mix_width<T>(N1 * N2); }
template <typename T, int N2, int N1> constexpr size_t mix_smem()
{
    return 2 * (size_t)ColLayout<N1 * N2, mix_width<T>(N1 * N2)>::SIZE * sizeof(cplx<T>);
}

// the radix-N1 step: v[n1][k] = Y_{n1}[k2] (k2 = reg_final_index<N2>(j, k))
// becomes v[k1][k] = X[k2 + N2 k1]; tw is the N-entry table
template <typename T, int N2, int N1, bool INV>
__device__ __forceinline__ void mix_final(cplx<T> (&v)[N1][8], int j, const cplx<T> *__restrict__ tw)
{
    constexpr int N = N1 * N2;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int k2 = reg_final_index<N2>(j, k);
        cplx<T> u[N1];
        u[0] = v[0][k];
#pragma unroll
        for (int n1 = 1; n1 < N1; ++n1) u[n1] = ctw(v[n1][k], __ldg(&tw[n1 * k2]), INV);
        Dft<N1, T>::run(u, INV, tw, N);
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) v[k1][k] = u[k1];
    }
}

// Column pass (contract of k_colpass).
template <typename T, int N2, int N1>
__global__ void __launch_bounds__(mix_threads<T, N2, N1>()) k_col_mix(ColPassArgs<T> a)
{
    constexpr int N = N1 * N2;
    constexpr int W = mix_width<T>(N);
    using Lay = ColLayout<N2, W * N1>;
    using Full = ColLayout<N, W>;
    static_assert(Lay::SIZE == Full::SIZE, "exchange and full layouts share the buffers");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if (a.ctl && blockIdx.x == 0 && blockIdx.y == 0) ctl_mid_update(a.ctl, a.partial, a.nparts, a.denom, a.hist);
    cplx<T> *sA = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *sB = sA + Lay::SIZE;
    const cplx<T> *tw = a.tw, *twp = a.tw + N;
    const int c = threadIdx.x % W, j = threadIdx.x / W;
    const int vc = c * N1;
    const int tile = blockIdx.x, other = blockIdx.y;
    const int col = tile * W + c;
    const bool valid = col < a.ncols;
    const cplx<T> zero = mk((T)0, (T)0);
    const int in_base = Lay::idx(j, vc);
    cplx<T> v[N1][8];
    {
        const cplx<T> *in = a.in + (long long)other * a.in_other + (long long)col * a.col_stride;
        const unsigned idim = (unsigned)a.in_dim;
#pragma unroll
        for (int k = 0; k < 8; ++k)
#pragma unroll
            for (int n1 = 0; n1 < N1; ++n1) {
                int e = n1 + N1 * (j + k * (N2 / 8)) + a.in_c;
                if (e >= N) e -= N;
                v[n1][k] = (valid && e < a.in_cnt) ? in[(unsigned)e * idim] : zero;
            }
    }
    int buf = 0;
    ErrAcc<T> err = 0;
    if (a.mode & 1) {
        reg_fft<T, N2, Lay, false, N1>(v, sA, sB, buf, j, vc, in_base, twp);
        mix_final<T, N2, N1, false>(v, j, tw);
    }
    if (a.mode & 2) {
        if (a.mode & 1) {
            cplx<T> *s = buf ? sB : sA;
            buf ^= 1;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int k2 = reg_final_index<N2>(j, k);
#pragma unroll
                for (int k1 = 0; k1 < N1; ++k1) s[Full::idx(k2 + N2 * k1, c)] = v[k1][k];
            }
            __syncthreads();
            if (a.mode & 4) {
                if (a.rtab) {
                    capture_rfree<T>(s, a, tile, W, other, [](int q3, int cl) { return Full::idx(q3, cl); });
                    __syncthreads();
                }
                err = apply_table<T, Full>(s, a, tile, W, other);
                block_partial(err, a.partial + (long long)other * gridDim.x + tile);
                __syncthreads();
            }
#pragma unroll
            for (int k = 0; k < 8; ++k)
#pragma unroll
                for (int n1 = 0; n1 < N1; ++n1) v[n1][k] = s[Full::idx(n1 + N1 * (j + k * (N2 / 8)), c)];
        }
        reg_fft<T, N2, Lay, true, N1>(v, sA, sB, buf, j, vc, in_base, twp);
        mix_final<T, N2, N1, true>(v, j, tw);
    }
    cplx<T> *out = a.out + (long long)other * a.out_other + (long long)col * a.col_stride;
    const unsigned odim = (unsigned)a.out_dim;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int k2 = reg_final_index<N2>(j, k);
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) {
            int e = k2 + N2 * k1 + a.out_c;
            if (e >= N) e -= N;
            if (valid && e < a.out_cnt) {
                const cplx<T> x = v[k1][k];
                out[(unsigned)e * odim] = mk(x.x * a.scale, x.y * a.scale);
            }
        }
    }
}

// Row passes (contracts of k_rows_r2c / k_rows_c2r): two real rows per
// complex transform.
template <typename T, int N2, int N1>
__global__ void __launch_bounds__(mix_threads<T, N2, N1>()) k_row_r2c_mix(RowPassArgs<T> a)
{
    constexpr int N = N1 * N2;
    constexpr int W = mix_width<T>(N);
    constexpr int TPC = N2 / 8;
    using Lay = RowLayout<N2, W * N1>;
    using Full = RowLayout<N, W>;
    static_assert(Lay::SIZE == Full::SIZE, "exchange and full layouts share the buffers");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *sA = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *sB = sA + Lay::SIZE;
    const int c = threadIdx.x / TPC, j = threadIdx.x % TPC;
    const int vc = c * N1;
    if (a.ctl && blockIdx.x == 0 && threadIdx.x == 0) ctl_begin_update(a.ctl, a.changes);
    if (row_pairs_empty(a, W)) {
        zero_half_rows(a, W);
        return;
    }
    const T *x = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int r0 = (blockIdx.x * W + c) * 2, r1 = r0 + 1;
    cplx<T> v[N1][8];
    load_row_pair<T, N, N1>(a, x, r0, j, v);
    int buf = 0;
    const int in_base = Lay::idx(j, vc);
    reg_fft<T, N2, Lay, false, N1>(v, sA, sB, buf, j, vc, in_base, a.tw + N);
    mix_final<T, N2, N1, false>(v, j, a.tw);
    cplx<T> *s = buf ? sB : sA;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int k2 = reg_final_index<N2>(j, k);
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) s[Full::idx(k2 + N2 * k1, c)] = v[k1][k];
    }
    __syncthreads();
    // split the pair's spectrum: each thread takes q = j, j + N2/8, ... of its own pair
    cplx<T> *ya = a.Y + (long long)r0 * a.ld1, *yb = ya + a.ld1;
    for (int q = j; q < a.h1; q += TPC) {
        const cplx<T> Z = s[Full::idx(q, c)];
        const cplx<T> Zm = s[Full::idx(q == 0 ? 0 : N - q, c)];
        const cplx<T> Xa = mk((T)0.5 * (Z.x + Zm.x), (T)0.5 * (Z.y - Zm.y));
        const cplx<T> Xb = mk((T)0.5 * (Z.y + Zm.y), (T)0.5 * (Zm.x - Z.x));
        if (r0 < a.nrows) ya[q] = Xa;
        if (r1 < a.nrows) yb[q] = Xb;
    }
}

template <typename T, int N2, int N1>
__global__ void __launch_bounds__(mix_threads<T, N2, N1>()) k_row_c2r_mix(RowPassArgs<T> a)
{
    constexpr int N = N1 * N2;
    constexpr int W = mix_width<T>(N);
    constexpr int TPC = N2 / 8;
    using Lay = RowLayout<N2, W * N1>;
    using Full = RowLayout<N, W>;
    static_assert(Lay::SIZE == Full::SIZE, "exchange and full layouts share the buffers");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *sA = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *sB = sA + Lay::SIZE;
    const int c = threadIdx.x / TPC, j = threadIdx.x % TPC;
    const int vc = c * N1;
    if (row_pairs_empty(a, W)) return;
    T *x = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int r0 = (blockIdx.x * W + c) * 2, r1 = r0 + 1;
    // pack the two half spectra of the pair: each thread takes q = j, j + N2/8, ...
    {
        const cplx<T> *ya = a.Y + (long long)r0 * a.ld1, *yb = ya + a.ld1;
        for (int q = j; q < a.h1; q += TPC) {
            cplx<T> ha = mk((T)0, (T)0), hb = ha;
            if (r0 < a.nrows) ha = ya[q];
            if (r1 < a.nrows) hb = yb[q];
            if (q == 0 || 2 * q == N) { ha.y = 0; hb.y = 0; }
            sA[Full::idx(q, c)] = mk(ha.x - hb.y, ha.y + hb.x);
            if (q != 0 && N - q >= a.h1) sA[Full::idx(N - q, c)] = mk(ha.x + hb.y, hb.x - ha.y);
        }
    }
    __syncthreads();
    cplx<T> v[N1][8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) v[n1][k] = sA[Full::idx(n1 + N1 * (j + k * TPC), c)];
    const int in_base = Lay::idx(j, vc);
    int buf = 1;  // sA holds the packed input: the first exchange goes to sB
    reg_fft<T, N2, Lay, true, N1>(v, sA, sB, buf, j, vc, in_base, a.tw + N);
    mix_final<T, N2, N1, true>(v, j, a.tw);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int k2 = reg_final_index<N2>(j, k);
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) {
            int e = k2 + N2 * k1 + a.c1;
            if (e >= N) e -= N;
            if (e < a.B1) {
                if (r0 < a.nrows) x[(long long)r0 * a.B1 + e] = v[k1][k].x * a.scale;
                if (r1 < a.nrows) x[(long long)r1 * a.B1 + e] = v[k1][k].y * a.scale;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// dispatch
// ---------------------------------------------------------------------------
template <typename T, int N2, int N1> static void mix_attrs()
{
    const int sm = (int)mix_smem<T, N2, N1>();
    GF_CUDA(cudaFuncSetAttribute((const void *)k_col_mix<T, N2, N1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    GF_CUDA(cudaFuncSetAttribute((const void *)k_row_r2c_mix<T, N2, N1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    GF_CUDA(cudaFuncSetAttribute((const void *)k_row_c2r_mix<T, N2, N1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
}

template <typename T> static void ensure_mix_attrs()
{
    static std::mutex mu;
    static std::set<int> done;
    int dev = 0;
    GF_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (done.count(dev)) return;
    mix_attrs<T, 64, 3>(); mix_attrs<T, 128, 3>(); mix_attrs<T, 256, 3>();
    if constexpr (sizeof(T) == 4) {
        mix_attrs<T, 512, 3>();
        mix_attrs<T, 64, 5>(); mix_attrs<T, 128, 5>(); mix_attrs<T, 256, 5>();
    }
    done.insert(dev);
}

// which (N2, N1) covers n; 0 when none
template <typename T> static int mix_split(int n, int &N1)
{
    const int n1s[2] = {3, 5};
    for (int f : n1s) {
        if (sizeof(T) == 8 && f != 3) continue;
        if (n % f) continue;
        const int m = n / f;
        const int maxN2 = (sizeof(T) == 8 || f == 5) ? 256 : 512;
        if (m >= 64 && m <= maxN2 && (m & (m - 1)) == 0) {
            N1 = f;
            return m;
        }
    }
    return 0;
}

template <typename T> bool mix_capable(int n)
{
    int N1 = 0;
    return mix_split<T>(n, N1) != 0;
}
template bool mix_capable<float>(int);
template bool mix_capable<double>(int);

#define GF_MIX_CASES(F)                                                                         \
    if (N1 == 3 && N2 == 64) { F(64, 3); return true; }                                           \
    if (N1 == 3 && N2 == 128) { F(128, 3); return true; }                                         \
    if (N1 == 3 && N2 == 256) { F(256, 3); return true; }                                         \
    if constexpr (sizeof(T) == 4) {                                                                \
        if (N1 == 3 && N2 == 512) { F(512, 3); return true; }                                     \
        if (N1 == 5 && N2 == 64) { F(64, 5); return true; }                                       \
        if (N1 == 5 && N2 == 128) { F(128, 5); return true; }                                     \
        if (N1 == 5 && N2 == 256) { F(256, 5); return true; }                                     \
    }

template <typename T> bool launch_col_mix(const ColPassArgs<T> &a, int other, cudaStream_t st)
{
    int N1 = 0;
    const int N2 = mix_split<T>(a.pl.n, N1);
    if (!N2) return false;
    if (a.W != mix_width<T>(a.pl.n)) fail(GENFIRE_ERR_STATE, "internal: mixed-radix tile width mismatch.");
    ensure_mix_attrs<T>();
    const dim3 grid(cdiv(a.ncols, a.W), other);
#define GF_COL(n2, n1) k_col_mix<T, n2, n1><<<grid, mix_threads<T, n2, n1>(), mix_smem<T, n2, n1>(), st>>>(a)
    GF_MIX_CASES(GF_COL)
#undef GF_COL
    return false;
}

template <typename T> bool launch_rows_mix(const RowPassArgs<T> &a, bool forward, cudaStream_t st)
{
    int N1 = 0;
    const int N2 = mix_split<T>(a.pl.n, N1);
    if (!N2) return false;
    if (a.W != mix_width<T>(a.pl.n)) fail(GENFIRE_ERR_STATE, "internal: mixed-radix tile width mismatch.");
    ensure_mix_attrs<T>();
    const dim3 grid(cdiv((a.nrows + 1) / 2, a.W));
#define GF_ROW(n2, n1)                                                                                    \
    do {                                                                                                  \
        if (forward) k_row_r2c_mix<T, n2, n1><<<grid, mix_threads<T, n2, n1>(), mix_smem<T, n2, n1>(), st>>>(a); \
        else k_row_c2r_mix<T, n2, n1><<<grid, mix_threads<T, n2, n1>(), mix_smem<T, n2, n1>(), st>>>(a);  \
    } while (0)
    GF_MIX_CASES(GF_ROW)
#undef GF_ROW
    return false;
}
#undef GF_MIX_CASES

template bool launch_col_mix<float>(const ColPassArgs<float> &, int, cudaStream_t);
template bool launch_col_mix<double>(const ColPassArgs<double> &, int, cudaStream_t);
template bool launch_rows_mix<float>(const RowPassArgs<float> &, bool, cudaStream_t);
template bool launch_rows_mix<double>(const RowPassArgs<double> &, bool, cudaStream_t);

}  // namespace gf
