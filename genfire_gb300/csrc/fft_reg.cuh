// fft_reg.cuh -- register-resident Stockham FFT for power-of-two lengths.
//
// Each thread owns 8 elements of one column: before every stage it holds
// x[j + k*N/8] (k = 0..7) of the stage's input.  A stage of radix R runs 8/R
// butterflies in registers; between stages the outputs are exchanged through
// one of two shared-memory buffers (ping-pong, one barrier per exchange).  A
// 512-point transform is three radix-8 stages and two exchanges; the first
// stage reads straight from global memory and the last stage's outputs go
// straight back, so zero-padded inputs and cropped outputs cost nothing.
// Radix schedule and twiddle strides are compile-time constants.
#pragma once

#include "fft.cuh"

namespace gf {

constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

template <int N> struct P2Plan {
    static constexpr int L = ilog2c(N);
    static constexpr int N8 = L / 3;          // radix-8 stages
    static constexpr int REM = L % 3;         // then one radix-4 (REM 2) or radix-2 (REM 1) stage
    static constexpr int NST = N8 + (REM ? 1 : 0);
    static constexpr int radix(int s) { return s < N8 ? 8 : (REM == 2 ? 4 : 2); }
    static constexpr int ns(int s) { return s == 0 ? 1 : ns(s - 1) * radix(s - 1); }
};

// shared-memory layouts with one padding row every 8 rows (bank spreading).
// idx(i0 + k*S, c) = idx(i0, c) + k * stride(S) whenever S is a multiple of 8,
// or S == 1 with i0 a multiple of 8 and k < 8 -- which covers every exchange
// of the schedules below, so each exchange is one base address plus
// compile-time offsets.
template <int N, int W> struct ColLayout {   // the W columns interleaved, column fastest
    static constexpr int SIZE = (N + N / 8) * W;
    static __device__ __forceinline__ int idx(int i, int c) { return (i + (i >> 3)) * W + c; }
    static constexpr int stride(int S) { return (S % 8 == 0 ? S + S / 8 : S) * W; }
};
template <int N, int W> struct RowLayout {   // each column contiguous
    static constexpr int PC = N + N / 8;
    static constexpr int SIZE = PC * W;
    static __device__ __forceinline__ int idx(int i, int c) { return c * PC + i + (i >> 3); }
    static constexpr int stride(int S) { return S % 8 == 0 ? S + S / 8 : S; }
};

template <typename T, int N, int S>
__device__ __forceinline__ void reg_stage(cplx<T> (&v)[8], int j, const cplx<T> *__restrict__ tw, bool inv)
{
    constexpr int R = P2Plan<N>::radix(S);
    constexpr int NS = P2Plan<N>::ns(S);
    constexpr int NB = 8 / R;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int jp = j + b * (N / 8);
        cplx<T> u[R];
#pragma unroll
        for (int r = 0; r < R; ++r) u[r] = v[b + r * NB];
        if (NS > 1) {
            const int kk = jp & (NS - 1);
            constexpr int step = N / (NS * R);
#pragma unroll
            for (int r = 1; r < R; ++r) u[r] = ctw(u[r], __ldg(&tw[kk * r * step]), inv);
        }
        Dft<R, T>::run(u, inv, tw, N);
#pragma unroll
        for (int r = 0; r < R; ++r) v[b + r * NB] = u[r];
    }
}

// FFT index held by register k after stage S
template <int N, int S> __device__ __forceinline__ int reg_out_index(int j, int k)
{
    constexpr int R = P2Plan<N>::radix(S);
    constexpr int NS = P2Plan<N>::ns(S);
    constexpr int NB = 8 / R;
    const int b = k % NB, r = k / NB;
    const int jp = j + b * (N / 8);
    const int kk = jp & (NS - 1);
    return (jp - kk) * R + kk + r * NS;
}
template <int N> __device__ __forceinline__ int reg_final_index(int j, int k)
{
    return reg_out_index<N, P2Plan<N>::NST - 1>(j, k);
}

// Shared-memory positions of the registers after stage S: register
// k = b + r*NB sits at out_base<S>(j, c, b) + r * Lay::stride(NS).
template <int N, class Lay, int S> __device__ __forceinline__ int out_base(int j, int c, int b)
{
    constexpr int R = P2Plan<N>::radix(S);
    constexpr int NS = P2Plan<N>::ns(S);
    const int jp = j + b * (N / 8);
    const int kk = jp & (NS - 1);
    return Lay::idx((jp - kk) * R + kk, c);
}

template <typename T, int N, class Lay, int S>
__device__ __forceinline__ void store_stage(cplx<T> *s, const cplx<T> (&v)[8], int j, int c)
{
    constexpr int R = P2Plan<N>::radix(S);
    constexpr int NB = 8 / R;
    constexpr int ST = Lay::stride(P2Plan<N>::ns(S));
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        cplx<T> *q = s + out_base<N, Lay, S>(j, c, b);
#pragma unroll
        for (int r = 0; r < R; ++r) q[r * ST] = v[b + r * NB];
    }
}

// next stage's inputs: register k holds x[j + k*N/8]
template <typename T, int N, class Lay>
__device__ __forceinline__ void load_stage(const cplx<T> *s, cplx<T> (&v)[8], int in_base)
{
    constexpr int ST = Lay::stride(N / 8);
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = s[in_base + k * ST];
}

template <typename T, int N, class Lay, int S = 0>
__device__ __forceinline__ void reg_fft(cplx<T> (&v)[8], cplx<T> *sA, cplx<T> *sB, int &buf, int j, int c,
                                        int in_base, const cplx<T> *__restrict__ tw, bool inv)
{
    reg_stage<T, N, S>(v, j, tw, inv);
    if constexpr (S + 1 < P2Plan<N>::NST) {
        cplx<T> *s = buf ? sB : sA;
        buf ^= 1;
        store_stage<T, N, Lay, S>(s, v, j, c);
        __syncthreads();
        load_stage<T, N, Lay>(s, v, in_base);
        reg_fft<T, N, Lay, S + 1>(v, sA, sB, buf, j, c, in_base, tw, inv);
    }
}

// Fourier constraint and errK terms on one shared-memory tile (see k_colpass);
// returns this thread's errK terms (a handful per thread, summed in FP32; the
// block and grid sums are FP64).
template <typename T, class Lay>
__device__ __forceinline__ float apply_table(cplx<T> *s, const ColPassArgs<T> &a, int tile, int W, int other)
{
    const int cid0 = other * a.h1 + tile * W;
    const int cid1 = min(cid0 + W, other * a.h1 + a.h1);
    const int e0 = a.tab_off[cid0], e1 = a.tab_off[cid1];
    const int ci = *a.cidx;
    float acc = 0.f;
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const TabEntry<T> t = a.tab[e];
        const int q3 = t.pos & 0xFFFF, cl = t.pos >> 16;
        const int si = Lay::idx(q3, cl);
        const cplx<T> k = s[si];
        const float mk_ = (float)sqrt(k.x * k.x + k.y * k.y);
        if (t.eflags & 1u) acc += fabsf(mk_ - (float)sqrt(t.Mq.x * t.Mq.x + t.Mq.y * t.Mq.y));
        if (t.eflags & 2u) acc += fabsf(mk_ - (float)sqrt(t.Mmq.x * t.Mmq.x + t.Mmq.y * t.Mmq.y));
        const bool eq = (t.cq >> ci) & 1u, emq = (t.cmq >> ci) & 1u;
        if (eq || emq) {
            const cplx<T> A = eq ? t.Mq : k;
            const cplx<T> B = emq ? cconj(t.Mmq) : k;
            s[si] = mk((T)0.5 * (A.x + B.x), (T)0.5 * (A.y + B.y));
        }
    }
    return acc;
}

// CTA sum of the per-thread errK terms: warp sums in FP32 (a few terms per
// thread), the per-warp partials in FP64.  FP64 arithmetic is kept to one warp
// because its throughput on this part is a small fraction of FP32's.
__device__ __forceinline__ void block_partial(float acc, double *out)
{
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (double)acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        const int nw = (blockDim.x + 31) / 32;
        for (int w = 0; w < nw; ++w) v += red[w];
        *out = v;
    }
}

// CTAs per SM the register-resident kernels are built for (registers per
// thread <= 65536 / (threads * this)); shared memory (2 x 37 KB) allows 3.
template <typename T> constexpr int kRegMinBlocks = sizeof(T) == 4 ? 3 : 2;

template <typename T> constexpr int reg_width(int n)
{
    return sizeof(T) == 4 ? (n * 8 > 4096 ? 4096 / n : 8) : (n * 4 > 2048 ? 2048 / n : 4);
}

// Column pass (same contract as k_colpass) for N a power of two.
template <typename T, int N>
__global__ void __launch_bounds__(N / 8 * reg_width<T>(N), kRegMinBlocks<T>) k_col_reg(ColPassArgs<T> a)
{
    constexpr int W = reg_width<T>(N);
    using Lay = ColLayout<N, W>;
    constexpr int NST = P2Plan<N>::NST;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *sA = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *sB = sA + Lay::SIZE;
    const int c = threadIdx.x % W, j = threadIdx.x / W;
    const int tile = blockIdx.x, other = blockIdx.y;
    const int col = tile * W + c;
    const bool valid = col < a.ncols;
    const cplx<T> zero = mk((T)0, (T)0);
    const int in_base = Lay::idx(j, c);
    cplx<T> v[8];
    {
        const cplx<T> *in = a.in + (long long)other * a.in_other + (long long)col * a.col_stride;
        const unsigned idim = (unsigned)a.in_dim;
        int e = j + a.in_c;
        if (e >= N) e -= N;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            v[k] = (valid && e < a.in_cnt) ? in[(unsigned)e * idim] : zero;
            e += N / 8;
            if (e >= N) e -= N;
        }
    }
    int buf = 0;
    float err = 0.f;
    if (a.mode & 1) reg_fft<T, N, Lay>(v, sA, sB, buf, j, c, in_base, a.tw, false);
    if (a.mode & 2) {
        if (a.mode & 1) {
            cplx<T> *s = buf ? sB : sA;
            buf ^= 1;
            store_stage<T, N, Lay, NST - 1>(s, v, j, c);
            __syncthreads();
            if (a.mode & 4) {
                err = apply_table<T, Lay>(s, a, tile, W, other);
                __syncthreads();
            }
            load_stage<T, N, Lay>(s, v, in_base);
        }
        reg_fft<T, N, Lay>(v, sA, sB, buf, j, c, in_base, a.tw, true);
    }
    cplx<T> *out = a.out + (long long)other * a.out_other + (long long)col * a.col_stride;
    const unsigned odim = (unsigned)a.out_dim;
    {
        constexpr int R = P2Plan<N>::radix(NST - 1);
        constexpr int NB = 8 / R;
        constexpr int NS = P2Plan<N>::ns(NST - 1);
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            const int jp = j + b * (N / 8);
            const int kk = jp & (NS - 1);
            int e = (jp - kk) * R + kk + a.out_c;
            if (e >= N) e -= N;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (valid && e < a.out_cnt) {
                    const cplx<T> x = v[b + r * NB];
                    out[(unsigned)e * odim] = mk(x.x * a.scale, x.y * a.scale);
                }
                e += NS;
                if (e >= N) e -= N;
            }
        }
    }
    if (a.mode & 4) block_partial(err, a.partial + (long long)other * gridDim.x + tile);
}

// Row passes (same contract as k_rows_r2c / k_rows_c2r) for N a power of two.
template <typename T, int N>
__global__ void __launch_bounds__(N / 8 * reg_width<T>(N), kRegMinBlocks<T>) k_row_r2c_reg(RowPassArgs<T> a)
{
    constexpr int W = reg_width<T>(N);
    constexpr int TPC = N / 8;
    using Lay = RowLayout<N, W>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *sA = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *sB = sA + Lay::SIZE;
    const int c = threadIdx.x / TPC, j = threadIdx.x % TPC;
    const T *x = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int r0 = (blockIdx.x * W + c) * 2, r1 = r0 + 1;
    cplx<T> v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int e = j + k * TPC + a.c1;
        if (e >= N) e -= N;
        T va = 0, vb = 0;
        if (e < a.B1) {
            if (r0 < a.nrows) {
                const long long o = (long long)r0 * a.B1 + e;
                va = x[o];
                if (a.positivity && va < (T)0) va = 0;
                if (a.support) va = va * (T)a.support[o];
            }
            if (r1 < a.nrows) {
                const long long o = (long long)r1 * a.B1 + e;
                vb = x[o];
                if (a.positivity && vb < (T)0) vb = 0;
                if (a.support) vb = vb * (T)a.support[o];
            }
        }
        v[k] = mk(va, vb);
    }
    int buf = 0;
    const int in_base = Lay::idx(j, c);
    reg_fft<T, N, Lay>(v, sA, sB, buf, j, c, in_base, a.tw, false);
    cplx<T> *s = buf ? sB : sA;
    store_stage<T, N, Lay, P2Plan<N>::NST - 1>(s, v, j, c);
    __syncthreads();
    const int rbase = blockIdx.x * W * 2;
    for (int idx = threadIdx.x; idx < W * a.h1; idx += blockDim.x) {
        const int cc = idx / a.h1, q = idx - cc * a.h1;
        const int q0 = rbase + 2 * cc, q1 = q0 + 1;
        const cplx<T> Z = s[Lay::idx(q, cc)];
        const cplx<T> Zm = s[Lay::idx(q == 0 ? 0 : N - q, cc)];
        const cplx<T> Xa = mk((T)0.5 * (Z.x + Zm.x), (T)0.5 * (Z.y - Zm.y));
        const cplx<T> Xb = mk((T)0.5 * (Z.y + Zm.y), (T)0.5 * (Zm.x - Z.x));
        if (q0 < a.nrows) a.Y[(long long)q0 * a.ld1 + q] = Xa;
        if (q1 < a.nrows) a.Y[(long long)q1 * a.ld1 + q] = Xb;
    }
}

template <typename T, int N>
__global__ void __launch_bounds__(N / 8 * reg_width<T>(N), kRegMinBlocks<T>) k_row_c2r_reg(RowPassArgs<T> a)
{
    constexpr int W = reg_width<T>(N);
    constexpr int TPC = N / 8;
    using Lay = RowLayout<N, W>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *sA = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *sB = sA + Lay::SIZE;
    const int c = threadIdx.x / TPC, j = threadIdx.x % TPC;
    T *x = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int rbase = blockIdx.x * W * 2;
    for (int idx = threadIdx.x; idx < W * a.h1; idx += blockDim.x) {
        const int cc = idx / a.h1, q = idx - cc * a.h1;
        const int q0 = rbase + 2 * cc, q1 = q0 + 1;
        cplx<T> ha = mk((T)0, (T)0), hb = ha;
        if (q0 < a.nrows) ha = a.Y[(long long)q0 * a.ld1 + q];
        if (q1 < a.nrows) hb = a.Y[(long long)q1 * a.ld1 + q];
        if (q == 0 || 2 * q == N) { ha.y = 0; hb.y = 0; }
        sA[Lay::idx(q, cc)] = mk(ha.x - hb.y, ha.y + hb.x);
        if (q != 0 && N - q >= a.h1) sA[Lay::idx(N - q, cc)] = mk(ha.x + hb.y, hb.x - ha.y);
    }
    __syncthreads();
    cplx<T> v[8];
    const int in_base = Lay::idx(j, c);
    load_stage<T, N, Lay>(sA, v, in_base);
    int buf = 1;
    reg_fft<T, N, Lay>(v, sA, sB, buf, j, c, in_base, a.tw, true);
    const int r0 = (blockIdx.x * W + c) * 2, r1 = r0 + 1;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int e = reg_final_index<N>(j, k) + a.c1;
        if (e >= N) e -= N;
        if (e < a.B1) {
            if (r0 < a.nrows) x[(long long)r0 * a.B1 + e] = v[k].x * a.scale;
            if (r1 < a.nrows) x[(long long)r1 * a.B1 + e] = v[k].y * a.scale;
        }
    }
}

template <typename T, int N> constexpr size_t reg_smem()
{
    return 2 * (size_t)ColLayout<N, reg_width<T>(N)>::SIZE * sizeof(cplx<T>);
}

}  // namespace gf
