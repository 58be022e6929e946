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

#include <type_traits>

namespace gf {

constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

template <int N> struct P2Plan {
    static constexpr int L = ilog2c(N);
    static constexpr int N8 = L / 3;          // radix-8 stages
    static constexpr int REM = L % 3;         // then one radix-4 (REM 2) or radix-2 (REM 1) stage
    static constexpr int NST = N8 + (REM ? 1 : 0);
    static constexpr int radix(int s) { return s < N8 ? 8 : (REM == 2 ? 4 : 2); }
    static constexpr int ns(int s) { return s == 0 ? 1 : ns(s - 1) * radix(s - 1); }
    // Packed twiddle table (stored right after the n-entry table tw[t] =
    // exp(-2 pi i t / n)): for every stage s with ns(s) > 1 and every kk < ns(s),
    // R = radix(s) entries tw[kk * r * n / (ns(s) * R)] for r = 1 .. R-1 and one
    // pad, so a butterfly's twiddles are R/2 aligned 16-byte loads (float) from
    // one base address.  twoff(s) is the offset of stage s.
    static constexpr int twoff(int s)
    {
        int o = 0;
        for (int t = 0; t < s; ++t) o += ns(t) > 1 ? ns(t) * radix(t) : 0;
        return o;
    }
};

// shared-memory layouts with one padding row every 8 rows (bank spreading).
// idx(i0 + k*S, c) = idx(i0, c) + k * stride(S) whenever S is a multiple of 8,
// or S == 1 with i0 a multiple of 8 and k < 8 -- which covers every exchange
// of the schedules below, so each exchange is one base address plus
// compile-time offsets.
template <int N, int W> struct ColLayout {   // the W columns interleaved, column fastest
    static constexpr int SIZE = (N + N / 8) * W;
    static constexpr int CSTR = 1;               // distance between adjacent columns
    static __device__ __forceinline__ int idx(int i, int c) { return (i + (i >> 3)) * W + c; }
    static constexpr int stride(int S) { return (S % 8 == 0 ? S + S / 8 : S) * W; }
};
template <int N, int W> struct RowLayout {   // each column contiguous
    static constexpr int PC = N + N / 8;
    static constexpr int SIZE = PC * W;
    static constexpr int CSTR = PC;
    static __device__ __forceinline__ int idx(int i, int c) { return c * PC + i + (i >> 3); }
    static constexpr int stride(int S) { return S % 8 == 0 ? S + S / 8 : S; }
};

// w[1 .. R-1] of one butterfly from the packed table
template <typename T, int R>
__device__ __forceinline__ void load_tw(const cplx<T> *__restrict__ p, cplx<T> (&w)[R])
{
    if constexpr (sizeof(T) == 4) {
        const float4 *q = reinterpret_cast<const float4 *>(p);
#pragma unroll
        for (int i = 0; i < R / 2; ++i) {
            const float4 t = __ldg(q + i);
            w[2 * i + 1] = mk(t.x, t.y);
            if (2 * i + 2 < R) w[2 * i + 2] = mk(t.z, t.w);
        }
    } else {
#pragma unroll
        for (int r = 1; r < R; ++r) w[r] = __ldg(p + r - 1);
    }
}

// One stage on the NC columns a thread holds: register k of column c holds
// x[j + k*N/8] of the stage's input.  The twiddles are loaded once and applied
// to every column.
template <typename T, int N, int S, bool INV, int NC>
__device__ __forceinline__ void reg_stage(cplx<T> (&v)[NC][8], int j, const cplx<T> *__restrict__ twp)
{
    constexpr int R = P2Plan<N>::radix(S);
    constexpr int NS = P2Plan<N>::ns(S);
    constexpr int NB = 8 / R;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        cplx<T> w[R];
        if constexpr (NS > 1) {
            const int kk = (j + b * (N / 8)) & (NS - 1);
            load_tw<T, R>(twp + P2Plan<N>::twoff(S) + kk * R, w);
        }
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            cplx<T> u[R];
#pragma unroll
            for (int r = 0; r < R; ++r) u[r] = v[c][b + r * NB];
            if constexpr (NS > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) u[r] = ctw(u[r], w[r], INV);
            }
            Dft<R, T>::run(u, INV, nullptr, N);
#pragma unroll
            for (int r = 0; r < R; ++r) v[c][b + r * NB] = u[r];
        }
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

// register k of the NC consecutive columns at q[c * Lay::CSTR] (one 16-byte
// access for two adjacent float columns of a ColLayout)
template <typename T, class Lay, int NC>
__device__ __forceinline__ void st_cols(cplx<T> *q, const cplx<T> (&v)[NC][8], int k)
{
    if constexpr (NC == 2 && sizeof(T) == 4 && Lay::CSTR == 1) {
        *reinterpret_cast<float4 *>(q) = make_float4(v[0][k].x, v[0][k].y, v[1][k].x, v[1][k].y);
    } else {
#pragma unroll
        for (int c = 0; c < NC; ++c) q[c * Lay::CSTR] = v[c][k];
    }
}
template <typename T, class Lay, int NC>
__device__ __forceinline__ void ld_cols(const cplx<T> *q, cplx<T> (&v)[NC][8], int k)
{
    if constexpr (NC == 2 && sizeof(T) == 4 && Lay::CSTR == 1) {
        const float4 t = *reinterpret_cast<const float4 *>(q);
        v[0][k] = mk(t.x, t.y);
        v[1][k] = mk(t.z, t.w);
    } else {
#pragma unroll
        for (int c = 0; c < NC; ++c) v[c][k] = q[c * Lay::CSTR];
    }
}

template <typename T, int N, class Lay, int S, int NC>
__device__ __forceinline__ void store_stage(cplx<T> *s, const cplx<T> (&v)[NC][8], int j, int c)
{
    constexpr int R = P2Plan<N>::radix(S);
    constexpr int NB = 8 / R;
    constexpr int ST = Lay::stride(P2Plan<N>::ns(S));
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        cplx<T> *q = s + out_base<N, Lay, S>(j, c, b);
#pragma unroll
        for (int r = 0; r < R; ++r) st_cols<T, Lay, NC>(q + r * ST, v, b + r * NB);
    }
}

// next stage's inputs: register k holds x[j + k*N/8]
template <typename T, int N, class Lay, int NC>
__device__ __forceinline__ void load_stage(const cplx<T> *s, cplx<T> (&v)[NC][8], int in_base)
{
    constexpr int ST = Lay::stride(N / 8);
#pragma unroll
    for (int k = 0; k < 8; ++k) ld_cols<T, Lay, NC>(s + in_base + k * ST, v, k);
}

template <typename T, int N, class Lay, bool INV, int NC, int S = 0>
__device__ __forceinline__ void reg_fft(cplx<T> (&v)[NC][8], cplx<T> *sA, cplx<T> *sB, int &buf, int j, int c,
                                        int in_base, const cplx<T> *__restrict__ twp)
{
    reg_stage<T, N, S, INV, NC>(v, j, twp);
    if constexpr (S + 1 < P2Plan<N>::NST) {
        cplx<T> *s = buf ? sB : sA;
        buf ^= 1;
        store_stage<T, N, Lay, S, NC>(s, v, j, c);
        __syncthreads();
        load_stage<T, N, Lay, NC>(s, v, in_base);
        reg_fft<T, N, Lay, INV, NC, S + 1>(v, sA, sB, buf, j, c, in_base, twp);
    }
}

// Accumulator of a thread's errK terms: FP32 for the MIXED passes (a handful
// of terms per thread; the block and grid sums are FP64), FP64 for the FP64
// passes.
template <typename T> using ErrAcc = typename std::conditional<sizeof(T) == 8, double, float>::type;

// Fourier constraint and errK terms on one shared-memory tile (see k_colpass);
// returns this thread's errK terms.
template <typename T, class Lay>
__device__ __forceinline__ ErrAcc<T> apply_table(cplx<T> *s, const ColPassArgs<T> &a, int tile, int W, int other)
{
    using A_ = ErrAcc<T>;
    const int cid0 = other * a.h1 + tile * W;
    const int cid1 = min(cid0 + W, other * a.h1 + a.h1);
    const int e0 = a.tab_off[cid0], e1 = a.tab_off[cid1];
    const int ci = *a.cidx;
    A_ acc = 0;
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const TabEntry<T> t = a.tab[e];
        const int q3 = t.pos & 0xFFFF, cl = t.pos >> 16;
        const int si = Lay::idx(q3, cl);
        const cplx<T> k = s[si];
        const A_ mk_ = (A_)sqrt(k.x * k.x + k.y * k.y);
        if (t.eflags & 1u) acc += fabs(mk_ - (A_)sqrt(t.Mq.x * t.Mq.x + t.Mq.y * t.Mq.y));
        if (t.eflags & 2u) acc += fabs(mk_ - (A_)sqrt(t.Mmq.x * t.Mmq.x + t.Mmq.y * t.Mmq.y));
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
template <typename A_> __device__ __forceinline__ void block_partial(A_ acc, double *out)
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

// Columns per thread of the column pass: two adjacent float columns (16-byte
// global and shared-memory accesses, twiddles and index arithmetic shared by
// both) when the host has checked unit column stride and 16-byte alignment.
template <typename T, int N, int NC> constexpr int col_threads() { return N / 8 * reg_width<T>(N) / NC; }

// global element access for the NC columns of a thread: nv of them exist
template <typename T, int NC>
__device__ __forceinline__ void ld_global(const cplx<T> *p, cplx<T> (&v)[NC][8], int k, int nv)
{
    const cplx<T> zero = mk((T)0, (T)0);
    if constexpr (NC == 2 && sizeof(T) == 4) {
        if (nv == 2) {
            const float4 t = *reinterpret_cast<const float4 *>(p);
            v[0][k] = mk(t.x, t.y);
            v[1][k] = mk(t.z, t.w);
        } else {
            v[0][k] = nv == 1 ? p[0] : zero;
            v[1][k] = zero;
        }
    } else {
#pragma unroll
        for (int c = 0; c < NC; ++c) v[c][k] = c < nv ? p[c] : zero;
    }
}
template <typename T, int NC>
__device__ __forceinline__ void st_global(cplx<T> *p, const cplx<T> (&v)[NC][8], int k, int nv, T scale)
{
    if constexpr (NC == 2 && sizeof(T) == 4) {
        if (nv == 2)
            *reinterpret_cast<float4 *>(p) =
                make_float4(v[0][k].x * scale, v[0][k].y * scale, v[1][k].x * scale, v[1][k].y * scale);
        else if (nv == 1)
            p[0] = mk(v[0][k].x * scale, v[0][k].y * scale);
    } else {
#pragma unroll
        for (int c = 0; c < NC; ++c)
            if (c < nv) p[c] = mk(v[c][k].x * scale, v[c][k].y * scale);
    }
}

// Column pass (same contract as k_colpass) for N a power of two; each thread
// holds NC adjacent columns (NC = 2 requires col_stride 1).
template <typename T, int N, int NC>
__global__ void __launch_bounds__(col_threads<T, N, NC>(), kRegMinBlocks<T>) k_col_reg(ColPassArgs<T> a)
{
    constexpr int W = reg_width<T>(N);
    constexpr int WT = W / NC;  // threads across the tile's columns
    using Lay = ColLayout<N, W>;
    constexpr int NST = P2Plan<N>::NST;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if (a.ctl && blockIdx.x == 0 && blockIdx.y == 0) ctl_mid_update(a.ctl, a.partial, a.nparts, a.denom, a.hist);
    cplx<T> *sA = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T> *sB = sA + Lay::SIZE;
    const cplx<T> *twp = a.tw + N;
    const int c = (threadIdx.x % WT) * NC, j = threadIdx.x / WT;
    const int tile = blockIdx.x, other = blockIdx.y;
    const int col = tile * W + c;
    const int nv = min(max(a.ncols - col, 0), NC);  // columns of this thread that exist
    const int in_base = Lay::idx(j, c);
    cplx<T> v[NC][8];
    {
        const cplx<T> *in = a.in + (long long)other * a.in_other + (long long)col * a.col_stride;
        const unsigned idim = (unsigned)a.in_dim;
        int e = j + a.in_c;
        if (e >= N) e -= N;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            ld_global<T, NC>(in + (unsigned)e * idim, v, k, e < a.in_cnt ? nv : 0);
            e += N / 8;
            if (e >= N) e -= N;
        }
    }
    int buf = 0;
    ErrAcc<T> err = 0;
    if (a.mode & 1) reg_fft<T, N, Lay, false, NC>(v, sA, sB, buf, j, c, in_base, twp);
    if (a.mode & 2) {
        if (a.mode & 1) {
            cplx<T> *s = buf ? sB : sA;
            buf ^= 1;
            store_stage<T, N, Lay, NST - 1, NC>(s, v, j, c);
            __syncthreads();
            if (a.mode & 4) {
                if (a.rtab) {
                    capture_rfree<T>(s, a, tile, W, other, [](int q3, int cl) { return Lay::idx(q3, cl); });
                    __syncthreads();
                }
                err = apply_table<T, Lay>(s, a, tile, W, other);
                block_partial(err, a.partial + (long long)other * gridDim.x + tile);
                __syncthreads();
            }
            load_stage<T, N, Lay, NC>(s, v, in_base);
        }
        reg_fft<T, N, Lay, true, NC>(v, sA, sB, buf, j, c, in_base, twp);
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
                if (e < a.out_cnt) st_global<T, NC>(out + (unsigned)e * odim, v, b + r * NB, nv, a.scale);
                e += NS;
                if (e >= N) e -= N;
            }
        }
    }
}

// Row passes (same contract as k_rows_r2c / k_rows_c2r) for N a power of two.
// The two real rows r0, r0+1 of a box (positivity and support applied) as the
// real and imaginary parts of register k of sequence n1: the element at
// position n1 + NSEQ * (j + k * N / (8 * NSEQ)) of a length-N transform.  All
// loads are issued before any value is used, so they are in flight together.
template <typename T, int N, int NSEQ>
__device__ __forceinline__ void load_row_pair(const RowPassArgs<T> &a, const T *__restrict__ x, int r0, int j,
                                              cplx<T> (&v)[NSEQ][8])
{
    constexpr int TPC = N / (8 * NSEQ);
    const bool ok0 = r0 < a.nrows, ok1 = r0 + 1 < a.nrows;
    const long long o0 = (long long)r0 * a.B1, o1 = o0 + a.B1;
    T xa[NSEQ][8], xb[NSEQ][8];
    uint8_t sa[NSEQ][8], sb[NSEQ][8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
#pragma unroll
        for (int n1 = 0; n1 < NSEQ; ++n1) {
            int e = n1 + NSEQ * (j + k * TPC) + a.c1;
            if (e >= N) e -= N;
            const bool in = e < a.B1;
            xa[n1][k] = (in && ok0) ? x[o0 + e] : (T)0;
            xb[n1][k] = (in && ok1) ? x[o1 + e] : (T)0;
            sa[n1][k] = (a.support && in && ok0) ? a.support[o0 + e] : (uint8_t)1;
            sb[n1][k] = (a.support && in && ok1) ? a.support[o1 + e] : (uint8_t)1;
        }
#pragma unroll
    for (int k = 0; k < 8; ++k)
#pragma unroll
        for (int n1 = 0; n1 < NSEQ; ++n1) {
            T va = xa[n1][k], vb = xb[n1][k];
            if (a.positivity) {
                if (va < (T)0) va = 0;
                if (vb < (T)0) vb = 0;
            }
            v[n1][k] = mk(va * (T)sa[n1][k], vb * (T)sb[n1][k]);
        }
}

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
    if (a.ctl && blockIdx.x == 0 && threadIdx.x == 0) ctl_begin_update(a.ctl, a.changes);
    if (row_pairs_empty(a, W)) {
        zero_half_rows(a, W);
        return;
    }
    const T *x = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int r0 = (blockIdx.x * W + c) * 2, r1 = r0 + 1;
    cplx<T> v[1][8];
    load_row_pair<T, N, 1>(a, x, r0, j, v);
    int buf = 0;
    const int in_base = Lay::idx(j, c);
    reg_fft<T, N, Lay, false, 1>(v, sA, sB, buf, j, c, in_base, a.tw + N);
    cplx<T> *s = buf ? sB : sA;
    store_stage<T, N, Lay, P2Plan<N>::NST - 1, 1>(s, v, j, c);
    __syncthreads();
    // split the pair's spectrum: each thread takes q = j, j + N/8, ... of its own pair
    {
        cplx<T> *ya = a.Y + (long long)r0 * a.ld1, *yb = ya + a.ld1;
        for (int q = j; q < a.h1; q += TPC) {
            const cplx<T> Z = s[Lay::idx(q, c)];
            const cplx<T> Zm = s[Lay::idx(q == 0 ? 0 : N - q, c)];
            const cplx<T> Xa = mk((T)0.5 * (Z.x + Zm.x), (T)0.5 * (Z.y - Zm.y));
            const cplx<T> Xb = mk((T)0.5 * (Z.y + Zm.y), (T)0.5 * (Zm.x - Z.x));
            if (r0 < a.nrows) ya[q] = Xa;
            if (r1 < a.nrows) yb[q] = Xb;
        }
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
    if (row_pairs_empty(a, W)) return;
    T *x = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int r0 = (blockIdx.x * W + c) * 2, r1 = r0 + 1;
    // pack the two half spectra of the pair: each thread takes q = j, j + N/8, ...
    // (h1 <= N/2 + 1); all loads are issued before the packing
    {
        constexpr int QIT = (N / 2 + TPC) / TPC;
        const cplx<T> *ya = a.Y + (long long)r0 * a.ld1, *yb = ya + a.ld1;
        cplx<T> HA[QIT], HB[QIT];
#pragma unroll
        for (int it = 0; it < QIT; ++it) {
            const int q = j + it * TPC;
            HA[it] = (q < a.h1 && r0 < a.nrows) ? ya[q] : mk((T)0, (T)0);
            HB[it] = (q < a.h1 && r1 < a.nrows) ? yb[q] : mk((T)0, (T)0);
        }
#pragma unroll
        for (int it = 0; it < QIT; ++it) {
            const int q = j + it * TPC;
            if (q >= a.h1) break;
            cplx<T> ha = HA[it], hb = HB[it];
            if (q == 0 || 2 * q == N) { ha.y = 0; hb.y = 0; }
            sA[Lay::idx(q, c)] = mk(ha.x - hb.y, ha.y + hb.x);
            if (q != 0 && N - q >= a.h1) sA[Lay::idx(N - q, c)] = mk(ha.x + hb.y, hb.x - ha.y);
        }
    }
    __syncthreads();
    cplx<T> v[1][8];
    const int in_base = Lay::idx(j, c);
    load_stage<T, N, Lay, 1>(sA, v, in_base);
    int buf = 1;
    reg_fft<T, N, Lay, true, 1>(v, sA, sB, buf, j, c, in_base, a.tw + N);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int e = reg_final_index<N>(j, k) + a.c1;
        if (e >= N) e -= N;
        if (e < a.B1) {
            if (r0 < a.nrows) x[(long long)r0 * a.B1 + e] = v[0][k].x * a.scale;
            if (r1 < a.nrows) x[(long long)r1 * a.B1 + e] = v[0][k].y * a.scale;
        }
    }
}

template <typename T, int N> constexpr size_t reg_smem()
{
    return 2 * (size_t)ColLayout<N, reg_width<T>(N)>::SIZE * sizeof(cplx<T>);
}

// Mixed-radix register passes (dr_mix.cu) for n = N1 * N2, N1 in {3, 5}:
// each returns false when n is not covered.
template <typename T> bool mix_capable(int n);
template <typename T> bool launch_col_mix(const ColPassArgs<T> &a, int other, cudaStream_t st);
template <typename T> bool launch_rows_mix(const RowPassArgs<T> &a, bool forward, cudaStream_t st);

// The power-of-two length whose packed table follows the n-entry twiddle
// table: n itself, or N2 of n = N1 * N2 (N1 in {3, 5}, N2 >= 64); 0 if none.
constexpr int packed_length(int n)
{
    if (n >= 8 && !(n & (n - 1))) return n;
    for (int f = 3; f <= 5; f += 2)
        if (n % f == 0) {
            const int m = n / f;
            if (m >= 64 && !(m & (m - 1))) return m;
        }
    return 0;
}

// Size of the packed table appended to the n-entry twiddle table (0 when
// packed_length(n) is 0); the host fills it in the order of P2Plan::twoff
// for the length packed_length(n).
constexpr int packed_twiddle_count(int n)
{
    n = packed_length(n);
    if (!n) return 0;
    int L = 0;
    while ((1 << L) < n) ++L;
    const int n8 = L / 3, rem = L % 3, nst = n8 + (rem ? 1 : 0);
    int o = 0, ns = 1;
    for (int s = 0; s < nst; ++s) {
        const int R = s < n8 ? 8 : (rem == 2 ? 4 : 2);
        if (ns > 1) o += ns * R;
        ns *= R;
    }
    return o;
}

}  // namespace gf
