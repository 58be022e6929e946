// fft_r32.cuh -- 512-point column passes with 32 elements per thread.
//
// A 512-point transform as one radix-32 and one radix-16 stage (512 = 32 x 16)
// with a single shared-memory exchange between them; the radix-8 engine of
// fft_reg.cuh needs two, and its exchanges are what bound those passes.
// Thread t (0..15) of a column holds the elements t + 16 m (m = 0..31) before
// and after a transform:
// The radix-4 and radix-8 butterflies are the packed-pair (f32x2) ones of
// fft.cuh for complex64.
//   stage 1: Y_t[k1] = sum_m x[t + 16 m] W32^(m k1) in registers
//            (m = 8a + b: radix 4 over a, rotation W32^(b k1'), radix 8 over b),
//            then times W512^(t k1) from the twiddle table;
//   exchange: S[k1][t] = Y_t[k1];
//   stage 2: X[k1 + 32 k2] = sum_t S[k1][t] W16^(t k2) for k1 = t and t + 16
//            (radix 4 x 4), which are the elements t + 16 m' again.
// Eight columns per CTA (the constraint table's tile width for n = 512),
// sixteen threads per column, the column fastest within a warp.
#pragma once

#include "fft_reg.cuh"

namespace gf {

constexpr int kR32N = 512;
constexpr int kR32W = 8;                     // columns per CTA
constexpr int kR32Threads = 16 * kR32W;      // 128
constexpr int kR32ColStride = 32 * 17 + 2;   // one column's S[k1][t] block, rows padded to 17:
                                             // every half-warp access is conflict-free
using R32Lay = ColLayout<kR32N, kR32W>;      // natural-order tile for the constraint table
constexpr int kR32Elems = R32Lay::SIZE > kR32W * kR32ColStride ? R32Lay::SIZE : kR32W * kR32ColStride;
template <typename T> constexpr size_t r32_smem() { return (size_t)kR32Elems * sizeof(cplx<T>); }

// W32^j = exp(-2 pi i j / 32) for j known at compile time after unrolling,
// from cos(pi k / 16), k = 0..8, by quadrant symmetry (exact zeros and ones)
template <typename T> __device__ __forceinline__ cplx<T> w32(int j)
{
    constexpr double C[9] = {1.0,
                             0.98078528040323044913,
                             0.92387953251128675613,
                             0.83146961230254523708,
                             0.70710678118654752440,
                             0.55557023301960222474,
                             0.38268343236508977173,
                             0.19509032201612826785,
                             0.0};
    j &= 31;
    const int q = j >> 3, k = j & 7;
    double c, s;  // cos and sin of 2 pi j / 32
    if (q == 0) { c = C[k]; s = C[8 - k]; }
    else if (q == 1) { c = -C[8 - k]; s = C[k]; }
    else if (q == 2) { c = -C[k]; s = -C[8 - k]; }
    else { c = C[8 - k]; s = -C[k]; }
    return mk((T)c, (T)-s);
}

// One 512-point transform of the thread's 32 elements.  In: slot m holds
// element t + 16 m.  Out: slot s holds element t + 16 r32_out_m(s).  Uses
// the CTA's exchange buffer (synchronises before and after writing it).
__device__ __forceinline__ constexpr int r32_out_m(int s)
{
    return (s >> 4) + 2 * (((s & 15) >> 2) + 4 * (s & 3));
}

// Radix 4 of (v0, 0, 0, v3): X[k] = v0 + v3 W4^(3k), the same operations as
// Dft<4> applied to those inputs (v0 + 0 and 0 - v3 are exact).
template <typename T, bool INV> __device__ __forceinline__ void dft4_outer(cplx<T> (&u)[4])
{
    if constexpr (sizeof(T) == 4) {
        // packed pairs: +i v = swap(v) (-1, 1), -i v = swap(v) (1, -1)
        const f32x2_t v0 = pk2(u[0]), v3 = pk2(u[3]), sw = swap2(v3);
        const f32x2_t sp = INV ? pk2(make_float2(1.f, -1.f)) : pk2(make_float2(-1.f, 1.f));
        u[0] = upk2(add2(v0, v3));
        u[2] = upk2(sub2(v0, v3));
        u[1] = upk2(fma2(sw, sp, v0));
        const f32x2_t sn = INV ? pk2(make_float2(-1.f, 1.f)) : pk2(make_float2(1.f, -1.f));
        u[3] = upk2(fma2(sw, sn, v0));
    } else {
        const cplx<T> v0 = u[0], v3 = u[3];
        const cplx<T> r = INV ? mul_mi(v3) : mul_pi(v3);  // W4^3 = +i forward, -i inverse
        u[0] = cadd(v0, v3);
        u[2] = csub(v0, v3);
        u[1] = cadd(v0, r);
        u[3] = csub(v0, r);
    }
}

// ZIN: the elements of slots 8..23 are known to be zero (the centred half of
// a box transform: entries t + 16 m + 128 mod 512 below 256 lie in slots
// 0..7 and 24..31), so the first radix-4 stage takes two inputs.
template <typename T, bool INV, bool ZIN = false>
__device__ __forceinline__ void r32_fft(cplx<T> (&x)[32], cplx<T> *S, int c, int t, const cplx<T> *__restrict__ tw)
{
    // stage 1, radix 4 over a: slot 8a + b -> Z_b[k1'] in slot 8 k1' + b, rotated by W32^(b k1')
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        cplx<T> u[4] = {x[b], x[8 + b], x[16 + b], x[24 + b]};
        if constexpr (ZIN) dft4_outer<T, INV>(u);
        else Dft<4, T>::run(u, INV, nullptr, 4);
#pragma unroll
        for (int k = 0; k < 4; ++k) x[8 * k + b] = (b && k) ? ctw(u[k], w32<T>(b * k), INV) : u[k];
    }
    // radix 8 over b: slots 8 k1' .. 8 k1' + 7 -> Y[k1' + 4 k2] in slot 8 k1' + k2
#pragma unroll
    for (int kp = 0; kp < 4; ++kp) Dft<8, T>::run(&x[8 * kp], INV, nullptr, 8);
    // W512^(t k1) and the exchange: S[k1][t]
    __syncthreads();  // the buffer may still be read by the previous step
    cplx<T> *Sc = S + c * kR32ColStride;
#pragma unroll
    for (int k1 = 0; k1 < 32; ++k1) {
        const int slot = 8 * (k1 & 3) + (k1 >> 2);
        const cplx<T> y = k1 ? ctw(x[slot], __ldg(tw + t * k1), INV) : x[slot];
        Sc[k1 * 17 + t] = y;
    }
    __syncthreads();
    // stage 2 for k1 = t + 16 h: slot 16 h + t' <- S[k1][t']
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int tp = 0; tp < 16; ++tp) x[16 * h + tp] = Sc[(t + 16 * h) * 17 + tp];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        // radix 4 over p of slot 16h + 4p + q -> slot 16h + 4 k2' + q, rotated by W16^(q k2')
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            cplx<T> u[4] = {x[16 * h + q], x[16 * h + 4 + q], x[16 * h + 8 + q], x[16 * h + 12 + q]};
            Dft<4, T>::run(u, INV, nullptr, 4);
#pragma unroll
            for (int k = 0; k < 4; ++k) x[16 * h + 4 * k + q] = (q && k) ? ctw(u[k], w32<T>(2 * q * k), INV) : u[k];
        }
        // radix 4 over q: slots 16h + 4k2' .. +3 -> X[k1 + 32 (k2' + 4 k3)] in slot 16h + 4k2' + k3
#pragma unroll
        for (int kp = 0; kp < 4; ++kp) Dft<4, T>::run(&x[16 * h + 4 * kp], INV, nullptr, 4);
    }
}

// slots of a transform's output (slot s holds element t + 16 r32_out_m(s)) that
// the centred half of a box keeps: r32_out_m(s) in 0..7 or 24..31
__device__ __forceinline__ constexpr bool r32_keep(int s)
{
    return r32_out_m(s) < 8 || r32_out_m(s) >= 24;
}

// For the centred half of a box (count 256 at offset 128), slot m (0..7 or
// 24..31) of thread t is box element t + r32_half_off(m), in 0..255: the
// offsets are compile-time constants once the slot loops are unrolled.
__device__ __forceinline__ constexpr int r32_half_off(int m)
{
    return m < 8 ? 16 * m + 128 : 16 * m - 384;
}

// Column pass (the contract of k_colpass) for n = 512.  ZIN: the input is the
// centred half of a box (in_cnt 256, in_c 128) and the pass starts with a
// forward transform; ZOUT: only the centred half is written (out_cnt 256,
// out_c 128), so the final transform's other outputs are never formed.
// Occupancy: 5 CTAs per SM (<= 96 registers) for the single-transform passes;
// the fused pass keeps 4 (at 96 registers it spills, and measured no faster).
template <typename T, bool ZIN, bool ZOUT>
__global__ void __launch_bounds__(kR32Threads, (ZIN && ZOUT) ? 4 : 5) k_col_r32(ColPassArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *s = reinterpret_cast<cplx<T> *>(smem_raw);
    if (a.ctl && blockIdx.x == 0 && blockIdx.y == 0) ctl_mid_update(a.ctl, a.partial, a.nparts, a.denom, a.hist);
    const int c = threadIdx.x % kR32W, t = threadIdx.x / kR32W;
    const int tile = blockIdx.x, other = blockIdx.y;
    const int col = tile * kR32W + c;
    const bool cv = col < a.ncols;
    const cplx<T> *twp = a.tw;  // tw[j] = exp(-2 pi i j / 512)
    cplx<T> x[32];
    {
        const cplx<T> *in = a.in + (long long)other * a.in_other + (long long)col * a.col_stride;
        const unsigned idim = (unsigned)a.in_dim;
#pragma unroll
        for (int m = 0; m < 32; ++m) {
            if constexpr (ZIN) {
                if (m >= 8 && m < 24) {
                    x[m] = mk((T)0, (T)0);
                    continue;
                }
                x[m] = cv ? in[(unsigned)(t + r32_half_off(m)) * idim] : mk((T)0, (T)0);
                continue;
            }
            int e = t + 16 * m + a.in_c;
            if (e >= kR32N) e -= kR32N;
            x[m] = (cv && e < a.in_cnt) ? in[(unsigned)e * idim] : mk((T)0, (T)0);
        }
    }
    ErrAcc<T> err = 0;
    bool fwd_layout = false;  // slots in the output order of a transform
    if (a.mode & 1) {
        r32_fft<T, false, ZIN>(x, s, c, t, twp);
        fwd_layout = true;
    }
    if (a.mode & 2) {
        if (a.mode & 1) {
            // back to slot m = element t + 16 m, through the natural-order tile
            // (where the Fourier constraint is applied)
            __syncthreads();
#pragma unroll
            for (int sl = 0; sl < 32; ++sl) s[R32Lay::idx(t + 16 * r32_out_m(sl), c)] = x[sl];
            __syncthreads();
            if (a.mode & 4) {
                if (a.rtab) {
                    capture_rfree<T>(s, a, tile, kR32W, other, [](int q3, int cl) { return R32Lay::idx(q3, cl); });
                    __syncthreads();
                }
                err = apply_table<T, R32Lay>(s, a, tile, kR32W, other);
                block_partial(err, a.partial + (long long)other * gridDim.x + tile);
                __syncthreads();
            }
#pragma unroll
            for (int m = 0; m < 32; ++m) x[m] = s[R32Lay::idx(t + 16 * m, c)];
        }
        r32_fft<T, true>(x, s, c, t, twp);
        fwd_layout = true;
    }
    if (!fwd_layout || !cv) return;
    cplx<T> *out = a.out + (long long)other * a.out_other + (long long)col * a.col_stride;
    const unsigned odim = (unsigned)a.out_dim;
#pragma unroll
    for (int sl = 0; sl < 32; ++sl) {
        if constexpr (ZOUT) {
            if (r32_keep(sl))
                out[(unsigned)(t + r32_half_off(r32_out_m(sl))) * odim] = mk(x[sl].x * a.scale, x[sl].y * a.scale);
            continue;
        }
        int e = t + 16 * r32_out_m(sl) + a.out_c;
        if (e >= kR32N) e -= kR32N;
        if (e < a.out_cnt) out[(unsigned)e * odim] = mk(x[sl].x * a.scale, x[sl].y * a.scale);
    }
}

// Row passes (the contracts of k_rows_r2c / k_rows_c2r) for n = 512: eight
// pairs of real rows per CTA, each pair one complex transform (row a the real
// part, row b the imaginary part), sixteen threads per pair with the index
// along the row fastest within a warp (64-byte row segments per access).
using R32RowLay = RowLayout<kR32N, kR32W>;
// elements whose loads are in flight together in the forward row pass: 8 keeps
// the pass at 118 registers (4 CTAs per SM); 16 and 32 cost occupancy and
// measured 13 % and 54 % slower at 512^3
constexpr int kRowLoadGroup = 8;
static_assert(R32RowLay::SIZE <= kR32Elems, "row tile fits the pass's buffer");

// ZIN: the rows are the centred half of the transform (B1 256, c1 128)
template <typename T, bool ZIN>
__global__ void __launch_bounds__(kR32Threads) k_row_r2c_r32(RowPassArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *s = reinterpret_cast<cplx<T> *>(smem_raw);
    const int t = threadIdx.x % 16, c = threadIdx.x / 16;
    if (a.ctl && blockIdx.x == 0 && threadIdx.x == 0) ctl_begin_update(a.ctl, a.changes);
    const T *xs = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int r0 = (blockIdx.x * kR32W + c) * 2, r1 = r0 + 1;
    const bool ok0 = r0 < a.nrows, ok1 = r1 < a.nrows;
    const long long o0 = (long long)r0 * a.B1, o1 = o0 + a.B1;
    cplx<T> x[32];
    // positivity and support (reconstruct.m:126-131) on the way in; the loads
    // of each group of kRowLoadGroup elements are in flight together
#pragma unroll
    for (int m0 = 0; m0 < 32; m0 += kRowLoadGroup) {
        T xa[kRowLoadGroup], xb[kRowLoadGroup];
        uint8_t sa[kRowLoadGroup], sb[kRowLoadGroup];
#pragma unroll
        for (int i = 0; i < kRowLoadGroup; ++i) {
            if constexpr (ZIN) {
                if (m0 + i >= 8 && m0 + i < 24) {
                    xa[i] = xb[i] = (T)0;
                    sa[i] = sb[i] = 1;
                    continue;
                }
                const int e = t + r32_half_off(m0 + i);
                xa[i] = ok0 ? xs[o0 + e] : (T)0;
                xb[i] = ok1 ? xs[o1 + e] : (T)0;
                sa[i] = (a.support && ok0) ? a.support[o0 + e] : (uint8_t)1;
                sb[i] = (a.support && ok1) ? a.support[o1 + e] : (uint8_t)1;
                continue;
            }
            int e = t + 16 * (m0 + i) + a.c1;
            if (e >= kR32N) e -= kR32N;
            const bool in = e < a.B1;
            xa[i] = (in && ok0) ? xs[o0 + e] : (T)0;
            xb[i] = (in && ok1) ? xs[o1 + e] : (T)0;
            sa[i] = (a.support && in && ok0) ? a.support[o0 + e] : (uint8_t)1;
            sb[i] = (a.support && in && ok1) ? a.support[o1 + e] : (uint8_t)1;
        }
#pragma unroll
        for (int i = 0; i < kRowLoadGroup; ++i) {
            T va = xa[i], vb = xb[i];
            if (a.positivity) {
                if (va < (T)0) va = 0;
                if (vb < (T)0) vb = 0;
            }
            x[m0 + i] = mk(va * (T)sa[i], vb * (T)sb[i]);
        }
    }
    r32_fft<T, false, ZIN>(x, s, c, t, a.tw);
    __syncthreads();  // the exchange buffer becomes the natural-order tile
#pragma unroll
    for (int sl = 0; sl < 32; ++sl) s[R32RowLay::idx(t + 16 * r32_out_m(sl), c)] = x[sl];
    __syncthreads();
    // split the pair's spectrum Z into the rows' half spectra:
    // Xa(q) = (Z(q) + conj Z(-q)) / 2, Xb(q) = (Z(q) - conj Z(-q)) / 2i
    cplx<T> *ya = a.Y + (long long)r0 * a.ld1, *yb = ya + a.ld1;
    for (int q = t; q < a.h1; q += 16) {
        const cplx<T> Z = s[R32RowLay::idx(q, c)];
        const cplx<T> Zm = s[R32RowLay::idx(q == 0 ? 0 : kR32N - q, c)];
        if (ok0) ya[q] = mk((T)0.5 * (Z.x + Zm.x), (T)0.5 * (Z.y - Zm.y));
        if (ok1) yb[q] = mk((T)0.5 * (Z.y + Zm.y), (T)0.5 * (Zm.x - Z.x));
    }
}

// ZOUT: only the centred half of each row is written (B1 256, c1 128)
template <typename T, bool ZOUT>
__global__ void __launch_bounds__(kR32Threads) k_row_c2r_r32(RowPassArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *s = reinterpret_cast<cplx<T> *>(smem_raw);
    const int t = threadIdx.x % 16, c = threadIdx.x / 16;
    T *xs = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int r0 = (blockIdx.x * kR32W + c) * 2, r1 = r0 + 1;
    const bool ok0 = r0 < a.nrows, ok1 = r1 < a.nrows;
    {
        // pack the two half spectra: Z = Ha + i Hb on q < h1, Z(-q) from the
        // conjugate symmetry of each row; all loads issued before the packing
        constexpr int QIT = (kR32N / 2 + 16) / 16;  // q = t + 16 it covers 0 .. N/2
        const cplx<T> *ya = a.Y + (long long)r0 * a.ld1, *yb = ya + a.ld1;
        cplx<T> HA[QIT], HB[QIT];
#pragma unroll
        for (int it = 0; it < QIT; ++it) {
            const int q = t + 16 * it;
            HA[it] = (q < a.h1 && ok0) ? ya[q] : mk((T)0, (T)0);
            HB[it] = (q < a.h1 && ok1) ? yb[q] : mk((T)0, (T)0);
        }
#pragma unroll
        for (int it = 0; it < QIT; ++it) {
            const int q = t + 16 * it;
            if (q >= a.h1) break;
            cplx<T> ha = HA[it], hb = HB[it];
            if (q == 0 || 2 * q == kR32N) { ha.y = 0; hb.y = 0; }
            s[R32RowLay::idx(q, c)] = mk(ha.x - hb.y, ha.y + hb.x);
            if (q != 0 && kR32N - q >= a.h1) s[R32RowLay::idx(kR32N - q, c)] = mk(ha.x + hb.y, hb.x - ha.y);
        }
    }
    __syncthreads();
    cplx<T> x[32];
#pragma unroll
    for (int m = 0; m < 32; ++m) x[m] = s[R32RowLay::idx(t + 16 * m, c)];
    r32_fft<T, true>(x, s, c, t, a.tw);  // synchronises before it reuses the buffer
#pragma unroll
    for (int sl = 0; sl < 32; ++sl) {
        if constexpr (ZOUT) {
            if (r32_keep(sl)) {
                const int e = t + r32_half_off(r32_out_m(sl));
                if (ok0) xs[(long long)r0 * a.B1 + e] = x[sl].x * a.scale;
                if (ok1) xs[(long long)r1 * a.B1 + e] = x[sl].y * a.scale;
            }
            continue;
        }
        int e = t + 16 * r32_out_m(sl) + a.c1;
        if (e >= kR32N) e -= kR32N;
        if (e < a.B1) {
            if (ok0) xs[(long long)r0 * a.B1 + e] = x[sl].x * a.scale;
            if (ok1) xs[(long long)r1 * a.B1 + e] = x[sl].y * a.scale;
        }
    }
}

}  // namespace gf
