// fft_r32.cuh -- 128- to 1024-point passes with 32 elements per thread.
//
// An N-point transform (N = 32 * P, P = 4 .. 32 threads per column) as one
// radix-32 stage and one radix-P stage with a single shared-memory exchange
// between them; the radix-8 engine of fft_reg.cuh needs two (three at 1024),
// and its exchanges are what bound those passes.  Thread t (0..P-1) of a
// column holds the elements t + P m (m = 0..31) before and after a transform:
//   stage 1: Y_t[k1] = sum_m x[t + P m] W32^(m k1) in registers
//            (m = 8a + b: radix 4 over a, rotation W32^(b k1'), radix 8 over b),
//            then times WN^(t k1) (four table entries and multiply chains);
//   exchange: S[k1][t] = Y_t[k1];
//   stage 2: X[k1 + 32 k2] = sum_t S[k1][t] WP^(t k2) for k1 = t + P h,
//            h < 32 / P: the 4- or 8-point DFTs (N = 128, 256), the two
//            16-point DFTs (radix 4 x 4, N = 512), or the 32-point DFT (the
//            stage-1 schedule again, N = 1024); either way the thread ends
//            with the elements t + P m' again.
// The radix-4 and radix-8 butterflies are the packed-pair (f32x2) ones of
// fft.cuh for complex64.  A CTA holds W columns of P threads -- W the
// constraint table's tile width, 8 up to 512 points and 4 at 1024 -- with
// the column fastest within a warp: 32, 64 or 128 threads.
#pragma once

#include "fft_reg.cuh"

#include <cuda.h>  // CUtensorMap (the type only; the map is encoded by the host)

namespace gf {

template <int N> struct R32 {
    static_assert(N == 128 || N == 256 || N == 512 || N == 1024, "radix-32 engines: 128 to 1024 points");
    static constexpr int P = N / 32;                 // threads per column
    static constexpr int W = N <= 512 ? 8 : 4;       // columns per CTA
    static constexpr int THREADS = P * W;
    static constexpr int ROW = P + 1;                // S[k1][t] row stride (odd: conflict-free reads)
    // column stride of the exchange buffer, 16 / W modulo 16: the W columns x
    // 16 / W threads of a half-warp hit 16 distinct 8-byte bank pairs
    static constexpr int CS = 32 * ROW + 16 / W;
    using Lay = ColLayout<N, W>;                     // natural-order tile for the constraint table
    using RowLay = RowLayout<N, W>;                  // natural-order tile of the row passes
    static constexpr int ELEMS_ = Lay::SIZE > W * CS ? Lay::SIZE : W * CS;
    static constexpr int ELEMS = RowLay::SIZE > ELEMS_ ? RowLay::SIZE : ELEMS_;
    template <typename T> static constexpr size_t smem() { return (size_t)ELEMS * sizeof(cplx<T>); }
    // the twiddle buffer of length N holds, after its N entries and the packed
    // per-stage table, WN^(t k1) at TWT + k1 P + t: the P threads of a column
    // read consecutive entries (one or two sectors per warp request; the
    // table in its natural order, at t k1, spreads a request over 4-8)
    static constexpr int TWT = N + packed_twiddle_count(N);

    // Out: slot s holds element t + P out_m(s)
    static __device__ __forceinline__ constexpr int out_m(int s)
    {
        if constexpr (N == 128) return (s >> 2) + 8 * (s & 3);
        else if constexpr (N == 256) return (s >> 3) + 4 * (s & 7);
        else if constexpr (N == 512) return (s >> 4) + 2 * (((s & 15) >> 2) + 4 * (s & 3));
        else return 4 * (s & 7) + (s >> 3);
    }
    // slots of a transform's output that the centred half of a box keeps:
    // out_m(s) in 0..7 or 24..31
    static __device__ __forceinline__ constexpr bool keep(int s) { return out_m(s) < 8 || out_m(s) >= 24; }
    // For the centred half of a box (count N/2 at offset N/4), slot m (0..7 or
    // 24..31) of thread t is box element t + half_off(m), in 0 .. N/2 - 1: the
    // offsets are compile-time constants once the slot loops are unrolled.
    static __device__ __forceinline__ constexpr int half_off(int m) { return m < 8 ? P * m + N / 4 : P * m - 3 * N / 4; }
};

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

// 32-point DFT of the thread's slots in registers: slot m = 8a + b holds
// input m; output k ends in slot 8 (k & 3) + (k >> 2).  ZIN: slots 8..23 are
// known to be zero, so the first radix-4 stage takes two inputs.
template <typename T, bool INV, bool ZIN>
__device__ __forceinline__ void dft32_regs(cplx<T> (&x)[32])
{
    // radix 4 over a: slot 8a + b -> Z_b[k1'] in slot 8 k1' + b, rotated by W32^(b k1')
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
}

// One N-point transform of the thread's 32 elements.  In: slot m holds
// element t + P m.  Out: slot s holds element t + P out_m(s).  Uses the
// CTA's exchange buffer (synchronises after writing it, and before unless
// sync_in is false: no thread of the CTA has used the buffer yet).  ZIN: the
// elements of slots 8..23 are zero (the centred half of a box transform:
// entries t + P m + N/4 mod N below N/2 lie in slots 0..7 and 24..31).
template <typename T, int N, bool INV, bool ZIN = false>
__device__ __forceinline__ void r32_fft(cplx<T> (&x)[32], cplx<T> *S, int c, int t, const cplx<T> *__restrict__ tw,
                                        bool sync_in = true)
{
    using G = R32<N>;
    dft32_regs<T, INV, ZIN>(x);
    // WN^(t k1) and the exchange: S[k1][t].  The twiddles come from four
    // loads, WN^(t b) for b = 1..3 and WN^(4t): k1 = 4a + b runs along the chain
    // of b, one product by WN^(4t) per step (at most 7 products, a few units
    // in the last place; 31 loads measured 3 % slower over the iteration)
    if (sync_in) __syncthreads();  // the buffer may still be read by the previous step
    cplx<T> *Sc = S + c * G::CS;
    const cplx<T> *tt = tw + G::TWT + t;  // tt[k1 P] = WN^(t k1)
    cplx<T> cur[4] = {__ldg(tt + 4 * G::P), __ldg(tt + G::P), __ldg(tt + 2 * G::P), __ldg(tt + 3 * G::P)};
    const cplx<T> w4 = cur[0];
#pragma unroll
    for (int k1 = 0; k1 < 32; ++k1) {
        const int slot = 8 * (k1 & 3) + (k1 >> 2), b = k1 & 3;
        cplx<T> y = x[slot];
        if (k1) {
            y = ctw(y, cur[b], INV);
            if (k1 + 4 < 32) cur[b] = cmul(cur[b], w4);
        }
        Sc[k1 * G::ROW + t] = y;
    }
    __syncthreads();
    if constexpr (N <= 256) {
        // stage 2 for k1 = t + P h: slot P h + t' <- S[k1][t'], then the P-point
        // DFT of each group (X[k1 + 32 k2] in slot P h + k2)
#pragma unroll
        for (int h = 0; h < 32 / G::P; ++h)
#pragma unroll
            for (int tp = 0; tp < G::P; ++tp) x[G::P * h + tp] = Sc[(t + G::P * h) * G::ROW + tp];
#pragma unroll
        for (int h = 0; h < 32 / G::P; ++h) Dft<G::P, T>::run(&x[G::P * h], INV, nullptr, G::P);
    } else if constexpr (N == 512) {
        // stage 2 for k1 = t + 16 h: slot 16 h + t' <- S[k1][t']
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int tp = 0; tp < 16; ++tp) x[16 * h + tp] = Sc[(t + 16 * h) * G::ROW + tp];
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
    } else {
        // stage 2 for k1 = t: slot t' <- S[t][t'], a 32-point DFT over t'
        // (X[t + 32 k2] in slot 8 (k2 & 3) + (k2 >> 2))
#pragma unroll
        for (int tp = 0; tp < 32; ++tp) x[tp] = Sc[t * G::ROW + tp];
        dft32_regs<T, INV, false>(x);
    }
}

// CTAs per SM the column passes are built for (registers <= 65536 / (threads x
// this)).  512 points: 5 (96 registers; the fused pass spills 8 bytes there and
// measured 5 % faster than at 4 CTAs).  1024 points: 4 (128 registers, no
// spills; the 32-point second stage keeps more values live; 5 CTAs measured 3 %
// slower over the iteration).  128 and 256 points: 128 registers.
constexpr int r32_col_min_blocks(int n) { return n == 512 ? 5 : n == 1024 ? 4 : 2048 / n; }

// L2 prefetch distance (blocks) of the single-transform 512-point column
// passes: 380 took F2 and I2 from 0.080 / 0.082 to 0.076 / 0.078 ms at 512^3;
// the fused pass (+2 %) and the 1024-point passes (+4-15 %) measured slower
// with it, so they do without.
constexpr int r32_prefetch_ahead(int n, bool fused) { return (n == 512 && !fused) ? 380 : 0; }

// The transforms, the table phase and the stores of one tile (tile, other)
// of a column pass whose input is already in x (slot m holds element t + P m);
// tiles_x is the number of tiles along the columns (the index of the tile's
// errK partial).  Shared by the one-tile-per-CTA pass and the persistent one.
template <typename T, int N, bool ZIN, bool ZOUT>
__device__ __forceinline__ void col_r32_tile(const ColPassArgs<T> &a, cplx<T> *s, cplx<T> (&x)[32], int tile, int other,
                                             int tiles_x)
{
    using G = R32<N>;
    constexpr int P = G::P, W = G::W;
    using Lay = typename G::Lay;
    const int c = threadIdx.x % W, t = threadIdx.x / W;
    const int col = tile * W + c;
    const bool cv = col < a.ncols;
    const cplx<T> *twp = a.tw;
    ErrAcc<T> err = 0;
    bool fwd_layout = false;  // slots in the output order of a transform
    if (a.mode & 1) {
        r32_fft<T, N, false, ZIN>(x, s, c, t, twp, false);
        fwd_layout = true;
    }
    if (a.mode & 2) {
        if (a.mode & 1) {
            // back to slot m = element t + P m, through the natural-order tile
            // (where the Fourier constraint is applied)
            __syncthreads();
#pragma unroll
            for (int sl = 0; sl < 32; ++sl) s[Lay::idx(t + P * G::out_m(sl), c)] = x[sl];
            __syncthreads();
            if (a.mode & 4) {
                if (a.rtab) {
                    capture_rfree<T>(s, a, tile, W, other, [](int q3, int cl) { return Lay::idx(q3, cl); });
                    __syncthreads();
                }
                err = apply_table<T, Lay>(s, a, tile, W, other);
                block_partial(err, a.partial + (long long)other * tiles_x + tile);
                __syncthreads();
            }
#pragma unroll
            for (int m = 0; m < 32; ++m) x[m] = s[Lay::idx(t + P * m, c)];
        }
        r32_fft<T, N, true>(x, s, c, t, twp, (a.mode & 1) != 0);
        fwd_layout = true;
    }
    if (!fwd_layout || !cv) return;
    cplx<T> *out = a.out + (long long)other * a.out_other + (long long)col * a.col_stride;
    const unsigned odim = (unsigned)a.out_dim;
#pragma unroll
    for (int sl = 0; sl < 32; ++sl) {
        if constexpr (ZOUT) {
            if (G::keep(sl))
                out[(unsigned)(t + G::half_off(G::out_m(sl))) * odim] = mk(x[sl].x * a.scale, x[sl].y * a.scale);
            continue;
        }
        int e = t + P * G::out_m(sl) + a.out_c;
        if (e >= N) e -= N;
        if (e < a.out_cnt) out[(unsigned)e * odim] = mk(x[sl].x * a.scale, x[sl].y * a.scale);
    }
}

// Column pass (the contract of k_colpass) for n = N.  ZIN: the input is the
// centred half of a box (in_cnt N/2, in_c N/4) and the pass starts with a
// forward transform; ZOUT: only the centred half is written (out_cnt N/2,
// out_c N/4), so the final transform's other outputs are never formed.
template <typename T, int N, bool ZIN, bool ZOUT>
__global__ void __launch_bounds__(R32<N>::THREADS, r32_col_min_blocks(N)) k_col_r32(ColPassArgs<T> a)
{
    using G = R32<N>;
    constexpr int P = G::P, W = G::W;
    using Lay = typename G::Lay;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *s = reinterpret_cast<cplx<T> *>(smem_raw);
    if (a.ctl && blockIdx.x == 0 && blockIdx.y == 0) ctl_mid_update(a.ctl, a.partial, a.nparts, a.denom, a.hist);
    const int c = threadIdx.x % W, t = threadIdx.x / W;
    const int tile = blockIdx.x, other = blockIdx.y;
    const int col = tile * W + c;
    const bool cv = col < a.ncols;
    if (a.zmask && !a.zmask[other]) {
        // a slab without support voxels (see ColPassArgs::zmask)
        if (a.zmask_zero && cv) {
            cplx<T> *out = a.out + (long long)other * a.out_other + (long long)col * a.col_stride;
#pragma unroll 4
            for (int m = 0; m < 32; ++m) {
                int e = t + P * m + a.out_c;
                if (e >= N) e -= N;
                if (e < a.out_cnt) out[(unsigned)e * (unsigned)a.out_dim] = mk((T)0, (T)0);
            }
        }
        return;
    }
    const cplx<T> *twp = a.tw;  // twiddles<T>(N): see R32<N>::TWT
    cplx<T> x[32];
    if constexpr (r32_prefetch_ahead(N, ZIN && ZOUT) > 0) {
        // the input rows of the CTA that many blocks later in launch order
        // (half a wave of resident CTAs) are fetched into L2 now: rows the
        // kernel reads itself (column 0 of a valid tile, r < in_cnt)
        const long long nb = (long long)gridDim.x * gridDim.y;
        const long long fb = (long long)blockIdx.y * gridDim.x + blockIdx.x + r32_prefetch_ahead(N, ZIN && ZOUT);
        if (fb < nb && a.col_stride == 1) {
            const int ftile = (int)(fb % gridDim.x), fother = (int)(fb / gridDim.x);
            const cplx<T> *fin = a.in + (long long)fother * a.in_other + (long long)ftile * W;
            for (int r = threadIdx.x; r < a.in_cnt; r += G::THREADS)
                asm volatile("prefetch.global.L2 [%0];" ::"l"(fin + (long long)r * a.in_dim));
        }
    }
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
                x[m] = cv ? in[(unsigned)(t + G::half_off(m)) * idim] : mk((T)0, (T)0);
                continue;
            }
            int e = t + P * m + a.in_c;
            if (e >= N) e -= N;
            x[m] = (cv && e < a.in_cnt) ? in[(unsigned)e * idim] : mk((T)0, (T)0);
        }
    }
    col_r32_tile<T, N, ZIN, ZOUT>(a, s, x, tile, other, gridDim.x);
}

// Persistent fused 512-point complex64 pass (F3 at 512 points): CTAs loop over
// the tiles (tile, other) = (item % tiles_x, item / tiles_x), item += gridDim.x,
// and each tile's input (the centred half of the box: N/2 rows x W columns,
// 16 KB) comes into a shared-memory stage by a TMA tensor copy issued one tile
// ahead, while the CTA transforms the current one.  tmap describes the input
// as floats: {2 x in_other, in_dim / in_other, in_cnt} with the box
// {2 W, 1, N/2} (x = 2 W tile, 64-byte aligned).  The wait for a copy is bounded
// (clock64); on expiry the CTA stops at a reducing barrier, sets *a.err, waits
// (full limit) for the copy in flight and returns.
namespace r32tma {
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz
__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ bool try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool wait(uint64_t *bar, uint32_t parity)
{
    const long long t0 = clock64();
    while (!try_wait(bar, parity))
        if (clock64() - t0 > kWaitCycles) return false;
    return true;
}
__device__ __forceinline__ void load_tile(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            saddr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(0), "r"(saddr(bar))
        : "memory");
}
}  // namespace r32tma

template <int N> constexpr size_t r32_tma_stage_offset() { return (R32<N>::template smem<float>() + 127) / 128 * 128; }
template <int N> constexpr uint32_t r32_tma_stage_bytes() { return (uint32_t)(N / 2 * R32<N>::W * sizeof(float2)); }
template <int N> constexpr size_t r32_tma_smem() { return r32_tma_stage_offset<N>() + r32_tma_stage_bytes<N>() + 16; }

template <int N>
__global__ void __launch_bounds__(R32<N>::THREADS, 4)
    k_col_r32_tma(ColPassArgs<float> a, const __grid_constant__ CUtensorMap tmap, int tiles_x, int ntiles)
{
    using G = R32<N>;
    constexpr int W = G::W;
    constexpr uint32_t kBytes = r32_tma_stage_bytes<N>();
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    cplx<float> *s = reinterpret_cast<cplx<float> *>(smem_raw);
    cplx<float> *stage = reinterpret_cast<cplx<float> *>(smem_raw + r32_tma_stage_offset<N>());  // [N/2 rows][W]
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + r32_tma_stage_offset<N>() + kBytes);
    const int c = threadIdx.x % W, t = threadIdx.x / W;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(r32tma::saddr(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int item = blockIdx.x;
    if (threadIdx.x == 0 && item < ntiles)
        r32tma::load_tile(stage, &tmap, 2 * W * (item % tiles_x), item / tiles_x, bar, kBytes);
    bool pending = item < ntiles;  // a copy is in flight (uniform)
    uint32_t phase = 0;
    bool ok = true;
    for (; item < ntiles; item += gridDim.x) {
        const bool got = r32tma::wait(bar, phase);
        if (__syncthreads_or(!got)) {
            ok = false;
            break;
        }
        pending = false;
        phase ^= 1;
        cplx<float> x[32];
#pragma unroll
        for (int m = 0; m < 32; ++m) {
            if (m >= 8 && m < 24) x[m] = mk(0.f, 0.f);
            else x[m] = stage[(t + G::half_off(m)) * W + c];
        }
        // generic-proxy reads of the stage before the next tensor copy (async proxy)
        // overwrites it; after the barrier the stage and the exchange buffer are free
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        const int next = item + gridDim.x;
        if (next < ntiles) {
            if (threadIdx.x == 0) r32tma::load_tile(stage, &tmap, 2 * W * (next % tiles_x), next / tiles_x, bar, kBytes);
            pending = true;
        }
        col_r32_tile<float, N, true, true>(a, s, x, item % tiles_x, item / tiles_x, tiles_x);
    }
    if (!ok && threadIdx.x == 0 && a.err) atomicExch(a.err, 1);
    if (pending && threadIdx.x == 0) r32tma::wait(bar, phase);  // the copy in flight lands before the CTA exits
}

// Row passes (the contracts of k_rows_r2c / k_rows_c2r) for n = N: W pairs of
// real rows per CTA, each pair one complex transform (row a the real part,
// row b the imaginary part), P threads per pair with the index along the row
// fastest within a warp (64- or 128-byte row segments per access).
// Elements whose loads are in flight together in the forward row pass: 8 keeps
// the 512-point pass at 118 registers (4 CTAs per SM); 16 and 32 cost
// occupancy and measured 13 % and 54 % slower at 512^3.
constexpr int kRowLoadGroup = 8;

// ZIN: the rows are the centred half of the transform (B1 N/2, c1 N/4)
template <typename T, int N, bool ZIN>
__global__ void __launch_bounds__(R32<N>::THREADS) k_row_r2c_r32(RowPassArgs<T> a)
{
    using G = R32<N>;
    constexpr int P = G::P, W = G::W;
    using RowLay = typename G::RowLay;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *s = reinterpret_cast<cplx<T> *>(smem_raw);
    const int t = threadIdx.x % P, c = threadIdx.x / P;
    if (a.ctl && blockIdx.x == 0 && threadIdx.x == 0) ctl_begin_update(a.ctl, a.changes);
    const T *xs = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int r0 = (blockIdx.x * W + c) * 2, r1 = r0 + 1;
    const bool ok0 = r0 < a.nrows, ok1 = r1 < a.nrows;
    const long long o0 = (long long)r0 * a.B1, o1 = o0 + a.B1;
    if (row_pairs_empty(a, W)) {
        zero_half_rows(a, W);
        return;
    }
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
                const int e = t + G::half_off(m0 + i);
                xa[i] = ok0 ? xs[o0 + e] : (T)0;
                xb[i] = ok1 ? xs[o1 + e] : (T)0;
                sa[i] = (a.support && ok0) ? a.support[o0 + e] : (uint8_t)1;
                sb[i] = (a.support && ok1) ? a.support[o1 + e] : (uint8_t)1;
                continue;
            }
            int e = t + P * (m0 + i) + a.c1;
            if (e >= N) e -= N;
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
    r32_fft<T, N, false, ZIN>(x, s, c, t, a.tw, false);
    __syncthreads();  // the exchange buffer becomes the natural-order tile
#pragma unroll
    for (int sl = 0; sl < 32; ++sl) s[RowLay::idx(t + P * G::out_m(sl), c)] = x[sl];
    __syncthreads();
    // split the pair's spectrum Z into the rows' half spectra:
    // Xa(q) = (Z(q) + conj Z(-q)) / 2, Xb(q) = (Z(q) - conj Z(-q)) / 2i
    cplx<T> *ya = a.Y + (long long)r0 * a.ld1, *yb = ya + a.ld1;
    for (int q = t; q < a.h1; q += P) {
        const cplx<T> Z = s[RowLay::idx(q, c)];
        const cplx<T> Zm = s[RowLay::idx(q == 0 ? 0 : N - q, c)];
        if (ok0) ya[q] = mk((T)0.5 * (Z.x + Zm.x), (T)0.5 * (Z.y - Zm.y));
        if (ok1) yb[q] = mk((T)0.5 * (Z.y + Zm.y), (T)0.5 * (Zm.x - Z.x));
    }
}

// ZOUT: only the centred half of each row is written (B1 N/2, c1 N/4)
template <typename T, int N, bool ZOUT>
__global__ void __launch_bounds__(R32<N>::THREADS) k_row_c2r_r32(RowPassArgs<T> a)
{
    using G = R32<N>;
    constexpr int P = G::P, W = G::W;
    // the CTA's rows hold no support voxel: the next forward pass treats them
    // as zero without reading them (the mask is only set when nothing else
    // reads this pass's output outside the support)
    if (row_pairs_empty(a, W)) return;
    using RowLay = typename G::RowLay;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *s = reinterpret_cast<cplx<T> *>(smem_raw);
    const int t = threadIdx.x % P, c = threadIdx.x / P;
    T *xs = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int r0 = (blockIdx.x * W + c) * 2, r1 = r0 + 1;
    const bool ok0 = r0 < a.nrows, ok1 = r1 < a.nrows;
    {
        // pack the two half spectra: Z = Ha + i Hb on q < h1, Z(-q) from the
        // conjugate symmetry of each row; all loads issued before the packing
        constexpr int QIT = (N / 2 + P) / P;  // q = t + P it covers 0 .. N/2
        const cplx<T> *ya = a.Y + (long long)r0 * a.ld1, *yb = ya + a.ld1;
        cplx<T> HA[QIT], HB[QIT];
#pragma unroll
        for (int it = 0; it < QIT; ++it) {
            const int q = t + P * it;
            HA[it] = (q < a.h1 && ok0) ? ya[q] : mk((T)0, (T)0);
            HB[it] = (q < a.h1 && ok1) ? yb[q] : mk((T)0, (T)0);
        }
#pragma unroll
        for (int it = 0; it < QIT; ++it) {
            const int q = t + P * it;
            if (q >= a.h1) break;
            cplx<T> ha = HA[it], hb = HB[it];
            if (q == 0 || 2 * q == N) { ha.y = 0; hb.y = 0; }
            s[RowLay::idx(q, c)] = mk(ha.x - hb.y, ha.y + hb.x);
            if (q != 0 && N - q >= a.h1) s[RowLay::idx(N - q, c)] = mk(ha.x + hb.y, hb.x - ha.y);
        }
    }
    __syncthreads();
    cplx<T> x[32];
#pragma unroll
    for (int m = 0; m < 32; ++m) x[m] = s[RowLay::idx(t + P * m, c)];
    r32_fft<T, N, true>(x, s, c, t, a.tw);  // synchronises before it reuses the buffer
#pragma unroll
    for (int sl = 0; sl < 32; ++sl) {
        if constexpr (ZOUT) {
            if (G::keep(sl)) {
                const int e = t + G::half_off(G::out_m(sl));
                if (ok0) xs[(long long)r0 * a.B1 + e] = x[sl].x * a.scale;
                if (ok1) xs[(long long)r1 * a.B1 + e] = x[sl].y * a.scale;
            }
            continue;
        }
        int e = t + P * G::out_m(sl) + a.c1;
        if (e >= N) e -= N;
        if (e < a.B1) {
            if (ok0) xs[(long long)r0 * a.B1 + e] = x[sl].x * a.scale;
            if (ok1) xs[(long long)r1 * a.B1 + e] = x[sl].y * a.scale;
        }
    }
}

}  // namespace gf
