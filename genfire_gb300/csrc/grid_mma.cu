// grid_mma.cu -- the reduced-precision gridding DFT on the 5th-generation
// tensor cores (tcgen05, sm_103a).
//
// For one projection P (D1 x D2) and a tile of 128 selected K-points j:
//   Q(j, b) = sum_a E_u(j, a) P(a, b),  E_u(j, a) = exp(-2 pi i a u_j / n1)
//   F_j     = sum_b Q(j, b) E_v(j, b),  E_v(j, b) = exp(-2 pi i b v_j / n2)
// (fillInFourierGrid_DFT.m:243).  Q is a GEMM with M = 128 K-points, N = D2
// and K = D1.  Operands are split into hi + lo parts of a 16-bit type and
// multiplied as hi*hi + hi*lo + lo*hi with FP32 accumulation:
//   Re Q += Re(E_u)_hi P_hi + Re(E_u)_hi P_lo + Re(E_u)_lo P_hi
//   Im Q += Im(E_u)_hi P_hi + Im(E_u)_hi P_lo + Im(E_u)_lo P_hi
// The 16-bit type is BF16 (GENFIRE_PREC_MIXED: ~16 significant bits per
// operand) or FP16 (GENFIRE_PREC_FP16_SCALED: ~22 bits, with each projection
// scaled by a power of two so that its largest value sits just below 2^14 and
// the lo parts stay in FP16's normal range; the scale is undone exactly in the
// epilogue).
//
// Work decomposition.  P is pre-split once into blocks of 128 columns (b) by
// 256 rows (a) in the canonical no-swizzle K-major layout (128 KB per block,
// hi and lo).  A unit of work is (tile of 128 points, block): the tile's
// partial Q over the block's rows and columns, contracted with E_v over the
// block's columns, gives a partial F; the partials of a point (one per block
// of its projection, two for 256 x 256 projections) are summed in block order
// afterwards.  Units are ordered by projection, block, tile, and each CTA
// (one per SM) takes a contiguous range of them, so it keeps one block
// resident in shared memory across many tiles and reloads it (one bulk copy)
// only a few times.
//
// Warp roles in each CTA:
//   warps 0-3   epilogue: thread = TMEM lane = point; tcgen05.ld of the Re and
//               Im accumulators, per 16-column group Horner's rule in E_v(2)
//               over its even and odd columns at once (packed FP32 pairs),
//               times an anchor E_v(b_g) (exact every 64 columns), partial F
//               stored;
//   warp 4      one thread loads blocks (cp.async.bulk into shared memory,
//               completing on an mbarrier) and issues tcgen05.mma (M = 128,
//               N <= 128, K = 16), committing to mbarriers;
//   warps 5-12  A producers: per 32-wide K chunk, each thread forms 16
//               consecutive E_u(j, a) of one point as packed FP32 pairs
//               (real parts of two neighbours in one register pair, imaginary
//               parts in another) by four independent chains of packed
//               rotations from an anchor (exact every 4 chunks), splits them
//               into hi/lo (one packed subtraction per pair) and stores them in
//               the K-major layout; three A stages.
// The accumulator (Re and Im, 2 x 128 columns) is double buffered in TMEM, so
// the epilogue of one unit overlaps the MMAs of the next.
//
// Every mbarrier wait is bounded by a clock limit.  A role whose wait expires
// sets a shared abort flag; the other roles see it in their own waits and
// stop.  The issuing thread then waits (full limit) for its MMAs (one final
// tcgen05.commit) and its block copy in flight, every thread meets at one
// barrier, TMEM is freed and the CTA returns; the host reports
// GENFIRE_ERR_TIMEOUT.
#include "internal.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdlib>
#include <cstring>
#include <mutex>
#include <set>
#include <utility>

namespace gf {

namespace umma {

constexpr int kM = 128;            // rows (points) per tile
constexpr int kKC = 32;            // K per chunk (two MMA k-steps of 16)
constexpr long long kWaitCycles = 4000000000LL;               // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Canonical no-swizzle K-major layout: core matrices of 8 rows x 8 bf16
// (16 bytes per row, 128 bytes each); core matrices adjacent along K are 128 B
// apart (leading byte offset), 8-row groups are 512 B apart (stride byte
// offset) for a 32-wide K chunk.
__device__ __forceinline__ int kmaj_index(int row, int k) { return (row >> 3) * 256 + (k >> 3) * 64 + (row & 7) * 8 + (k & 7); }
constexpr uint32_t kLBO = 128, kSBO = 512;

__device__ __forceinline__ uint64_t sdesc(uint32_t addr)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((kLBO >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((kSBO >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of the 5th-generation tensor core
    return d;                // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity)
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
// non-blocking test of a phase
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait; returns false on expiry.  try_wait may suspend the thread for a
// time the hardware chooses before it reports failure, so a limit shorter than
// the default (the error-path test) polls with test_wait, which never suspends.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long limit = kWaitCycles)
{
    const long long t0 = clock64();
    if (limit < kWaitCycles) {
        while (!mbar_test(bar, parity))
            if (clock64() - t0 > limit) return false;
        return true;
    }
    while (!mbar_try(bar, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     saddr(dst)),
                 "l"(src), "r"(bytes), "r"(saddr(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(dst)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t accum)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(accum)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
                 : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// exp(-2 pi i * a * w / n) for integer a and FP32 w, phase reduced in FP64
__device__ __forceinline__ float2 phase_exact(int a, float w, double inv_n)
{
    double t = (double)a * (double)w * inv_n;
    t -= rint(t);
    float s, c;
    sincospif((float)(-2.0 * t), &s, &c);
    return make_float2(c, s);
}
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

// v * 2^-sh as a float for |v| < 2^62 and 1 <= sh <= 125, from three 23-bit
// chunks, each converted exactly by the 2^23 bias trick (0x4B000000 | c is the
// float 2^23 + c) and combined with FP32 fused multiply-adds, smallest first.
// A 64-bit integer conversion would issue on the FP64 pipe, which this part
// runs at 2 operations per clock per SM.
__device__ __forceinline__ float i64_scaled(long long v, int sh)
{
    const unsigned long long a = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
    const float c0 = __int_as_float(0x4B000000 | (unsigned)(a & 0x7FFFFFull)) - 8388608.f;
    const float c1 = __int_as_float(0x4B000000 | (unsigned)((a >> 23) & 0x7FFFFFull)) - 8388608.f;
    const float c2 = __int_as_float(0x4B000000 | (unsigned)((a >> 46) & 0x7FFFFFull)) - 8388608.f;
    auto p2 = [](int e) { return __int_as_float((127 + e) << 23); };  // 2^e, -126 < e < 128
    float f = c0 * p2(-sh);
    f = fmaf(c1, p2(23 - sh), f);
    f = fmaf(c2, p2(46 - sh), f);
    return v < 0 ? -f : f;
}

// exp(-2 pi i * a * w / 2^t) with the phase reduced exactly in integer
// arithmetic: w = m * 2^e (m the 24-bit significand), a * m is exact in 64
// bits, and the fraction of a*m*2^(e-t) is its low (t-e) bits.  No FP64 (the
// FP64 pipe issues 2 instructions per clock per SM on this part).
__device__ __forceinline__ float2 phase_pow2(int a, float w, int t)
{
    const int bits = __float_as_int(w);
    const int ex = (bits >> 23) & 0xFF;
    float f;
    if (ex == 0) {
        f = 0.f;  // zero or subnormal: the phase is below 2^-100
    } else {
        long long m = (long long)((bits & 0x7FFFFF) | 0x800000);
        if (bits < 0) m = -m;
        const int sh = t - (ex - 150);  // a*w/2^t = (a*m) * 2^-sh
        const long long P = (long long)a * m;
        if (sh <= 0) {
            f = 0.f;  // an integer number of turns
        } else if (sh >= 62) {
            f = sh > 125 ? 0.f : i64_scaled(P, sh);  // |P| < 2^47: below 2^-15 turns
        } else {
            long long low = P & ((1LL << sh) - 1);
            if (low >= (1LL << (sh - 1))) low -= (1LL << sh);  // to [-1/2, 1/2) turns
            f = i64_scaled(low, sh);
        }
    }
    float sv, cv;
    sincospif(-2.f * f, &sv, &cv);
    return make_float2(cv, sv);
}

// exact phase: the integer form for power-of-two n (POW2, chosen at compile
// time so the FP64 form is not speculated alongside), else FP64
template <bool POW2> __device__ __forceinline__ float2 phase_any(int a, float w, int log2n, double inv_n)
{
    if constexpr (POW2) return phase_pow2(a, w, log2n);
    else return phase_exact(a, w, inv_n);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo_elem, float hi_elem)
{
    __nv_bfloat162 t = __floats2bfloat162_rn(lo_elem, hi_elem);  // .x = first (lower address)
    return *reinterpret_cast<uint32_t *>(&t);
}
// the two BF16 halves of a packed word as floats (exact)
__device__ __forceinline__ float bf16_lo_f(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi_f(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

}  // namespace umma

namespace umma {

constexpr int kN = 128;                        // columns of one block (N of the MMAs)
constexpr int kKR = 256;                       // rows of one block (its K range)
constexpr int kKCB = kKR / kKC;                // K chunks per block (8)
constexpr int kABytes = kM * kKC * 2;          // one A array of a chunk (8 KB)
constexpr int kAStage = 4 * kABytes;           // re_hi, re_lo, im_hi, im_lo (32 KB)
constexpr int kStages = 3;
constexpr int kBArr = kN * kKC;                // elements of one B array of a chunk
constexpr int kBChunk = 2 * kBArr * 2;         // hi + lo of one chunk (16 KB)
constexpr int kBBytes = kKCB * kBChunk;        // one block (128 KB)
constexpr int kEpiWarps = 4, kMmaWarp = 4, kProdWarp0 = 5, kProdWarps = 8;
constexpr int kProdThreads = 32 * kProdWarps;
constexpr int kWsThreads = 32 * (kProdWarp0 + kProdWarps);  // 416
constexpr int kNBars = 2 * kStages + 4 + 3;    // afull, aempty, tfull x2, tempty x2, bfull, bdone, drain
constexpr size_t kWsSmem = (size_t)kBBytes + kStages * kAStage + 8 * kNBars + 16;

// kind::f16 instruction descriptor: FP32 accumulator, FP16 A and B, both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N)
{
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(bar)) : "memory");
}

// Bounded wait that also stops when another role of the CTA has given up
// (abort flag); an expired wait sets the flag.
__device__ __forceinline__ bool ws_wait(uint64_t *bar, uint32_t parity, long long limit, volatile int *abort_flag)
{
    const long long t0 = clock64();
    const bool poll = limit < kWaitCycles;
    for (;;) {
        if (poll ? mbar_test(bar, parity) : mbar_try(bar, parity)) return true;
        if (*abort_flag) return false;
        if (clock64() - t0 > limit) {
            *abort_flag = 1;
            return false;
        }
    }
}

// two floats rounded to a packed pair of the 16-bit operand type (first at the
// lower address), and the halves of such a pair back as floats (exact)
template <bool F16> __device__ __forceinline__ uint32_t pack2(float a, float b)
{
    if constexpr (F16) {
        __half2 t = __floats2half2_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&t);
    } else {
        return pack_bf16(a, b);
    }
}
template <bool F16> __device__ __forceinline__ float half_lo(uint32_t w)
{
    if constexpr (F16) return __half2float(__ushort_as_half((unsigned short)(w & 0xFFFFu)));
    else return bf16_lo_f(w);
}
template <bool F16> __device__ __forceinline__ float half_hi(uint32_t w)
{
    if constexpr (F16) return __half2float(__ushort_as_half((unsigned short)(w >> 16)));
    else return bf16_hi_f(w);
}

// Packed FP32 pairs (add/sub/mul/fma.rn.f32x2: one instruction for both
// halves; each half rounds as the scalar operation would).
typedef unsigned long long f2x_t;
__device__ __forceinline__ f2x_t pk(float lo, float hi)
{
    f2x_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float2 upk(f2x_t r)
{
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
__device__ __forceinline__ f2x_t sub_x2(f2x_t a, f2x_t b)
{
    f2x_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x_t mul_x2(f2x_t a, f2x_t b)
{
    f2x_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x_t fma_x2(f2x_t a, f2x_t b, f2x_t c)
{
    f2x_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// Two complex values held as (X, Y) = ((re0, re1), (im0, im1)), both rotated
// by the complex w given as the pairs (w.x, w.x), (w.y, w.y), (-w.y, -w.y).
__device__ __forceinline__ void rot_x2(f2x_t &X, f2x_t &Y, f2x_t wx, f2x_t wy, f2x_t nwy)
{
    const f2x_t x = fma_x2(Y, nwy, mul_x2(X, wx));
    Y = fma_x2(Y, wx, mul_x2(X, wy));
    X = x;
}
// hi/lo split of a pair: hi = the pair rounded to the 16-bit type (packed),
// lo = (pair - hi) rounded (packed); the residual is one packed subtraction
template <bool F16> __device__ __forceinline__ void split_x2(f2x_t v, uint32_t &hi, uint32_t &lo)
{
    const float2 f = upk(v);
    hi = pack2<F16>(f.x, f.y);
    const float2 r = upk(sub_x2(v, pk(half_lo<F16>(hi), half_hi<F16>(hi))));
    lo = pack2<F16>(r.x, r.y);
}

}  // namespace umma

// One unit of work: a tile of up to 128 consecutive selected points of one
// projection against one block (128 columns x 256 rows) of that projection.
struct WsUnit {
    long long j0;  // first point
    int proj;
    int blk;       // block index (proj * nnc + nc) * nkr + kr
    int nj;        // points in the tile (<= 128)
    int pad;
};

struct WsArgs {
    const uint16_t *B;        // pre-split blocks: [blk][K chunk][hi|lo][128 x 32], 16-bit words
    const WsUnit *units;
    int nunits;
    const float *u, *v;
    const float *inv_scale;   // per projection (1 for BF16)
    float2 *F;                // partial F: [part][ntot], part = nc * nkr + kr
    long long ntot;
    int D1, D2, D1p, D2p;     // D1p: D1 rounded up to 32; D2p: D2 rounded up to 16
    int n1, n2, log2n1, log2n2;
    int nnc, nkr;
    // first form, one K block of D1 = 64 H rows: K runs a = 0 .. 32H-1 (chunks
    // 0 .. H-1) then a = -1 .. -32H (chunks H .. 2H-1), consumed as the pairs
    // (p, H + p); 0 for the natural order
    int mirror;
    int *err;                 // set to 1 when a bounded wait expired
    long long wait_cycles;    // limit of the pipeline's waits (the drain always allows kWaitCycles)
};

template <bool F16, bool POW2>
__global__ void __launch_bounds__(umma::kWsThreads, 1) k_dft_tcgen05(WsArgs a)
{
    using namespace umma;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *sB = smem_raw;
    unsigned char *sA = smem_raw + kBBytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw + kBBytes + kStages * kAStage);
    uint64_t *afull = bars, *aempty = bars + kStages, *tfull = bars + 2 * kStages, *tempty = tfull + 2;
    uint64_t *bfull = tempty + 2, *bdone = bfull + 1, *drain = bdone + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + kNBars);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&afull[s], kProdThreads);
            mbar_init(&aempty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 32 * kEpiWarps);
        }
        mbar_init(bfull, 1);
        mbar_init(bdone, 1);
        mbar_init(drain, 1);
        *abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == kMmaWarp) {
        tmem_alloc(tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // this CTA's contiguous range of units
    const int u0 = (int)((long long)a.nunits * blockIdx.x / gridDim.x);
    const int u1 = (int)((long long)a.nunits * (blockIdx.x + 1) / gridDim.x);
    const long long lim = a.wait_cycles;
    const int nparts = a.nnc * a.nkr;

    if (warp == kMmaWarp) {
        if (lane == 0) {
            // ---------------------------------------------------------------- MMA issue
            int cur_blk = -1;
            uint32_t g = 0, nbf = 0, nbd = 0;  // A chunks consumed; bfull / bdone phases seen
            bool b_pending = false;             // a block copy issued but not seen complete
            for (int i = u0; i < u1; ++i) {
                const WsUnit un = a.units[i];
                const int part = un.blk % nparts, nc = part / a.nkr, kr = part % a.nkr;
                const int Nc = min(kN, a.D2p - kN * nc);
                const int nkc = min(kKCB, (a.D1p - kKR * kr) / kKC);
                bool ok = true;
                if (un.blk != cur_blk) {
                    if (cur_blk >= 0) {  // the MMAs that read the resident block must be complete
                        mma_commit(bdone);
                        if (!ws_wait(bdone, nbd & 1, lim, abort_flag)) break;
                        ++nbd;
                    }
                    mbar_expect_tx(bfull, (uint32_t)(nkc * kBChunk));
                    const unsigned char *src = reinterpret_cast<const unsigned char *>(a.B) + (size_t)un.blk * kBBytes;
                    for (int c = 0; c < nkc; ++c) bulk_g2s(sB + c * kBChunk, src + (size_t)c * kBChunk, kBChunk, bfull);
                    b_pending = true;
                    if (!ws_wait(bfull, nbf & 1, lim, abort_flag)) break;
                    ++nbf;
                    b_pending = false;
                    cur_blk = un.blk;
                }
                const int li = i - u0, buf = li & 1;
                if (li >= 2 && !ws_wait(&tempty[buf], ((li >> 1) - 1) & 1, lim, abort_flag)) break;
                tc_fence_after();
                const uint32_t idesc = F16 ? idesc_f16(kM, Nc) : idesc_bf16(kM, Nc);
                const uint32_t dre = tmem + (uint32_t)(buf * 256), dim = dre + 128;
                for (int kc = 0; kc < nkc; ++kc, ++g) {
                    const int s = (int)(g % kStages);
                    if (!ws_wait(&afull[s], (g / kStages) & 1, lim, abort_flag)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    // the B chunk of this A chunk (pairs (p, H + p) in the mirrored order)
                    const int bc = a.mirror ? ((kc & 1) ? a.mirror + (kc >> 1) : (kc >> 1)) : kc;
                    const uint32_t a_base = saddr(sA + s * kAStage), b_base = saddr(sB + bc * kBChunk);
#pragma unroll
                    for (int ks = 0; ks < 2; ++ks) {
                        const uint32_t ko = ks * 16 * 16;  // 16 k = two core matrices = 256 bytes
                        const uint64_t b_hi = sdesc(b_base + ko), b_lo = sdesc(b_base + kBArr * 2 + ko);
                        const uint64_t a_rh = sdesc(a_base + ko), a_rl = sdesc(a_base + kABytes + ko);
                        const uint64_t a_ih = sdesc(a_base + 2 * kABytes + ko), a_il = sdesc(a_base + 3 * kABytes + ko);
                        const uint32_t first = (kc == 0 && ks == 0) ? 0u : 1u;
                        mma_bf16(dre, a_rh, b_hi, idesc, first);
                        mma_bf16(dre, a_rh, b_lo, idesc, 1u);
                        mma_bf16(dre, a_rl, b_hi, idesc, 1u);
                        mma_bf16(dim, a_ih, b_hi, idesc, first);
                        mma_bf16(dim, a_ih, b_lo, idesc, 1u);
                        mma_bf16(dim, a_il, b_hi, idesc, 1u);
                    }
                    mma_commit(&aempty[s]);  // the stage is free once these MMAs have read it
                }
                if (!ok) break;
                mma_commit(&tfull[buf]);  // the unit's accumulator is complete
            }
            // drain: every MMA this thread issued, then a block copy still in flight
            mma_commit(drain);
            mbar_wait(drain, 0);
            if (b_pending) mbar_wait(bfull, nbf & 1);
        }
    } else if (warp >= kProdWarp0) {
        // -------------------------------------------------------------------- A producers
        const int q = tid - kProdWarp0 * 32;
        const int r = q & (kM - 1), h = q >> 7;  // point (row) and half of the 32-wide chunk
        const double inv1 = 1.0 / (double)a.n1;
        const int amin = -(a.D1 / 2);
        uint32_t g = 0;
        bool ok = true;
        for (int i = u0; i < u1 && ok; ++i) {
            const WsUnit un = a.units[i];
            const int kr = (un.blk % nparts) % a.nkr;
            const int nkc = min(kKCB, (a.D1p - kKR * kr) / kKC);
            const bool row_ok = r < un.nj;
            const float uj = row_ok ? a.u[un.j0 + r] : 0.f;
            // rotations of the row: by 1 (odd elements), 2 (chain step), 4, 8, 12 (chain
            // starts) and 32 (next chunk); the packed ones as ((x, x), (y, y), (-y, -y))
            const float2 w1 = phase_any<POW2>(1, uj, a.log2n1, inv1);
            const float2 w4 = phase_any<POW2>(4, uj, a.log2n1, inv1);
            const float2 w2 = cmulf(w1, w1), w8 = cmulf(w4, w4), w12 = cmulf(w8, w4);
            const float2 w32 = cmulf(cmulf(w8, w8), cmulf(w8, w8));
            const f2x_t w2x = pk(w2.x, w2.x), w2y = pk(w2.y, w2.y), w2n = pk(-w2.y, -w2.y);
            const f2x_t w4x = pk(w4.x, w4.x), w4y = pk(w4.y, w4.y), w4n = pk(-w4.y, -w4.y);
            const f2x_t w8x = pk(w8.x, w8.x), w8y = pk(w8.y, w8.y), w8n = pk(-w8.y, -w8.y);
            const f2x_t wcx = pk(w12.x, w12.x), wcy = pk(w12.y, w12.y), wcn = pk(-w12.y, -w12.y);
            float2 anchor = make_float2(0.f, 0.f);
            // 16 consecutive k of row r from an anchor E_u(a): 8 pairs (2p, 2p+1), each
            // pair's real parts and imaginary parts packed: pair 0 from the anchor,
            // pairs 2, 4, 6 rotated from it by 4, 8, 12 and every odd pair from the one
            // before it by 2 (four independent chains of packed rotations, at most
            // three rotations from the anchor), split into hi/lo words
            uint32_t rh[9], rl[9], ih[9], il[9];
            auto gen = [&](float2 anc) {
                const float2 e1 = cmulf(anc, w1);
                f2x_t X[8], Y[8];
                X[0] = pk(anc.x, e1.x);
                Y[0] = pk(anc.y, e1.y);
                X[2] = X[0]; Y[2] = Y[0]; rot_x2(X[2], Y[2], w4x, w4y, w4n);
                X[4] = X[0]; Y[4] = Y[0]; rot_x2(X[4], Y[4], w8x, w8y, w8n);
                X[6] = X[0]; Y[6] = Y[0]; rot_x2(X[6], Y[6], wcx, wcy, wcn);
#pragma unroll
                for (int m = 0; m < 8; m += 2) {
                    X[m + 1] = X[m];
                    Y[m + 1] = Y[m];
                    rot_x2(X[m + 1], Y[m + 1], w2x, w2y, w2n);
                }
#pragma unroll
                for (int m = 0; m < 8; ++m) {
                    split_x2<F16>(X[m], rh[m], rl[m]);
                    split_x2<F16>(Y[m], ih[m], il[m]);
                }
                // the 17th value, E_u(a + 16) = E_u(a + 15) E_u(1), in the low halves
                const float2 v15 = make_float2(upk(X[7]).y, upk(Y[7]).y);
                const float2 v16 = cmulf(v15, w1);
                split_x2<F16>(pk(v16.x, 0.f), rh[8], rl[8]);
                split_x2<F16>(pk(v16.y, 0.f), ih[8], il[8]);
            };
            // the next A stage, once the MMAs that read it last have completed
            auto acquire = [&](int &st) -> bool {
                st = (int)(g % kStages);
                return g < (uint32_t)kStages || ws_wait(&aempty[st], ((g / kStages) - 1) & 1, lim, abort_flag);
            };
            auto store = [&](int st, const uint32_t *wrh, const uint32_t *wrl, const uint32_t *wih, const uint32_t *wil) {
                uint16_t *As = reinterpret_cast<uint16_t *>(sA + st * kAStage);
#pragma unroll
                for (int c8 = 0; c8 < 2; ++c8) {
                    const int idx = kmaj_index(r, 16 * h + 8 * c8);  // one 16-byte core-matrix row
                    const int k0 = 4 * c8;
                    *reinterpret_cast<uint4 *>(As + 0 * (kABytes / 2) + idx) = make_uint4(wrh[k0], wrh[k0 + 1], wrh[k0 + 2], wrh[k0 + 3]);
                    *reinterpret_cast<uint4 *>(As + 1 * (kABytes / 2) + idx) = make_uint4(wrl[k0], wrl[k0 + 1], wrl[k0 + 2], wrl[k0 + 3]);
                    *reinterpret_cast<uint4 *>(As + 2 * (kABytes / 2) + idx) = make_uint4(wih[k0], wih[k0 + 1], wih[k0 + 2], wih[k0 + 3]);
                    *reinterpret_cast<uint4 *>(As + 3 * (kABytes / 2) + idx) = make_uint4(wil[k0], wil[k0 + 1], wil[k0 + 2], wil[k0 + 3]);
                }
                fence_proxy_async();  // the stores are visible to the tensor core
                mbar_arrive(&afull[st]);
                ++g;
            };
            if (a.mirror) {
                // K as a = 0 .. 32H-1, then a = -1 .. -32H: the chunk pair (p, H + p).
                // The negative chunk's element k holds E_u(-(32p + k) - 1) =
                // conj E_u(32p + k + 1): this thread's values shifted by one (its 17th
                // value closes the row), the words re-paired by a byte permute and the
                // imaginary parts negated by their sign bits (the hi/lo split of -x is
                // -hi, -lo).  The anchor E_u(32p + 16h) is exact every 4 pairs.
                for (int pp = 0; pp < nkc / 2; ++pp) {
                    if ((pp & 3) == 0)
                        anchor = row_ok ? phase_any<POW2>(kKC * pp + 16 * h, uj, a.log2n1, inv1) : make_float2(0.f, 0.f);
                    else
                        anchor = cmulf(anchor, w32);
                    gen(anchor);
                    int st;
                    if (!acquire(st)) { ok = false; break; }
                    store(st, rh, rl, ih, il);
                    uint32_t nrh[8], nrl[8], nih[8], nil[8];
#pragma unroll
                    for (int m = 0; m < 8; ++m) {
                        nrh[m] = __byte_perm(rh[m], rh[m + 1], 0x5432);
                        nrl[m] = __byte_perm(rl[m], rl[m + 1], 0x5432);
                        nih[m] = __byte_perm(ih[m], ih[m + 1], 0x5432) ^ 0x80008000u;
                        nil[m] = __byte_perm(il[m], il[m + 1], 0x5432) ^ 0x80008000u;
                    }
                    if (!acquire(st)) { ok = false; break; }
                    store(st, nrh, nrl, nih, nil);
                }
            } else {
                for (int kc = 0; kc < nkc; ++kc) {
                    // 16 consecutive k of row r: a = amin + kr*256 + kc*32 + 16h + 0..15; the
                    // anchor E_u(a) is exact every 4 chunks and one rotation by 32 from the
                    // previous chunk's otherwise
                    if ((kc & 3) == 0)
                        anchor = row_ok ? phase_any<POW2>(amin + kKR * kr + kKC * kc + 16 * h, uj, a.log2n1, inv1)
                                        : make_float2(0.f, 0.f);
                    else
                        anchor = cmulf(anchor, w32);
                    gen(anchor);
                    int st;
                    if (!acquire(st)) { ok = false; break; }
                    store(st, rh, rl, ih, il);
                }
            }
        }
    } else {
        // -------------------------------------------------------------------- epilogue
        const int row = warp * 32 + lane;  // TMEM lane of this warp's quadrant
        const double inv2 = 1.0 / (double)a.n2;
        const int bmin = -(a.D2 / 2);
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
        for (int i = u0; i < u1; ++i) {
            const WsUnit un = a.units[i];
            const int part = un.blk % nparts, nc = part / a.nkr;
            const int Nc = min(kN, a.D2p - kN * nc);
            const int li = i - u0, buf = li & 1;
            if (!ws_wait(&tfull[buf], (li >> 1) & 1, lim, abort_flag)) break;
            tc_fence_after();
            const bool row_ok = row < un.nj;
            const float vj = row_ok ? a.v[un.j0 + row] : 0.f;
            const float2 v1 = phase_any<POW2>(1, vj, a.log2n2, inv2);
            const float2 v16 = phase_any<POW2>(16, vj, a.log2n2, inv2);
            const float2 v2 = cmulf(v1, v1);
            const f2x_t v2x = pk(v2.x, v2.x), v2y = pk(v2.y, v2.y), v2n = pk(-v2.y, -v2.y);
            const uint32_t cre = tmem + lane_base + (uint32_t)(buf * 256), cim = cre + 128;
            float2 Fsum = make_float2(0.f, 0.f), an = make_float2(0.f, 0.f);
            // F += sum_b Q(j,b) E_v(j,b) over 16-column groups: with w = E_v(1), a group's
            // sum_i Q_i w^i is A(w^2) + w B(w^2), A and B the polynomials of its even and
            // odd columns, both evaluated by Horner's rule in one packed chain (the pair
            // (A, B) of real parts and the pair of imaginary parts), then multiplied by
            // the group's anchor E_v(b_g) (exact every 64 columns, one rotation by 16
            // from the previous group otherwise); two groups per step (independent
            // chains, one wait for both loads)
            auto group = [&](const uint32_t(&re)[16], const uint32_t(&im)[16], float2 anc) {
                f2x_t H = pk(__uint_as_float(re[14]), __uint_as_float(re[15]));
                f2x_t G = pk(__uint_as_float(im[14]), __uint_as_float(im[15]));
#pragma unroll
                for (int t = 6; t >= 0; --t) {
                    const f2x_t qr = pk(__uint_as_float(re[2 * t]), __uint_as_float(re[2 * t + 1]));
                    const f2x_t qi = pk(__uint_as_float(im[2 * t]), __uint_as_float(im[2 * t + 1]));
                    const f2x_t h2 = fma_x2(H, v2x, fma_x2(G, v2n, qr));
                    G = fma_x2(H, v2y, fma_x2(G, v2x, qi));
                    H = h2;
                }
                const float2 hr = upk(H), hi = upk(G);  // (A.re, B.re), (A.im, B.im)
                const float2 sB = cmulf(make_float2(hr.y, hi.y), v1);
                const float2 p = cmulf(make_float2(hr.x + sB.x, hi.x + sB.y), anc);
                Fsum.x += p.x;
                Fsum.y += p.y;
            };
            for (int c = 0; c < Nc; c += 32) {
                const bool two = c + 16 < Nc;  // warp-uniform
                uint32_t re0[16], im0[16], re1[16], im1[16];
                tmem_ld16(cre + (uint32_t)c, re0);
                tmem_ld16(cim + (uint32_t)c, im0);
                if (two) {
                    tmem_ld16(cre + (uint32_t)(c + 16), re1);
                    tmem_ld16(cim + (uint32_t)(c + 16), im1);
                }
                const float2 an0 = (c & 63) == 0 ? (row_ok ? phase_any<POW2>(bmin + kN * nc + c, vj, a.log2n2, inv2)
                                                          : make_float2(0.f, 0.f))
                                                 : cmulf(an, v16);
                an = cmulf(an0, v16);  // the second group's anchor
                tmem_wait_ld();
                group(re0, im0, an0);
                if (two) group(re1, im1, an);
            }
            tc_fence_before();
            mbar_arrive(&tempty[buf]);  // this thread's TMEM reads of the buffer are complete
            if (row_ok) {
                const float sc = a.inv_scale[un.proj];
                a.F[(size_t)part * a.ntot + un.j0 + row] = make_float2(Fsum.x * sc, Fsum.y * sc);
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0 && *abort_flag) atomicExch(a.err, 1);
    if (warp == kMmaWarp) tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// Second form (opt-in): Re and Im stacked in the MMA rows, N = 256.
//
// A tile holds 64 points; its 128 MMA rows are, in each 32-lane quadrant q,
// lanes 0-15 the real parts and lanes 16-31 the imaginary parts of E_u for
// points 16 q .. 16 q + 15.  The accumulator of a unit is then one 128-lane x
// N matrix (row = Re or Im of a point), so N = 256 fits twice in the 512
// tensor-memory columns and stays double buffered.  B blocks are 256 columns
// x 128 rows (four K chunks of [hi | lo][256 x 32], 128 KB), and per K = 16
// step three MMAs (M = 128, N = 256): A_hi B_hi, A_hi B_lo, A_lo B_hi.  An MMA
// reads 4 KB of A and 8 KB of B for 2 x 128 x 128 x 16 MACs: 6 KB per
// 128 x 128 x 16, against 8 KB in the first form, whose MMAs the shared-memory
// pipe bounds.  A stages: 128 rows x 32 K, hi and lo (16 KB), six of them.
//
// Roles: two epilogue groups of four warps (group g drains accumulator buffer
// g), one MMA warp, eight producers.  Producers: warp 9 + i writes quadrant
// (9 + i) % 4 and half (i / 4) of each 32-wide K chunk; of the two lanes of a
// point, the Re lane forms E_u for the first 8 K of its half and the Im lane
// for the last 8, and they swap the other component's words with one shuffle
// per packed pair, so each lane holds its row's 16 K (two 16-byte stores per
// part).  Epilogue: each lane contracts its row (real Q) with E_v by the
// packed Horner scheme; F = S_re + i S_im, the Im lane's sum taken by a
// shuffle.  Waits are bounded as in the first form; their outcome is made
// warp-uniform before the warp-collective tensor-memory loads.
namespace umma {
constexpr int kWPoints = 64;                          // points per tile
constexpr int kWN = 256;                              // columns of one block (N of the MMAs)
constexpr int kWKR = 128;                             // rows of one block (its K range)
constexpr int kWKCB = kWKR / kKC;                     // K chunks per block (4)
constexpr int kWAArr = 128 * kKC;                     // elements of one A array of a chunk (8 KB)
constexpr int kWAStage = 2 * kWAArr * 2;              // hi + lo (16 KB)
constexpr int kWStages = 6;
constexpr int kWBArr = kWN * kKC;                     // elements of one B array of a chunk
constexpr int kWBChunk = 2 * kWBArr * 2;              // hi + lo of one chunk (32 KB)
constexpr int kWBBytes = kWKCB * kWBChunk;            // one block (128 KB)
constexpr int kWNBars = 2 * kWStages + 4 + 3;         // afull, aempty, tfull x2, tempty x2, bfull, bdone, drain
// roles: warps 0-7 epilogue (warp w drains accumulator buffer w / 4, quadrant
// w % 4), warp 8 MMA issue and block copies, warps 9-16 A producers
constexpr int kWMmaWarp = 8, kWProdWarp0 = 9;  // warps 0 .. kWMmaWarp - 1 are the epilogue
constexpr int kWThreads = 32 * (kWProdWarp0 + kProdWarps);  // 544
constexpr size_t kWSmem = (size_t)kWBBytes + (size_t)kWStages * kWAStage + 8 * kWNBars + 16;
static_assert(kWSmem <= 227 * 1024, "shared memory of the N = 256 form");

// a bounded wait whose outcome every lane of the warp shares
__device__ __forceinline__ bool ws_wait_warp(uint64_t *bar, uint32_t parity, long long limit, volatile int *abort_flag)
{
    const bool got = ws_wait(bar, parity, limit, abort_flag);
    return __all_sync(0xffffffffu, got);
}
}  // namespace umma

template <bool F16, bool POW2>
__global__ void __launch_bounds__(umma::kWThreads, 1) k_dft_tcgen05_w(WsArgs a)
{
    using namespace umma;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *sB = smem_raw;
    unsigned char *sA = smem_raw + kWBBytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw + kWBBytes + kWStages * kWAStage);
    uint64_t *afull = bars, *aempty = bars + kWStages, *tfull = bars + 2 * kWStages, *tempty = tfull + 2;
    uint64_t *bfull = tempty + 2, *bdone = bfull + 1, *drain = bdone + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + kWNBars);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < kWStages; ++s) {
            mbar_init(&afull[s], kProdThreads);
            mbar_init(&aempty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 32 * 4);  // the four warps of buffer b's epilogue group
        }
        mbar_init(bfull, 1);
        mbar_init(bdone, 1);
        mbar_init(drain, 1);
        *abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == kWMmaWarp) {
        tmem_alloc(tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    const int u0 = (int)((long long)a.nunits * blockIdx.x / gridDim.x);
    const int u1 = (int)((long long)a.nunits * (blockIdx.x + 1) / gridDim.x);
    const long long lim = a.wait_cycles;
    const int nparts = a.nnc * a.nkr;

    if (warp == kWMmaWarp) {
        if (lane == 0) {
            // ---------------------------------------------------------------- MMA issue
            int cur_blk = -1;
            uint32_t g = 0, nbf = 0, nbd = 0;
            bool b_pending = false;
            for (int i = u0; i < u1; ++i) {
                const WsUnit un = a.units[i];
                const int part = un.blk % nparts, nc = part / a.nkr, kr = part % a.nkr;
                const int Nc = min(kWN, a.D2p - kWN * nc);
                const int nkc = min(kWKCB, (a.D1p - kWKR * kr) / kKC);
                bool ok = true;
                if (un.blk != cur_blk) {
                    if (cur_blk >= 0) {
                        mma_commit(bdone);
                        if (!ws_wait(bdone, nbd & 1, lim, abort_flag)) break;
                        ++nbd;
                    }
                    mbar_expect_tx(bfull, (uint32_t)(nkc * kWBChunk));
                    const unsigned char *src = reinterpret_cast<const unsigned char *>(a.B) + (size_t)un.blk * kWBBytes;
                    for (int c = 0; c < nkc; ++c) bulk_g2s(sB + c * kWBChunk, src + (size_t)c * kWBChunk, kWBChunk, bfull);
                    b_pending = true;
                    if (!ws_wait(bfull, nbf & 1, lim, abort_flag)) break;
                    ++nbf;
                    b_pending = false;
                    cur_blk = un.blk;
                }
                const int li = i - u0, buf = li & 1;
                if (li >= 2 && !ws_wait(&tempty[buf], ((li >> 1) - 1) & 1, lim, abort_flag)) break;
                tc_fence_after();
                const uint32_t idesc = F16 ? idesc_f16(128, Nc) : idesc_bf16(128, Nc);
                const uint32_t dacc = tmem + (uint32_t)(buf * kWN);
                for (int kc = 0; kc < nkc; ++kc, ++g) {
                    const int s = (int)(g % kWStages);
                    if (!ws_wait(&afull[s], (g / kWStages) & 1, lim, abort_flag)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a_base = saddr(sA + s * kWAStage), b_base = saddr(sB + kc * kWBChunk);
#pragma unroll
                    for (int ks = 0; ks < 2; ++ks) {
                        const uint32_t ko = ks * 16 * 16;  // 16 k = two core matrices = 256 bytes
                        const uint64_t b_hi = sdesc(b_base + ko), b_lo = sdesc(b_base + kWBArr * 2 + ko);
                        const uint64_t a_hi = sdesc(a_base + ko), a_lo = sdesc(a_base + kWAArr * 2 + ko);
                        const uint32_t first = (kc == 0 && ks == 0) ? 0u : 1u;
                        mma_bf16(dacc, a_hi, b_hi, idesc, first);
                        mma_bf16(dacc, a_hi, b_lo, idesc, 1u);
                        mma_bf16(dacc, a_lo, b_hi, idesc, 1u);
                    }
                    mma_commit(&aempty[s]);
                }
                if (!ok) break;
                mma_commit(&tfull[buf]);
            }
            mma_commit(drain);
            mbar_wait(drain, 0);
            if (b_pending) mbar_wait(bfull, nbf & 1);
        }
    } else if (warp >= kWProdWarp0) {
        // -------------------------------------------------------------------- A producers
        const int qd = warp & 3, hh = (warp - kWProdWarp0) >> 2;
        const int row = 32 * qd + lane;
        const int pt = 16 * qd + (lane & 15), comp = lane >> 4;  // point of the tile; 0 = Re lane, 1 = Im lane
        const double inv1 = 1.0 / (double)a.n1;
        const int amin = -(a.D1 / 2);
        uint32_t g = 0;
        bool ok = true;
        for (int i = u0; i < u1 && ok; ++i) {
            const WsUnit un = a.units[i];
            const int kr = (un.blk % nparts) % a.nkr;
            const int nkc = min(kWKCB, (a.D1p - kWKR * kr) / kKC);
            const bool row_ok = pt < un.nj;
            const float uj = row_ok ? a.u[un.j0 + pt] : 0.f;
            const float2 w1 = phase_any<POW2>(1, uj, a.log2n1, inv1);
            const float2 w4 = phase_any<POW2>(4, uj, a.log2n1, inv1);
            const float2 w2 = cmulf(w1, w1), w8 = cmulf(w4, w4);
            const float2 w32 = cmulf(cmulf(w8, w8), cmulf(w8, w8));
            const f2x_t w2x = pk(w2.x, w2.x), w2y = pk(w2.y, w2.y), w2n = pk(-w2.y, -w2.y);
            const f2x_t w4x = pk(w4.x, w4.x), w4y = pk(w4.y, w4.y), w4n = pk(-w4.y, -w4.y);
            float2 anchor = make_float2(0.f, 0.f);
            for (int kc = 0; kc < nkc; ++kc, ++g) {
                const int s = (int)(g % kWStages);
                if (g >= (uint32_t)kWStages &&
                    !ws_wait_warp(&aempty[s], ((g / kWStages) - 1) & 1, lim, abort_flag)) {
                    ok = false;
                    break;
                }
                // this lane's 8 consecutive k: a = amin + 128 kr + 32 kc + 16 hh + 8 comp + 0..7,
                // as 4 packed pairs: pair 0 from the anchor (exact every 4 chunks, one
                // rotation by 32 from the previous chunk's otherwise), pair 2 rotated
                // from it by 4, pairs 1 and 3 from pairs 0 and 2 by 2
                if ((kc & 3) == 0)
                    anchor = row_ok ? phase_any<POW2>(amin + kWKR * kr + kKC * kc + 16 * hh + 8 * comp, uj, a.log2n1, inv1)
                                    : make_float2(0.f, 0.f);
                else
                    anchor = cmulf(anchor, w32);
                const float2 e1 = cmulf(anchor, w1);
                f2x_t X[4], Y[4];
                X[0] = pk(anchor.x, e1.x);
                Y[0] = pk(anchor.y, e1.y);
                X[2] = X[0]; Y[2] = Y[0]; rot_x2(X[2], Y[2], w4x, w4y, w4n);
                X[1] = X[0]; Y[1] = Y[0]; rot_x2(X[1], Y[1], w2x, w2y, w2n);
                X[3] = X[2]; Y[3] = Y[2]; rot_x2(X[3], Y[3], w2x, w2y, w2n);
                uint32_t hi[8], lo[8];
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    uint32_t rh, rl, ih, il;
                    split_x2<F16>(X[m], rh, rl);
                    split_x2<F16>(Y[m], ih, il);
                    // the Re lane keeps its real words and sends its imaginary ones to
                    // the Im lane (lane ^ 16), which sends its real words back
                    const uint32_t oh = comp ? ih : rh, ol = comp ? il : rl;
                    const uint32_t xh = __shfl_xor_sync(0xffffffffu, comp ? rh : ih, 16);
                    const uint32_t xl = __shfl_xor_sync(0xffffffffu, comp ? rl : il, 16);
                    hi[m] = comp ? xh : oh;
                    hi[4 + m] = comp ? oh : xh;
                    lo[m] = comp ? xl : ol;
                    lo[4 + m] = comp ? ol : xl;
                }
                uint16_t *As = reinterpret_cast<uint16_t *>(sA + s * kWAStage);
#pragma unroll
                for (int c8 = 0; c8 < 2; ++c8) {
                    const int idx = kmaj_index(row, 16 * hh + 8 * c8);  // one 16-byte core-matrix row
                    const int k0 = 4 * c8;
                    *reinterpret_cast<uint4 *>(As + idx) = make_uint4(hi[k0], hi[k0 + 1], hi[k0 + 2], hi[k0 + 3]);
                    *reinterpret_cast<uint4 *>(As + kWAArr + idx) = make_uint4(lo[k0], lo[k0 + 1], lo[k0 + 2], lo[k0 + 3]);
                }
                fence_proxy_async();  // the stores are visible to the tensor core
                mbar_arrive(&afull[s]);
            }
        }
    } else {
        // -------------------------------------------------------------------- epilogue
        const int qd = warp & 3, grp = warp >> 2;  // group grp drains buffer grp: units u0 + grp, + 2, ...
        const int pt = 16 * qd + (lane & 15), comp = lane >> 4;
        const double inv2 = 1.0 / (double)a.n2;
        const int bmin = -(a.D2 / 2);
        const uint32_t lane_base = (uint32_t)(32 * qd) << 16;
        for (int i = u0 + grp; i < u1; i += 2) {
            const WsUnit un = a.units[i];
            const int part = un.blk % nparts, nc = part / a.nkr;
            const int Nc = min(kWN, a.D2p - kWN * nc);
            const int li = i - u0, buf = li & 1;
            if (!ws_wait_warp(&tfull[buf], (li >> 1) & 1, lim, abort_flag)) break;
            tc_fence_after();
            const bool row_ok = pt < un.nj;
            const float vj = row_ok ? a.v[un.j0 + pt] : 0.f;
            const float2 v1 = phase_any<POW2>(1, vj, a.log2n2, inv2);
            const float2 v16 = phase_any<POW2>(16, vj, a.log2n2, inv2);
            const float2 v2 = cmulf(v1, v1);
            const f2x_t v2x = pk(v2.x, v2.x), v2y = pk(v2.y, v2.y), v2n = pk(-v2.y, -v2.y);
            const uint32_t cacc = tmem + lane_base + (uint32_t)(buf * kWN);
            float2 S = make_float2(0.f, 0.f), an = make_float2(0.f, 0.f);
            // S = sum_b q_b E_v(j, b) for this lane's real row q, in 16-column
            // groups: A(w^2) + w B(w^2) (even and odd columns, one packed chain)
            // times the group's anchor
            auto group = [&](const uint32_t(&q)[16], float2 anc) {
                f2x_t H = pk(__uint_as_float(q[14]), __uint_as_float(q[15]));
                f2x_t G = pk(0.f, 0.f);
#pragma unroll
                for (int t = 6; t >= 0; --t) {
                    const f2x_t qr = pk(__uint_as_float(q[2 * t]), __uint_as_float(q[2 * t + 1]));
                    const f2x_t h2 = fma_x2(H, v2x, fma_x2(G, v2n, qr));
                    G = fma_x2(H, v2y, mul_x2(G, v2x));
                    H = h2;
                }
                const float2 hr = upk(H), hi = upk(G);
                const float2 sB = cmulf(make_float2(hr.y, hi.y), v1);
                const float2 p = cmulf(make_float2(hr.x + sB.x, hi.x + sB.y), anc);
                S.x += p.x;
                S.y += p.y;
            };
            for (int c = 0; c < Nc; c += 32) {
                const bool two = c + 16 < Nc;  // warp-uniform
                uint32_t q0[16], q1[16];
                tmem_ld16(cacc + (uint32_t)c, q0);
                if (two) tmem_ld16(cacc + (uint32_t)(c + 16), q1);
                const float2 an0 = (c & 63) == 0 ? (row_ok ? phase_any<POW2>(bmin + kWN * nc + c, vj, a.log2n2, inv2)
                                                          : make_float2(0.f, 0.f))
                                                 : cmulf(an, v16);
                an = cmulf(an0, v16);
                tmem_wait_ld();
                group(q0, an0);
                if (two) group(q1, an);
            }
            tc_fence_before();
            mbar_arrive(&tempty[buf]);
            // F = S_re + i S_im: the Re lane takes the Im lane's sum
            const float ox = __shfl_xor_sync(0xffffffffu, S.x, 16), oy = __shfl_xor_sync(0xffffffffu, S.y, 16);
            if (comp == 0 && row_ok) {
                const float sc = a.inv_scale[un.proj];
                a.F[(size_t)part * a.ntot + un.j0 + pt] = make_float2((S.x - oy) * sc, (S.y + ox) * sc);
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0 && *abort_flag) atomicExch(a.err, 1);
    if (warp == kWMmaWarp) tmem_dealloc(tmem, 512);
}

// Per-projection power-of-two scales for FP16 operands: 2^(14 - e) with
// max|P| < 2^e, so that the largest scaled value is below 2^14; inv = 2^(e - 14).
__global__ void __launch_bounds__(256) k_proj_scale(const double *__restrict__ proj, long long per, float *scale,
                                                    float *inv_scale)
{
    const double *src = proj + (long long)blockIdx.x * per;
    float m = 0.f;
    for (long long i = threadIdx.x; i < per; i += 256) m = fmaxf(m, fabsf((float)src[i]));
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float wm[8];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; ++w) m = fmaxf(m, wm[w]);
        m = fmaxf(m, wm[0]);
        int e = 0;
        if (m > 0.f) frexpf(m, &e);
        const int sh = max(-100, min(100, 14 - e));
        scale[blockIdx.x] = m > 0.f ? ldexpf(1.f, sh) : 1.f;
        inv_scale[blockIdx.x] = m > 0.f ? ldexpf(1.f, -sh) : 1.f;
    }
}

// Pre-split (scaled) projections into hi/lo blocks in the B layout: block
// (p, nc, kr) holds columns b = NB nc + (0..NB-1) and rows a = KR kr + (0..KR-1)
// as KR / 32 K chunks of [hi | lo][NB x 32]; zero beyond D1 x D2.  NB x KR is
// 128 x 256 (first form) or 256 x 128 (second form), 128 KB either way.
// Grid: x = block, y = K chunk.
template <bool F16, int NB, int KR>
__global__ void __launch_bounds__(256) k_split_projections(const double *__restrict__ proj, int D1, int D2, int nnc,
                                                           int nkr, int mirror_m, const float *__restrict__ scale,
                                                           uint16_t *__restrict__ B)
{
    using namespace umma;
    constexpr int kArr = NB * kKC;                 // elements of one array of a chunk
    constexpr int kBlk = (KR / kKC) * 2 * kArr;    // elements of one block
    const int blk = blockIdx.x, kc = blockIdx.y;
    const int kr = blk % nkr, nc = (blk / nkr) % nnc, p = blk / (nkr * nnc);
    const double *src = proj + (long long)p * D1 * D2;
    const float sc = scale[p];
    uint16_t *dst = B + (size_t)blk * kBlk + (size_t)kc * (2 * kArr);
    for (int e = threadIdx.x; e < kArr; e += 256) {
        // e is the linear position in the layout: invert kmaj_index
        const int rg = e >> 8, kg = (e >> 6) & 3, rr = (e >> 3) & 7, kk = e & 7;
        // K row: natural (aa = a + D1/2), or with mirror_m = D1/2 the order
        // a = 0 .. m-1 then a = -1 .. -m (see WsArgs::mirror)
        const int kabs = kc * kKC + kg * 8 + kk;
        const int b = nc * NB + rg * 8 + rr;
        const int aa = mirror_m ? (kabs < mirror_m ? kabs + mirror_m : 2 * mirror_m - 1 - kabs) : kr * KR + kabs;
        // rows outside 0 .. D1-1 (the block's padding, in either order) are zero
        const float xf = (b < D2 && aa >= 0 && aa < D1) ? (float)src[aa + (long long)D1 * b] * sc : 0.f;
        if constexpr (F16) {
            const __half hi = __float2half_rn(xf);
            dst[e] = __half_as_ushort(hi);
            dst[kArr + e] = __half_as_ushort(__float2half_rn(xf - __half2float(hi)));
        } else {
            const __nv_bfloat16 hi = __float2bfloat16_rn(xf);
            dst[e] = __bfloat16_as_ushort(hi);
            dst[kArr + e] = __bfloat16_as_ushort(__float2bfloat16_rn(xf - __bfloat162float(hi)));
        }
    }
}

// F[j] = sum over the parts of partial F (in part order).
__global__ void k_sum_parts(const float2 *__restrict__ Fp, int nparts, long long ntot, float2 *__restrict__ F)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < ntot; j += (long long)gridDim.x * blockDim.x) {
        float2 s = Fp[j];
        for (int q = 1; q < nparts; ++q) {
            const float2 t = Fp[(size_t)q * ntot + j];
            s.x += t.x;
            s.y += t.y;
        }
        F[j] = s;
    }
}

// uoff[p] = units of the projections before p (uoff[P] = all units), from the
// points' offsets: a projection with nk points has ceil(nk / tp) tiles per
// block and nnc * nkr blocks.  One CTA of 1024 threads: a block scan per 1024
// projections with the running total carried.
__global__ void __launch_bounds__(1024) k_unit_offsets(const long long *__restrict__ off, int P, int tp, int per_tile,
                                                       long long *__restrict__ uoff)
{
    __shared__ long long wsum[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long carry = 0;
    if (threadIdx.x == 0) uoff[0] = 0;
    for (int base = 0; base < P; base += 1024) {
        const int p = base + threadIdx.x;
        const long long x = p < P ? (off[p + 1] - off[p] + tp - 1) / tp * per_tile : 0;
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
        if (p < P) uoff[p + 1] = carry + before + inc;
        carry += tot;
        __syncthreads();
    }
}

// The unit list, ordered by projection, block (nc, kr) and tile: unit u belongs
// to the last projection p with uoff[p] <= u (a projection without points has
// uoff[p] = uoff[p + 1] and is skipped by that rule).
__global__ void __launch_bounds__(256) k_make_units(const long long *__restrict__ off,
                                                    const long long *__restrict__ uoff, int P, int tp, int nnc,
                                                    int nkr, long long nunits, WsUnit *__restrict__ units)
{
    const long long u = blockIdx.x * 256LL + threadIdx.x;
    if (u >= nunits) return;
    int lo = 0, hi = P - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (uoff[mid] <= u) lo = mid;
        else hi = mid - 1;
    }
    const int p = lo;
    const long long nk = off[p + 1] - off[p];
    const long long tiles = (nk + tp - 1) / tp, local = u - uoff[p];
    const long long t = local % tiles, rest = local / tiles;
    const int kr = (int)(rest % nkr), nc = (int)(rest / nkr);
    units[u] = WsUnit{off[p] + t * tp, p, (p * nnc + nc) * nkr + kr, (int)min((long long)tp, nk - t * tp), 0};
}

__global__ void k_fill_f32(float *__restrict__ x, int n, float v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = v;
}

// The DFT kernels' dynamic shared memory is raised once per device and kernel.
static void ws_smem_attr(int device, const void *kern, size_t bytes)
{
    static std::mutex m;
    static std::set<std::pair<int, const void *>> done;
    std::lock_guard<std::mutex> g(m);
    if (done.count({device, kern})) return;
    GF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    done.insert({device, kern});
}

// Which tensor-core DFT: the first form (N = 128, 128-point tiles) by default;
// GENFIRE_DFT_KERNEL=n256 selects the second (Re and Im stacked in rows,
// N = 256, 64-point tiles).  On 256 x 256 projections (90 of them, 2.77 M
// points) the first takes 1.63 ms and the second 1.80 ms: the second's MMAs
// alone run in 1.15 ms against the first's 1.31 ms (fewer shared-memory bytes
// per MAC), but its K split (blocks of 128 rows) and row-wise Re/Im double the
// E_v contraction twice over.  The choice is a fixed rule, not a timing, so
// that a gridding call gives the same bits in every process (the two forms
// round differently).
static bool dft_use_wide()
{
    const char *e = std::getenv("GENFIRE_DFT_KERNEL");
    return e && std::strcmp(e, "n256") == 0;
}

// The first form's mirrored K order (WsArgs::mirror) where the shape allows it;
// GENFIRE_DFT_MIRROR=0 keeps the natural order.
static bool dft_mirror_enabled()
{
    const char *e = std::getenv("GENFIRE_DFT_MIRROR");
    return !(e && e[0] == '0');
}

// Host: F (float2, one per selected point) for all projections.  Everything is
// enqueued on the context stream without a host synchronisation: the unit list
// and the scales are made on the device, and the error flag is the caller's to
// read once it synchronises.
void dft_tcgen05(genfire_ctx *ctx, const double *d_proj, int D1, int D2, int n1, int n2, int P,
                 const std::vector<long long> &nk, const long long *d_off, const float *d_u, const float *d_v,
                 float2 *d_F, int *d_err, cudaEvent_t ev_begin, cudaEvent_t ev_end, bool fp16)
{
    using namespace umma;
    cudaStream_t st = ctx->stream;
    const bool wide = dft_use_wide();
    const int NB = wide ? kWN : kN, KR = wide ? kWKR : kKR;  // block shape
    const int D1p = (D1 + kKC - 1) / kKC * kKC, D2p = (D2 + 15) / 16 * 16;
    const int nnc = (D2p + NB - 1) / NB, nkr = (D1p + KR - 1) / KR;
    const int nparts = nnc * nkr;
    const int nblk = P * nnc * nkr;
    const int tp = wide ? kWPoints : kM;  // points per tile
    long long ntot = 0, nunits = 0;
    for (int p = 0; p < P; ++p) {
        ntot += nk[p];
        nunits += (nk[p] + tp - 1) / tp * nparts;
    }
    if (ntot == 0) return;
    if (nunits > INT32_MAX) fail(GENFIRE_ERR_ARG, "tensor-core gridding: too many selected points.");

    static_assert(kBBytes == kWBBytes, "both block shapes hold 128 KB");
    DevBuf B((size_t)nblk * kBBytes, st), scl(2 * sizeof(float) * P, st);
    float *d_scale = scl.as<float>(), *d_inv = d_scale + P;
    if (fp16) {
        k_proj_scale<<<P, 256, 0, st>>>(d_proj, (long long)D1 * D2, d_scale, d_inv);
    } else {
        k_fill_f32<<<(2 * P + 255) / 256, 256, 0, st>>>(d_scale, 2 * P, 1.f);
    }
    GF_CHECK_LAUNCH();
    // the mirrored K order of the first form: one K block of D1 = 64 H rows
    const int mirror = (!wide && D1 % 64 == 0 && D1 <= kKR && dft_mirror_enabled()) ? D1 / 64 : 0;
    const dim3 sgrid((unsigned)nblk, KR / kKC);
    uint16_t *dB = B.as<uint16_t>();
    if (wide) {
        if (fp16) k_split_projections<true, kWN, kWKR><<<sgrid, 256, 0, st>>>(d_proj, D1, D2, nnc, nkr, 0, d_scale, dB);
        else k_split_projections<false, kWN, kWKR><<<sgrid, 256, 0, st>>>(d_proj, D1, D2, nnc, nkr, 0, d_scale, dB);
    } else {
        const int mm = mirror ? D1 / 2 : 0;
        if (fp16) k_split_projections<true, kN, kKR><<<sgrid, 256, 0, st>>>(d_proj, D1, D2, nnc, nkr, mm, d_scale, dB);
        else k_split_projections<false, kN, kKR><<<sgrid, 256, 0, st>>>(d_proj, D1, D2, nnc, nkr, mm, d_scale, dB);
    }
    GF_CHECK_LAUNCH();

    DevBuf du(sizeof(WsUnit) * (size_t)nunits, st), duoff(sizeof(long long) * (P + 1), st);
    k_unit_offsets<<<1, 1024, 0, st>>>(d_off, P, tp, nparts, duoff.as<long long>());
    GF_CHECK_LAUNCH();
    k_make_units<<<(unsigned)((nunits + 255) / 256), 256, 0, st>>>(d_off, duoff.as<long long>(), P, tp, nnc, nkr,
                                                                   nunits, du.as<WsUnit>());
    GF_CHECK_LAUNCH();
    DevBuf Fp(nparts > 1 ? sizeof(float2) * (size_t)nparts * ntot : 0, st);
    WsArgs a;
    a.B = B.as<uint16_t>();
    a.units = du.as<WsUnit>();
    a.nunits = (int)nunits;
    a.u = d_u;
    a.v = d_v;
    a.inv_scale = d_inv;
    a.F = nparts > 1 ? Fp.as<float2>() : d_F;
    a.ntot = ntot;
    a.D1 = D1; a.D2 = D2; a.D1p = D1p; a.D2p = D2p;
    a.n1 = n1; a.n2 = n2;
    auto lg = [](int n) { int t = 0; while ((1 << t) < n) ++t; return (1 << t) == n ? t : -1; };
    a.log2n1 = lg(n1); a.log2n2 = lg(n2);
    a.nnc = nnc; a.nkr = nkr;
    a.mirror = mirror;
    a.err = d_err;
    // GENFIRE_DEBUG_DFT_WAIT_CYCLES (a positive count of clock cycles) shortens
    // the pipeline's waits so that a test can make one expire and exercise the
    // kernel's error path on real work: the drain still waits with the full
    // limit for the copies and MMAs in flight, so the call returns
    // GENFIRE_ERR_TIMEOUT with the context intact.
    a.wait_cycles = kWaitCycles;
    if (const char *dbg = std::getenv("GENFIRE_DEBUG_DFT_WAIT_CYCLES")) {
        const long long v = std::atoll(dbg);
        if (v > 0 && v < kWaitCycles) a.wait_cycles = v;
    }
    const bool pow2 = a.log2n1 >= 0 && a.log2n2 >= 0;
    const void *kern;
    if (wide)
        kern = fp16 ? (pow2 ? (const void *)k_dft_tcgen05_w<true, true> : (const void *)k_dft_tcgen05_w<true, false>)
                    : (pow2 ? (const void *)k_dft_tcgen05_w<false, true> : (const void *)k_dft_tcgen05_w<false, false>);
    else
        kern = fp16 ? (pow2 ? (const void *)k_dft_tcgen05<true, true> : (const void *)k_dft_tcgen05<true, false>)
                    : (pow2 ? (const void *)k_dft_tcgen05<false, true> : (const void *)k_dft_tcgen05<false, false>);
    const size_t smem = wide ? kWSmem : kWsSmem;
    ws_smem_attr(ctx->device, kern, smem);
    const int grid = (int)std::min<long long>(nunits, (long long)ctx->sm_count);
    if (ev_begin) GF_CUDA(cudaEventRecord(ev_begin, st));
    void *args[] = {&a};
    GF_CUDA(cudaLaunchKernel(kern, dim3((unsigned)grid), dim3(wide ? kWThreads : kWsThreads), args, smem, st));
    GF_CHECK_LAUNCH();
    if (ev_end) GF_CUDA(cudaEventRecord(ev_end, st));
    if (nparts > 1) {
        k_sum_parts<<<(unsigned)std::min<long long>((ntot + 255) / 256, 16LL * ctx->sm_count), 256, 0, st>>>(
            Fp.as<float2>(), nparts, ntot, d_F);
        GF_CHECK_LAUNCH();
    }
    // the buffers are released stream-ordered (cudaFreeAsync) after the kernels
}

}  // namespace gf
