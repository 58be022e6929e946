// dr.cu -- the Fourier-constraint iteration of reconstruct.m on the GPU, the
// recIFFT of the gridding, and the test-facing 3-D FFT.
//
// One iteration (reconstruct.m:117-186) is five FFT passes (five launches; the
// loop's control updates run inside CTA 0 of F1 and I2), captured once as a
// CUDA graph:
//   F1         rows along dim 1: positivity and support, real -> half spectrum;
//              its CTA 0 also starts the iteration (iteration count,
//              constraint change points, bestErr reset)
//   F2         dim 2 forward
//   F3         dim 3 forward, errK terms, Fourier constraint, dim 3 inverse
//   I2         dim 2 inverse; its CTA 0 first forms errK = sum / sum|M| from
//              F3's partials and does the best-object bookkeeping (which
//              buffer the next object goes to, read by I1)
//   I1         rows along dim 1: half spectrum -> real
// The object is held only on its "box": the Dim1 x Dim2 x Dim1 region the
// support can be non-zero on (the whole n1 x n2 x n1 grid when the support
// constraint is off).  Everything outside the box is multiplied by zero at
// the next iteration and never observed (the result and the R-factor read
// the same centred box), so the forward passes skip the zero rows and the
// inverse passes only produce the box.
#include <cub/cub.cuh>
#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled_v12000

#include "fft.cuh"
#include "fft_reg.cuh"
#include "fft_r32.cuh"
#include "internal.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <tuple>

namespace gf {

// ===========================================================================
// twiddle tables, one per (device, n, precision), kept for the process: the
// n entries exp(-2 pi i t / n), then (power-of-two n) the packed per-stage
// table of the register-resident passes (P2Plan::twoff), copied from them,
// then (n = 128 .. 1024) the radix-32 engines' table W_n^(t k1) ordered by k1
// then t (R32<n>::TWT)
// ===========================================================================
template <typename T> const cplx<T> *twiddles(int n, cudaStream_t s)
{
    static std::mutex mu;
    static std::map<std::tuple<int, int, int>, void *> cache;
    int dev = 0;
    GF_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_tuple(dev, n, (int)sizeof(T));
    auto it = cache.find(key);
    if (it != cache.end()) return static_cast<const cplx<T> *>(it->second);
    const int np = packed_twiddle_count(n);
    const bool r32 = n == 128 || n == 256 || n == 512 || n == 1024;
    const int nr = r32 ? 32 * (n / 32) : 0;  // radix-32 table: k1 < 32, t < n / 32
    std::vector<cplx<T>> h((size_t)n + np + nr);
    const double pi = 3.14159265358979323846;
    for (int t = 0; t < n; ++t) {
        double a = -2.0 * pi * (double)t / (double)n;
        h[t] = mk((T)std::cos(a), (T)std::sin(a));
    }
    if (np) {
        // the packed table of length m = packed_length(n): W_m^x = W_n^(x * n / m)
        const int m = packed_length(n), f = n / m;
        int L = 0;
        while ((1 << L) < m) ++L;
        const int n8 = L / 3, rem = L % 3, nst = n8 + (rem ? 1 : 0);
        size_t o = (size_t)n;
        for (int st = 0, ns = 1; st < nst; ns *= (st < n8 ? 8 : (rem == 2 ? 4 : 2)), ++st) {
            const int R = st < n8 ? 8 : (rem == 2 ? 4 : 2);
            if (ns == 1) continue;
            const int step = m / (ns * R);
            for (int kk = 0; kk < ns; ++kk) {
                for (int r = 1; r < R; ++r) h[o++] = h[(size_t)kk * r * step * f];
                h[o++] = mk((T)1, (T)0);  // pad
            }
        }
        if (o != (size_t)n + np) fail(GENFIRE_ERR_STATE, "internal: packed twiddle table size.");
    }
    if (nr) {
        const int P = n / 32;
        const size_t o = (size_t)(n == 128 ? R32<128>::TWT : n == 256 ? R32<256>::TWT
                                  : n == 512 ? R32<512>::TWT : R32<1024>::TWT);
        if (o != (size_t)n + np) fail(GENFIRE_ERR_STATE, "internal: radix-32 twiddle table offset.");
        for (int k1 = 0; k1 < 32; ++k1)
            for (int t = 0; t < P; ++t) h[o + (size_t)k1 * P + t] = h[(size_t)t * k1];
    }
    void *d = nullptr;
    GF_CUDA(cudaMalloc(&d, sizeof(cplx<T>) * h.size()));
    GF_CUDA(cudaMemcpyAsync(d, h.data(), sizeof(cplx<T>) * h.size(), cudaMemcpyHostToDevice, s));
    GF_CUDA(cudaStreamSynchronize(s));
    cache[key] = d;
    return static_cast<const cplx<T> *>(d);
}
template const float2 *twiddles<float>(int, cudaStream_t);
template const double2 *twiddles<double>(int, cudaStream_t);

static FftPlan plan_or_fail(int n)
{
    FftPlan pl;
    if (!make_fft_plan(n, pl))
        fail(GENFIRE_ERR_UNSUPPORTED,
             "FFT length " + std::to_string(n) + " has a prime factor above 7 (choose Dim*oversamplingRatio "
             "with factors 2, 3, 5 and 7).");
    return pl;
}

template <typename T, int N> static void set_reg_attrs()
{
    const int sm = (int)reg_smem<T, N>();
    GF_CUDA(cudaFuncSetAttribute((const void *)k_col_reg<T, N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    if constexpr (sizeof(T) == 4)
        GF_CUDA(cudaFuncSetAttribute((const void *)k_col_reg<T, N, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    GF_CUDA(cudaFuncSetAttribute((const void *)k_row_r2c_reg<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    GF_CUDA(cudaFuncSetAttribute((const void *)k_row_c2r_reg<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
}

// Launch variants of a column pass: the generic shared-memory engine, the
// register-resident engine with one column per thread, or with two adjacent
// float columns per thread (unit column stride and 16-byte aligned column
// pairs: even strides, aligned bases; tiles start at even columns), the
// mixed-radix engine, the radix-32 engines for 512 and 1024 complex64 points
// (fft_r32.cuh: 32 x 16 and 32 x 32, one exchange per transform), and for the
// fused 512-point pass the persistent radix-32 pass fed by TMA tensor copies
// (measured 6 % slower than variant 4 on the 512^3 iteration; an autotuner
// candidate).
enum ColVariant { kColAuto = -1, kColGeneric = 0, kColReg1 = 1, kColReg2 = 2, kColMix = 3, kColR32 = 4, kColR32Tma = 5 };

// GENFIRE_COL_VARIANT=<v> forces variant v wherever it is valid (tuning and
// tests); unset, the built-in choice or the autotuner decides
static int forced_col_variant()
{
    const char *e = std::getenv("GENFIRE_COL_VARIANT");
    return (e && *e) ? std::atoi(e) : kColAuto;
}

template <typename T> static bool pair_capable(const ColPassArgs<T> &a)
{
    auto al = [](const void *p) { return ((uintptr_t)p & 15u) == 0; };
    return sizeof(T) == 4 && a.col_stride == 1 && al(a.in) && al(a.out) && a.in_dim % 2 == 0 &&
           a.in_other % 2 == 0 && a.out_dim % 2 == 0 && a.out_other % 2 == 0;
}

// Register-resident passes for power-of-two lengths 64..1024.
template <typename T, int N> static void col_reg(const ColPassArgs<T> &a, int other, cudaStream_t st, int nc)
{
    constexpr int W = reg_width<T>(N);
    if (a.W != W) fail(GENFIRE_ERR_STATE, "internal: column tile width mismatch.");
    dim3 grid(cdiv(a.ncols, W), other);
    if constexpr (sizeof(T) == 4) {
        if (nc == 2) {
            k_col_reg<T, N, 2><<<grid, col_threads<T, N, 2>(), reg_smem<T, N>(), st>>>(a);
            return;
        }
    }
    k_col_reg<T, N, 1><<<grid, col_threads<T, N, 1>(), reg_smem<T, N>(), st>>>(a);
}
template <typename T, int N> static void rows_reg(const RowPassArgs<T> &a, bool forward, cudaStream_t st)
{
    constexpr int W = reg_width<T>(N);
    if (a.W != W) fail(GENFIRE_ERR_STATE, "internal: row tile width mismatch.");
    dim3 grid(cdiv((a.nrows + 1) / 2, W));
    if (forward) k_row_r2c_reg<T, N><<<grid, N / 8 * W, reg_smem<T, N>(), st>>>(a);
    else k_row_c2r_reg<T, N><<<grid, N / 8 * W, reg_smem<T, N>(), st>>>(a);
}
// element offsets along the transform are 32-bit in the register passes
template <typename T> static bool span_ok(const ColPassArgs<T> &a)
{
    return (long long)(a.pl.n - 1) * std::max(a.in_dim, a.out_dim) + 1 < (1LL << 32);
}
template <typename T> static bool reg_capable(const ColPassArgs<T> &a)
{
    const int n = a.pl.n;
    return span_ok(a) && (n == 64 || n == 128 || n == 256 || n == 512 || n == 1024);
}
template <typename T> static void col_reg_any(const ColPassArgs<T> &a, int other, cudaStream_t st, int nc)
{
    switch (a.pl.n) {
    case 64: col_reg<T, 64>(a, other, st, nc); break;
    case 128: col_reg<T, 128>(a, other, st, nc); break;
    case 256: col_reg<T, 256>(a, other, st, nc); break;
    case 512: col_reg<T, 512>(a, other, st, nc); break;
    default: col_reg<T, 1024>(a, other, st, nc); break;
    }
}
template <typename T> static bool try_rows_reg(const RowPassArgs<T> &a, bool forward, cudaStream_t st)
{
    switch (a.pl.n) {
    case 64: rows_reg<T, 64>(a, forward, st); return true;
    case 128: rows_reg<T, 128>(a, forward, st); return true;
    case 256: rows_reg<T, 256>(a, forward, st); return true;
    case 512: rows_reg<T, 512>(a, forward, st); return true;
    case 1024: rows_reg<T, 1024>(a, forward, st); return true;
    default: return false;
    }
}

// Opt every FFT pass kernel into large dynamic shared memory once per device
// (before any graph capture; the attribute only raises the limit).
template <typename T> static void ensure_smem_attrs()
{
    static std::mutex mu;
    static std::set<int> done;
    int dev = 0;
    GF_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (done.count(dev)) return;
    const int lim = 200 * 1024;
    GF_CUDA(cudaFuncSetAttribute((const void *)k_colpass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    GF_CUDA(cudaFuncSetAttribute((const void *)k_rows_r2c<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    GF_CUDA(cudaFuncSetAttribute((const void *)k_rows_c2r<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim));
    set_reg_attrs<T, 64>();
    set_reg_attrs<T, 128>();
    set_reg_attrs<T, 256>();
    set_reg_attrs<T, 512>();
    set_reg_attrs<T, 1024>();
    if constexpr (sizeof(T) == 4) {
        // the persistent fused pass: 53 KB per CTA, 4 CTAs per SM
        GF_CUDA(cudaFuncSetAttribute((const void *)k_col_r32_tma<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)r32_tma_smem<512>()));
        GF_CUDA(cudaFuncSetAttribute((const void *)k_col_r32_tma<512>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    }

    done.insert(dev);
}

// columns per CTA of the radix-32 engine for length n, 0 when it has none
static int r32_width(int n)
{
    switch (n) {
    case 128: return R32<128>::W;
    case 256: return R32<256>::W;
    case 512: return R32<512>::W;
    case 1024: return R32<1024>::W;
    default: return 0;
    }
}

// The driver's tensor-map encoder (cuTensorMapEncodeTiled), through the
// runtime's entry-point query so the library needs no link to libcuda.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

static int device_sm_count()
{
    static std::mutex mu;
    static std::map<int, int> cache;
    int dev = 0;
    GF_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    int n = 0;
    GF_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    cache[dev] = n;
    return n;
}

// The persistent, TMA-fed fused 512-point pass (k_col_r32_tma): complex64, the
// centred half of a box in and out, unit column stride, tiles inside the rows
// of the input, strides that a tensor map can describe.
template <typename T> static bool tma_capable(const ColPassArgs<T> &a, int other)
{
    if constexpr (sizeof(T) != 4) {
        return false;
    } else {
        constexpr int N = 512, W = R32<N>::W;
        if (a.pl.n != N || !(a.mode & 1) || !(a.mode & 2) || a.col_stride != 1 || a.W != W) return false;
        if (!(a.in_cnt == N / 2 && a.in_c == N / 4 && a.out_cnt == N / 2 && a.out_c == N / 4)) return false;
        if (((uintptr_t)a.in & 15u) != 0 || a.in_other <= 0 || a.in_dim % a.in_other != 0) return false;
        if ((a.in_other * 8) % 16 != 0 || (a.in_dim * 8) % 16 != 0) return false;
        if ((long long)cdiv(a.ncols, W) * W > a.in_other || other > a.in_dim / a.in_other) return false;
        return span_ok(a) && tensor_map_encoder() != nullptr;
    }
}

template <typename T> static bool col_variant_ok(const ColPassArgs<T> &a, int v, int other = 1)
{
    if (v == kColGeneric) return true;
    if (v == kColR32Tma) return tma_capable(a, other);
    if (v == kColR32)
        return sizeof(T) == 4 && r32_width(a.pl.n) > 0 && span_ok(a) && (!(a.mode & 4) || a.W == r32_width(a.pl.n));
    if (v == kColMix) return span_ok(a) && mix_capable<T>(a.pl.n);
    if (!reg_capable(a)) return false;
    return v == kColReg1 || (v == kColReg2 && pair_capable(a));
}

// Column pass launcher.  Without a tuned variant: the radix-32 engines for
// 512 and 1024 complex64 points (one exchange per transform: 8-28 % faster
// than the radix-8 engine on the three column passes at 512^3); otherwise, for
// powers of two, two columns per thread in the fused forward + constraint +
// inverse pass (two transforms per load) and one column per thread in the
// single-transform passes (twice the resident warps); the mixed-radix
// register engine for 3 or 5 times a power of two; the generic engine for
// other lengths.
template <typename T> static int default_col_variant(const ColPassArgs<T> &a)
{
    // below 512 points the radix-32 engine is a candidate of the autotuner, not
    // the built-in choice (at 256 points it took the 128^3 workload from 11.4 k
    // to 12.8 k iterations/s; as the default it cost the batched problems 1.5 %)
    if (a.pl.n >= 512 && col_variant_ok(a, kColR32)) return kColR32;
    if (reg_capable(a)) return ((a.mode & 3) == 3 && pair_capable(a)) ? kColReg2 : kColReg1;
    if (col_variant_ok(a, kColMix)) return kColMix;
    return kColGeneric;
}

// The radix-32 engines (128 to 1024 complex64 points), with compile-time
// pruning when the pass reads / writes the centred half of a box.  Input
// pruning only with output pruning (the fused dim-3 pass): the forward-only
// 512-point variant with it takes 128 registers and measured 3 % slower.
template <typename T, int N> static void col_r32(const ColPassArgs<T> &a, int other, cudaStream_t st)
{
    using G = R32<N>;
    const bool zin = (a.mode & 1) && a.in_cnt == N / 2 && a.in_c == N / 4;
    const bool zout = a.out_cnt == N / 2 && a.out_c == N / 4;
    const dim3 grid(cdiv(a.ncols, G::W), other);
    const size_t sm = G::template smem<T>();
    if (zin && zout) k_col_r32<T, N, true, true><<<grid, G::THREADS, sm, st>>>(a);
    else if (zout) k_col_r32<T, N, false, true><<<grid, G::THREADS, sm, st>>>(a);
    else k_col_r32<T, N, false, false><<<grid, G::THREADS, sm, st>>>(a);
}
// Launch of k_col_r32_tma: the input as a float tensor {2 in_other, in_dim /
// in_other, in_cnt} (strides in_other and in_dim complex values), boxes of
// {2 W, 1, N/2}; a persistent grid of 4 CTAs per SM.
static void col_r32_tma(const ColPassArgs<float> &a, int other, cudaStream_t st)
{
    constexpr int N = 512;
    using G = R32<N>;
    CUtensorMap map;
    const cuuint64_t dims[3] = {(cuuint64_t)(2 * a.in_other), (cuuint64_t)(a.in_dim / a.in_other), (cuuint64_t)a.in_cnt};
    const cuuint64_t strides[2] = {(cuuint64_t)(a.in_other * 8), (cuuint64_t)(a.in_dim * 8)};
    const cuuint32_t box[3] = {2 * G::W, 1, N / 2};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<cplx<float> *>(a.in), dims,
                                            strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(GENFIRE_ERR_CUDA, "tensor map of the fused column pass could not be encoded.");
    const int tiles_x = (int)cdiv(a.ncols, G::W), ntiles = tiles_x * other;
    const int grid = std::min(ntiles, 4 * device_sm_count());
    k_col_r32_tma<N><<<grid, G::THREADS, r32_tma_smem<N>(), st>>>(a, map, tiles_x, ntiles);
}

template <typename T, int N> static void rows_r32(const RowPassArgs<T> &a, bool forward, cudaStream_t st)
{
    using G = R32<N>;
    const dim3 grid(cdiv((a.nrows + 1) / 2, G::W));
    const size_t sm = G::template smem<T>();
    const bool half = a.B1 == N / 2 && a.c1 == N / 4;  // the centred half of the row
    if (forward) {
        if (half) k_row_r2c_r32<T, N, true><<<grid, G::THREADS, sm, st>>>(a);
        else k_row_r2c_r32<T, N, false><<<grid, G::THREADS, sm, st>>>(a);
    } else {
        if (half) k_row_c2r_r32<T, N, true><<<grid, G::THREADS, sm, st>>>(a);
        else k_row_c2r_r32<T, N, false><<<grid, G::THREADS, sm, st>>>(a);
    }
}

template <typename T> static void launch_colpass(ColPassArgs<T> a, int other, cudaStream_t st, int variant = kColAuto)
{
    a.P = a.W + 1;
    const int forced = forced_col_variant();
    if (forced != kColAuto && col_variant_ok(a, forced, other)) variant = forced;
    if (variant == kColAuto || !col_variant_ok(a, variant, other)) variant = default_col_variant(a);
    if (variant == kColR32Tma) {
        if constexpr (sizeof(T) == 4) col_r32_tma(a, other, st);
    } else if (variant == kColR32) {
        if constexpr (sizeof(T) == 4) {
            switch (a.pl.n) {
            case 128: col_r32<T, 128>(a, other, st); break;
            case 256: col_r32<T, 256>(a, other, st); break;
            case 512: col_r32<T, 512>(a, other, st); break;
            default: col_r32<T, 1024>(a, other, st); break;
            }
        }
    } else if (variant == kColMix) {
        if (!launch_col_mix<T>(a, other, st)) fail(GENFIRE_ERR_STATE, "internal: mixed-radix pass not available.");
    } else if (variant == kColGeneric) {
        const size_t sm = tile_smem<T>(a.pl.n, a.W);
        dim3 grid(cdiv(a.ncols, a.W), other);
        k_colpass<T><<<grid, tile_threads(a.pl.n, a.W), sm, st>>>(a);
    } else {
        col_reg_any<T>(a, other, st, variant == kColReg2 ? 2 : 1);
    }
    GF_CHECK_LAUNCH();
}

// Autotuner of the column passes: every valid variant is timed on the
// caller's own buffers (one warm-up launch, then the mean of 3 launches
// bracketed by CUDA events) and the fastest is kept for the process, keyed by
// the device, the precision and the pass geometry.  Runs at setup, outside
// any stream capture; the timed launches only write the pass's output buffer
// and its errK partials, which the first real iteration overwrites.
template <typename T> static int autotune_colpass(ColPassArgs<T> a, int other, cudaStream_t st)
{
    static std::mutex mu;
    static std::map<std::vector<long long>, int> cache;
    ensure_smem_attrs<T>();
    {
        const int f = forced_col_variant();
        if (f != kColAuto && col_variant_ok(a, f, other)) return f;
    }
    int dev = 0;
    GF_CUDA(cudaGetDevice(&dev));
    const std::vector<long long> key = {dev, (long long)sizeof(T), a.pl.n, a.mode, a.ncols, other, a.in_cnt,
                                        a.in_c, a.out_cnt, a.out_c, a.in_dim, a.in_other, a.out_dim, a.out_other};
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    cudaEvent_t e0, e1;
    GF_CUDA(cudaEventCreate(&e0));
    GF_CUDA(cudaEventCreate(&e1));
    // the built-in choice stays unless another variant is more than 3 % faster
    // (keeps the choice stable against timing noise)
    int best = kColAuto;
    float best_ms = 0, default_ms = -1;
    for (int v : {kColGeneric, kColReg1, kColReg2, kColMix, kColR32, kColR32Tma}) {
        if (!col_variant_ok(a, v, other)) continue;
        launch_colpass<T>(a, other, st, v);
        GF_CUDA(cudaEventRecord(e0, st));
        for (int r = 0; r < 3; ++r) launch_colpass<T>(a, other, st, v);
        GF_CUDA(cudaEventRecord(e1, st));
        GF_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        GF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (v == default_col_variant(a)) default_ms = ms;
        if (best == kColAuto || ms < best_ms) { best = v; best_ms = ms; }
    }
    if (default_ms >= 0 && best_ms > 0.97f * default_ms) best = default_col_variant(a);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = best;
    return best;
}

// Row passes of 512 and 1024 complex64 points run on the radix-32 engines
// (GENFIRE_ROW_VARIANT=1 selects the radix-8 register engine instead).
static bool rows_r32_enabled()
{
    const char *e = std::getenv("GENFIRE_ROW_VARIANT");
    return !(e && e[0] == '1');
}

template <typename T> static void launch_rows(RowPassArgs<T> a, bool forward, cudaStream_t st)
{
    a.P = a.W + 1;
    if constexpr (sizeof(T) == 4) {
        if ((a.pl.n == 512 || a.pl.n == 1024) && rows_r32_enabled()) {
            if (a.pl.n == 512) rows_r32<T, 512>(a, forward, st);
            else rows_r32<T, 1024>(a, forward, st);
            GF_CHECK_LAUNCH();
            return;
        }
    }
    if (!try_rows_reg<T>(a, forward, st) && !launch_rows_mix<T>(a, forward, st)) {
        const size_t sm = tile_smem<T>(a.pl.n, a.W);
        const int pairs = (a.nrows + 1) / 2;
        dim3 grid(cdiv(pairs, a.W));
        if (forward) k_rows_r2c<T><<<grid, tile_threads(a.pl.n, a.W), sm, st>>>(a);
        else k_rows_c2r<T><<<grid, tile_threads(a.pl.n, a.W), sm, st>>>(a);
    }
    GF_CHECK_LAUNCH();
}

// ===========================================================================
// half spectrum of the Hermitian part of a centred grid:
// H(q) = (M(q) + conj(M(-q))) / 2 for q1 in [0, h1), FFT order
// ===========================================================================
template <typename T>
__global__ void k_half_from_centered(const cplx<T> *__restrict__ M, int n1, int n2, int h1, int ld1,
                                     cplx<T> *__restrict__ H)
{
    // grid: x over q1, y = q2, z = q3
    const int q2 = blockIdx.y, q3 = blockIdx.z;
    const int m2 = (n2 - q2) % n2, m3 = (n1 - q3) % n1;
    const long long ra = (long long)n1 * (((q2 + n2 / 2) % n2) + (long long)n2 * ((q3 + n1 / 2) % n1));
    const long long rb = (long long)n1 * (((m2 + n2 / 2) % n2) + (long long)n2 * ((m3 + n1 / 2) % n1));
    for (int q1 = blockIdx.x * blockDim.x + threadIdx.x; q1 < h1; q1 += gridDim.x * blockDim.x) {
        const int m1 = (n1 - q1) % n1;
        const cplx<T> x = M[ra + (q1 + n1 / 2) % n1], y = M[rb + (m1 + n1 / 2) % n1];
        H[q1 + (long long)ld1 * (q2 + (long long)n2 * q3)] = mk((T)0.5 * (x.x + y.x), (T)0.5 * (x.y - y.y));
    }
}

static int round_up(int a, int b) { return (a + b - 1) / b * b; }

// inverse chain: half spectrum Hs (ld1 x n2 x n1) -> real box B1 x B2 x B3
template <typename T> struct InvChain {
    int n1, n2, h1, ld1, B1, B2, B3;
    FftPlan pl1, pl2, pl3;
    const cplx<T> *tw1, *tw2, *tw3;
    int W1, W2, W3;
};

template <typename T> static InvChain<T> make_chain(int n1, int n2, int B1, int B2, int B3, cudaStream_t st)
{
    InvChain<T> c;
    c.n1 = n1; c.n2 = n2; c.h1 = n1 / 2 + 1; c.ld1 = round_up(c.h1, 8);
    c.B1 = B1; c.B2 = B2; c.B3 = B3;
    c.pl1 = plan_or_fail(n1); c.pl2 = plan_or_fail(n2); c.pl3 = c.pl1;
    c.tw1 = twiddles<T>(n1, st); c.tw2 = twiddles<T>(n2, st); c.tw3 = c.tw1;
    c.W1 = tile_width<T>(n1); c.W2 = tile_width<T>(n2); c.W3 = c.W1;
    return c;
}

template <typename T> static ColPassArgs<T> colargs(const FftPlan &pl, const cplx<T> *tw, int W, int ncols)
{
    ColPassArgs<T> a;
    std::memset(&a, 0, sizeof(a));
    a.pl = pl; a.tw = tw; a.W = W; a.ncols = ncols; a.col_stride = 1; a.scale = (T)1;
    return a;
}

template <typename T>
static void rec_ifft_t(genfire_ctx *ctx, const cplx<T> *d_M, int n1, int n2, int D1, int D2, T *d_rec)
{
    cudaStream_t st = ctx->stream;
    ensure_smem_attrs<T>();
    InvChain<T> c = make_chain<T>(n1, n2, D1, D2, D1, st);
    DevBuf H(sizeof(cplx<T>) * (size_t)c.ld1 * n2 * n1, st);
    DevBuf Y(sizeof(cplx<T>) * (size_t)c.ld1 * n2 * D1, st);
    DevBuf Z(sizeof(cplx<T>) * (size_t)c.ld1 * D2 * D1, st);
    k_half_from_centered<T><<<dim3(cdiv(c.h1, 256), n2, n1), 256, 0, st>>>(d_M, n1, n2, c.h1, c.ld1, H.as<cplx<T>>());
    GF_CHECK_LAUNCH();
    // dim 3 inverse: all n1 entries in, the D1 box entries out
    ColPassArgs<T> a = colargs<T>(c.pl3, c.tw3, c.W3, c.h1);
    a.in = H.as<cplx<T>>(); a.in_dim = (long long)c.ld1 * n2; a.in_other = c.ld1; a.in_cnt = n1; a.in_c = 0;
    a.out = Y.as<cplx<T>>(); a.out_dim = (long long)c.ld1 * n2; a.out_other = c.ld1; a.out_cnt = D1; a.out_c = D1 / 2;
    a.mode = 2;
    launch_colpass<T>(a, n2, st);
    // dim 2 inverse
    ColPassArgs<T> b = colargs<T>(c.pl2, c.tw2, c.W2, c.h1);
    b.in = Y.as<cplx<T>>(); b.in_dim = c.ld1; b.in_other = (long long)c.ld1 * n2; b.in_cnt = n2; b.in_c = 0;
    b.out = Z.as<cplx<T>>(); b.out_dim = c.ld1; b.out_other = (long long)c.ld1 * D2; b.out_cnt = D2; b.out_c = D2 / 2;
    b.mode = 2;
    launch_colpass<T>(b, D1, st);
    // dim 1 C2R
    RowPassArgs<T> r;
    std::memset(&r, 0, sizeof(r));
    r.pl = c.pl1; r.tw = c.tw1; r.W = c.W1; r.nrows = D2 * D1; r.B1 = D1; r.c1 = D1 / 2; r.h1 = c.h1; r.ld1 = c.ld1;
    r.xs[0] = d_rec; r.xsel = nullptr; r.Y = Z.as<cplx<T>>();
    r.scale = (T)(1.0 / ((double)n1 * n2 * n1));
    launch_rows<T>(r, false, st);
}

void rec_ifft(genfire_ctx *ctx, int precision, const void *d_M, int n1, int n2, int D1, int D2, void *d_rec)
{
    if (precision == GENFIRE_PREC_FP64)
        rec_ifft_t<double>(ctx, (const double2 *)d_M, n1, n2, D1, D2, (double *)d_rec);
    else
        rec_ifft_t<float>(ctx, (const float2 *)d_M, n1, n2, D1, D2, (float *)d_rec);
}

// ===========================================================================
// plain 3-D FFT (fftn / ifftn) on a full complex array, along the dimensions
// set in axes (bit 0 = dim 1, ...); the inverse scales by 1 / (product of the
// transformed lengths)
// ===========================================================================
template <typename T>
static void fftn_t(genfire_ctx *ctx, cplx<T> *d, int n1, int n2, int n3, bool inv, int axes = 7)
{
    cudaStream_t st = ctx->stream;
    ensure_smem_attrs<T>();
    const int dims[3] = {n1, n2, n3};
    int last = -1;
    double prod = 1.0;
    for (int ax = 0; ax < 3; ++ax)
        if (dims[ax] > 1 && ((axes >> ax) & 1)) { last = ax; prod *= dims[ax]; }
    const T sc = inv ? (T)(1.0 / prod) : (T)1;
    for (int ax = 0; ax < 3; ++ax) {
        const int n = dims[ax];
        if (n == 1 || !((axes >> ax) & 1)) continue;
        ColPassArgs<T> a = colargs<T>(plan_or_fail(n), twiddles<T>(n, st), tile_width<T>(n), 0);
        a.mode = inv ? 2 : 1;
        a.in = d; a.out = d; a.in_cnt = a.out_cnt = n; a.in_c = a.out_c = 0;
        a.scale = (ax == last) ? sc : (T)1;
        int other = 1;
        if (ax == 0) {
            a.col_stride = n1; a.ncols = n2 * n3; a.in_dim = a.out_dim = 1;
        } else if (ax == 1) {
            a.ncols = n1; a.in_dim = a.out_dim = n1; a.in_other = a.out_other = (long long)n1 * n2; other = n3;
        } else {
            a.ncols = n1; a.in_dim = a.out_dim = (long long)n1 * n2; a.in_other = a.out_other = n1; other = n2;
        }
        launch_colpass<T>(a, other, st);
    }
}

void fftn_device(genfire_ctx *ctx, int precision, void *d_data, int n1, int n2, int n3, bool inverse, int axes)
{
    if (precision == GENFIRE_PREC_FP64) fftn_t<double>(ctx, (double2 *)d_data, n1, n2, n3, inverse, axes);
    else fftn_t<float>(ctx, (float2 *)d_data, n1, n2, n3, inverse, axes);
}

// ===========================================================================
// the iteration
// ===========================================================================
// Constraint table: one entry per half-spectrum point q with q in E or -q in E
// (E = measuredK ~= 0 & mask, reconstruct.m:99), grouped by column q1 + h1*q2.
struct TabGeom {
    int n1, n2, h1, W3, m;
    // delay indices whose test 1 - Q > delay holds at every point: make_Kspace_indices'
    // coordinates lie in [-1, 1], so Q <= sqrt(3) and 1 - Q > -0.7321 everywhere; a
    // delay below -0.75 (mode 3's -999, the -10 of modes 1 and 2) needs no Q
    uint32_t always;
    double delay[32];
};

// |k| / (n/2) of make_Kspace_indices, rounded step by step as the oracle does
__device__ __forceinline__ double q_radius(double kx, double ky, double kz)
{
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz)));
}

// make_Kspace_indices coordinate: (i - r) / r with r = n2K (n/2 or (n-1)/2), 0 for n == 1
__device__ __forceinline__ double kspace_k(int n, int i)
{
    if (n == 1) return 0.0;
    const int r = (n % 2 == 0) ? n / 2 : (n - 1) / 2;
    return (double)(i - r) / (double)r;
}

// |M| of one measured value, summed in FP64 by the caller: complex64 values in
// FP32 (the iteration's own precision), complex128 in FP64
__device__ __forceinline__ double abs_val(float2 v) { return (double)sqrtf(fmaf(v.x, v.x, v.y * v.y)); }
__device__ __forceinline__ double abs_val(double2 v) { return sqrt(v.x * v.x + v.y * v.y); }

// One half-spectrum point q of the constraint table.  MASKS: also the
// per-delay masks (the counting pass needs only whether q is an entry and the
// |M| it contributes).
template <typename T, bool MASKS>
__device__ __forceinline__ bool tab_point(const cplx<T> *__restrict__ M, const uint8_t *__restrict__ mask,
                                          const TabGeom &g, int q1, int q2, int q3, TabEntry<T> &e, double &absM)
{
    const int n1 = g.n1, n2 = g.n2;
    const int c1 = (q1 + n1 / 2) % n1, c2 = (q2 + n2 / 2) % n2, c3 = (q3 + n1 / 2) % n1;
    const int m1 = (n1 - q1) % n1, m2 = (n2 - q2) % n2, m3 = (n1 - q3) % n1;
    const int d1 = (m1 + n1 / 2) % n1, d2 = (m2 + n2 / 2) % n2, d3 = (m3 + n1 / 2) % n1;
    const long long a = c1 + (long long)n1 * (c2 + (long long)n2 * c3);
    const long long b = d1 + (long long)n1 * (d2 + (long long)n2 * d3);
    const cplx<T> Ma = M[a], Mb = M[b];
    const bool inEq = (Ma.x != 0 || Ma.y != 0) && (!mask || mask[a]);
    const bool inEm = (Mb.x != 0 || Mb.y != 0) && (!mask || mask[b]);
    absM = 0;
    if (!inEq && !inEm) return false;
    const bool mate_stored = m1 < g.h1;
    e.pos = (uint32_t)q3 | ((uint32_t)(q1 % g.W3) << 16);
    e.eflags = (inEq ? 1u : 0u) | ((inEm && !mate_stored) ? 2u : 0u);
    // constraintIndicators = 1 - Q (reconstruct.m:36-42, make_Kspace_indices.m)
    auto kv = [](int n, int i) -> double { return kspace_k(n, i); };
    const uint32_t all = g.m >= 32 ? 0xFFFFFFFFu : ((1u << g.m) - 1u);
    uint32_t cq = 0, cm = 0;
    if (inEq) {
        if constexpr (MASKS) {
            cq = g.always;
            if (cq != all) {
                const double ci = 1.0 - q_radius(kv(n2, c2), kv(n1, c1), kv(n1, c3));
                for (int k = 0; k < g.m; ++k) cq |= (ci > g.delay[k]) ? (1u << k) : 0u;
            }
        } else {
            absM += abs_val(Ma);
        }
    }
    if (inEm) {
        if constexpr (MASKS) {
            cm = g.always;
            if (cm != all) {
                const double ci = 1.0 - q_radius(kv(n2, d2), kv(n1, d1), kv(n1, d3));
                for (int k = 0; k < g.m; ++k) cm |= (ci > g.delay[k]) ? (1u << k) : 0u;
            }
        } else if (!mate_stored) {
            absM += abs_val(Mb);
        }
    }
    e.cq = cq;
    e.cmq = cm;
    e.Mq = Ma;
    e.Mmq = Mb;
    return true;
}

// The table is built per (column, segment of kTabSeg consecutive q3): counts
// (and |M| sums) per segment, one ordered exclusive scan over (column,
// segment) with the segment fastest, then each segment writes its entries at
// its offset, so a column's entries stay in q3 order.  Grid: x = 128
// consecutive columns (q1 fastest: coalesced reads of M), y = segment.
constexpr int kTabSeg = 32;

template <typename T>
__global__ void k_tab_count(const cplx<T> *__restrict__ M, const uint8_t *__restrict__ mask, TabGeom g, int nseg,
                            int *__restrict__ counts, double *__restrict__ colsum)
{
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= g.h1 * g.n2) return;
    const int q1 = col % g.h1, q2 = col / g.h1, seg = blockIdx.y;
    const int e3 = min(g.n1, (seg + 1) * kTabSeg);
    int cnt = 0;
    double s = 0;
    for (int q3 = seg * kTabSeg; q3 < e3; ++q3) {
        TabEntry<T> e;
        double am;
        if (tab_point<T, false>(M, mask, g, q1, q2, q3, e, am)) { ++cnt; s += am; }
    }
    counts[(long long)col * nseg + seg] = cnt;
    colsum[(long long)col * nseg + seg] = s;
}

template <typename T>
__global__ void k_tab_write(const cplx<T> *__restrict__ M, const uint8_t *__restrict__ mask, TabGeom g, int nseg,
                            const int *__restrict__ segoff, TabEntry<T> *__restrict__ tab)
{
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= g.h1 * g.n2) return;
    const int q1 = col % g.h1, q2 = col / g.h1, seg = blockIdx.y;
    const int e3 = min(g.n1, (seg + 1) * kTabSeg);
    int o = segoff[(long long)col * nseg + seg];
    for (int q3 = seg * kTabSeg; q3 < e3; ++q3) {
        TabEntry<T> e;
        double am;
        if (tab_point<T, true>(M, mask, g, q1, q2, q3, e, am)) tab[o++] = e;
    }
}

// column offsets of the table (CSR) from the segment offsets
__global__ void k_tab_coloff(const int *__restrict__ segoff, int ncol, int nseg, int *__restrict__ taboff)
{
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col <= ncol) taboff[col] = segoff[(long long)col * nseg];
}

// exclusive scan of n ints (single CTA) and the total in off[n]; also the
// ordered sum of the column sums
__global__ void __launch_bounds__(1024) k_scan_cols(const int *__restrict__ counts, const double *__restrict__ colsum,
                                                    int n, int *__restrict__ off, double *__restrict__ total)
{
    __shared__ long long part[1024];
    __shared__ double dpart[1024];
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(b + per, n);
    long long s = 0;
    double d = 0;
    for (int i = b; i < e; ++i) { s += counts[i]; d += colsum[i]; }
    part[threadIdx.x] = s;
    dpart[threadIdx.x] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long run = 0;
        double dr = 0;
        for (int i = 0; i < (int)blockDim.x; ++i) { long long t = part[i]; part[i] = run; run += t; dr += dpart[i]; }
        off[n] = (int)run;
        *total = dr;
    }
    __syncthreads();
    long long run = part[threadIdx.x];
    for (int i = b; i < e; ++i) { off[i] = (int)run; run += counts[i]; }
}

// ---------------------------------------------------------------- Rfree
// Candidates of one shell (reconstruct.m:48): measuredK ~= 0 & Q >= lo & Q < hi,
// Q = make_Kspace_indices (same rounding as tab_point), in ascending linear
// order.  Pass 1 (out == NULL) counts per 1024-point block; pass 2 writes the
// indices at the block offsets (warp ballots, block prefix in warp order).
template <typename T>
__global__ void __launch_bounds__(1024) k_rfree_mark(const cplx<T> *__restrict__ M, int n1, int n2, double lo, double hi,
                                                     int *__restrict__ bcount, const int *__restrict__ boff,
                                                     int *__restrict__ out)
{
    __shared__ int wc[32];
    const long long N = (long long)n1 * n2 * n1;
    const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
    bool f = false;
    if (i < N) {
        const cplx<T> v = M[i];
        if (v.x != 0 || v.y != 0) {
            const int c1 = (int)(i % n1), c2 = (int)((i / n1) % n2), c3 = (int)(i / ((long long)n1 * n2));
            const double q = q_radius(kspace_k(n2, c2), kspace_k(n1, c1), kspace_k(n1, c3));
            f = q >= lo && q < hi;
        }
    }
    const unsigned b = __ballot_sync(0xffffffffu, f);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) wc[w] = __popc(b);
    __syncthreads();
    if (!out) {
        if (threadIdx.x == 0) {
            int t = 0;
            for (int k = 0; k < 32; ++k) t += wc[k];
            bcount[blockIdx.x] = t;
        }
        return;
    }
    if (f) {
        int pre = boff[blockIdx.x];
        for (int k = 0; k < w; ++k) pre += wc[k];
        out[pre + __popc(b & ((1u << l) - 1u))] = (int)i;
    }
}

template <typename T>
__global__ void k_rfree_gather(const cplx<T> *__restrict__ M, const long long *__restrict__ idx, long long n,
                               cplx<T> *__restrict__ vals)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        vals[i] = M[idx[i]];
}

// Rfree of each shell for the current iteration (reconstruct.m:137-146):
// sum |k - M| / sum |M| over the shell's withheld points, from the values F3
// captured before the constraint; FP64 sums in a fixed order.  One CTA per shell.
template <typename T>
__global__ void __launch_bounds__(256) k_rfree_shells(const cplx<T> *__restrict__ cap, const cplx<T> *__restrict__ vals,
                                                      const long long *__restrict__ off, int nshells,
                                                      const Ctl *__restrict__ ctl, double *__restrict__ out)
{
    __shared__ double rn[256], rd[256];
    const int sh = blockIdx.x, t = threadIdx.x;
    double num = 0, den = 0;
    for (long long i = off[sh] + t; i < off[sh + 1]; i += 256) {
        const cplx<T> k = cap[i], v = vals[i];
        const double dx = (double)k.x - (double)v.x, dy = (double)k.y - (double)v.y;
        num += sqrt(dx * dx + dy * dy);
        den += sqrt((double)v.x * (double)v.x + (double)v.y * (double)v.y);
    }
    rn[t] = num;
    rd[t] = den;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o) {
            rn[t] += rn[t + o];
            rd[t] += rd[t + o];
        }
        __syncthreads();
    }
    if (t == 0) out[(long long)(ctl->it - 1) * nshells + sh] = rn[0] / rd[0];
}

template <typename T>
static void rfree_candidates_t(genfire_ctx *ctx, const cplx<T> *dM, int n1, int n2, int nbins, int64_t *counts,
                               int64_t *indices)
{
    cudaStream_t st = ctx->stream;
    const long long N = (long long)n1 * n2 * n1;
    const int nb = (int)cdiv(N, 1024);
    DevBuf bc(sizeof(int) * nb, st), bo(sizeof(int) * (nb + 1), st), dz(sizeof(double) * nb, st), dt(sizeof(double), st);
    GF_CUDA(cudaMemsetAsync(dz.p, 0, dz.bytes, st));
    long long filled = 0;
    for (int s = 0; s < nbins; ++s) {
        // edges linspace(0, 1, nbins + 1): (i * 1) / nbins; resRange = -0.05 (reconstruct.m:36, :47-48)
        const double lo = (double)s / (double)nbins + -0.05, hi = (double)(s + 1) / (double)nbins;
        k_rfree_mark<T><<<nb, 1024, 0, st>>>(dM, n1, n2, lo, hi, bc.as<int>(), nullptr, nullptr);
        GF_CHECK_LAUNCH();
        k_scan_cols<<<1, 1024, 0, st>>>(bc.as<int>(), dz.as<double>(), nb, bo.as<int>(), dt.as<double>());
        GF_CHECK_LAUNCH();
        int tot = 0;
        GF_CUDA(cudaMemcpyAsync(&tot, bo.as<int>() + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
        counts[s] = tot;
        if (indices && tot > 0) {
            DevBuf out(sizeof(int) * (size_t)tot, st);
            k_rfree_mark<T><<<nb, 1024, 0, st>>>(dM, n1, n2, lo, hi, bc.as<int>(), bo.as<int>(), out.as<int>());
            GF_CHECK_LAUNCH();
            std::vector<int> h((size_t)tot);
            GF_CUDA(cudaMemcpyAsync(h.data(), out.p, sizeof(int) * (size_t)tot, cudaMemcpyDeviceToHost, st));
            GF_CUDA(cudaStreamSynchronize(st));
            for (int k = 0; k < tot; ++k) indices[filled + k] = h[k];
        }
        filled += tot;
    }
}

void rfree_candidates(genfire_ctx *ctx, const genfire_params &p, const void *M, bool on_device, int nbins,
                      int64_t *counts, int64_t *indices)
{
    if (nbins < 1) fail(GENFIRE_ERR_ARG, "numBinsRfree must be positive.");
    if (!M || !counts) fail(GENFIRE_ERR_ARG, "measuredK or counts is NULL.");
    int n1, n2;
    grid_dims(p, n1, n2);
    const size_t N = (size_t)n1 * n2 * n1;
    cudaStream_t st = ctx->stream;
    const size_t es = p.precision == GENFIRE_PREC_FP64 ? sizeof(double2) : sizeof(float2);
    DevBuf dM;
    const void *d = M;
    if (!on_device) {
        dM.alloc(es * N, st);
        GF_CUDA(cudaMemcpyAsync(dM.p, M, es * N, cudaMemcpyHostToDevice, st));
        d = dM.p;
    }
    if (p.precision == GENFIRE_PREC_FP64) rfree_candidates_t<double>(ctx, static_cast<const double2 *>(d), n1, n2, nbins, counts, indices);
    else rfree_candidates_t<float>(ctx, static_cast<const float2 *>(d), n1, n2, nbins, counts, indices);
}

// Object in box coordinates from an initial object (D1 x D2 x D1) or zeros.
// grid: x over e1, y = e2, z = e3
// Support masks of the passes: mask[b] = 1 when one of rows
// [rows_per_cta b, rows_per_cta (b + 1)) of the box-shaped support holds a
// voxel (2 rows per entry: the row passes' pairs; B2 rows: the slabs along
// dim 3 of the radix-32 dim-2 passes).  One CTA per entry.
__global__ void __launch_bounds__(256) k_row_support_mask(const uint8_t *__restrict__ S, int B1, int nrows,
                                                          int rows_per_cta, uint8_t *__restrict__ mask)
{
    const long long r0 = (long long)blockIdx.x * rows_per_cta;
    const long long r1 = min((long long)nrows, r0 + rows_per_cta);
    int any = 0;
    for (long long e = r0 * B1 + threadIdx.x; e < r1 * B1; e += 256) any |= S[e];
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) mask[blockIdx.x] = any ? 1 : 0;
}

template <typename T>
__global__ void k_place(const T *__restrict__ init, int D1, int D2, int B1, int B2, int B3, T *__restrict__ x)
{
    const int o1 = B1 / 2 - D1 / 2, o2 = B2 / 2 - D2 / 2, o3 = B3 / 2 - D1 / 2;
    const int e2 = blockIdx.y, e3 = blockIdx.z;
    const int b = e2 - o2, c = e3 - o3;
    const bool in23 = init && b >= 0 && b < D2 && c >= 0 && c < D1;
    T *row = x + (long long)B1 * (e2 + (long long)B2 * e3);
    for (int e1 = blockIdx.x * blockDim.x + threadIdx.x; e1 < B1; e1 += gridDim.x * blockDim.x) {
        const int a = e1 - o1;
        row[e1] = (in23 && a >= 0 && a < D1) ? init[a + (long long)D1 * (b + (long long)D2 * c)] : (T)0;
    }
}

// reconstruction = My_stripzero(fftshift(best), [D1 D2 D1]) with the best
// object taken after positivity and support (reconstruct.m:126-131, 152, 192)
// grid: x over a (dim 1), y = b, z = c
template <typename T>
__global__ void k_extract(const T *const *__restrict__ xs, const Ctl *__restrict__ ctl, const uint8_t *__restrict__ S,
                          int positivity, int D1, int D2, int B1, int B2, int B3, T *__restrict__ out)
{
    const int o1 = B1 / 2 - D1 / 2, o2 = B2 / 2 - D2 / 2, o3 = B3 / 2 - D1 / 2;
    const int sel = ctl->xbest;
    const int b = blockIdx.y, c = blockIdx.z;
    const long long rin = (long long)B1 * ((b + o2) + (long long)B2 * (c + o3)) + o1;
    T *orow = out + (long long)D1 * (b + (long long)D2 * c);
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < D1; a += gridDim.x * blockDim.x) {
        T v = 0;
        if (sel >= 0) {
            v = xs[sel][rin + a];
            if (positivity && v < (T)0) v = 0;
            if (S) v = v * (T)S[rin + a];
        }
        orow[a] = v;
    }
}

struct ReconBase {
    virtual ~ReconBase() {}
    virtual void iterate(int count) = 0;
    // one iteration as a (not instantiated) graph, for batches
    virtual cudaGraph_t capture_iteration() = 0;
    // one iteration's launches on st (for a caller's own capture), the kernel
    // attributes that must be set before a capture, and the grid size (the
    // batch orders members by it)
    virtual void enqueue(cudaStream_t st) = 0;
    virtual void check_device_error() = 0;
    virtual void prepare_capture() = 0;
    virtual long long grid_points() const = 0;
    // iterations still allowed, and the bookkeeping after one batched iteration
    virtual int remaining() const = 0;
    virtual void advance() = 0;
    virtual void profile(int count, double *ms, double *bytes) = 0;
    virtual void tuning(int *variants) const = 0;
    virtual void result(void *rec, double *errK, double *errR, double *Rarr, double *Rarr2, bool on_device) = 0;
    virtual void set_rfree(int nshells, const int64_t *counts, const int64_t *indices) = 0;
    virtual int rfree(double *out) const = 0;
};

template <typename T> struct ReconT : ReconBase {
    genfire_ctx *ctx;
    genfire_params p;
    int n1, n2, D1, D2, h1, ld1, B1, B2, B3, W1, W2, W3;
    FftPlan pl1, pl2;
    const cplx<T> *tw1, *tw2;
    DevBuf xbuf[2], xptrs, S, Y1, Y2, M, mask, tab, taboff, partial, ctl, changes, hist, dmeas, dR, dsums;
    DevBuf pairmask;  // per row pair of the row passes: any support voxel in its two rows
    DevBuf zmask;    // per slab of the box along dim 3: any support voxel in it
    double frac_rows = 1.0, frac_slabs = 1.0;  // the shares of those masks that are set
    DevBuf rtab, rtaboff, rcap, rvals, rshoff, rhist;  // Rfree monitor
    DevBuf errf;  // set by a pass whose bounded device-side wait expired
    int m = 0, nparts = 0, tiles1 = 0, ntab = 0, nshells = 0;
    long long nrfree = 0;
    double denom = 0;
    int it_done = 0;
    int vF2 = kColAuto, vF3 = kColAuto, vI2 = kColAuto;  // column-pass variants (autotuned)
    cudaGraphExec_t exec = nullptr;
    std::vector<double> errR, Rarr, Rarr2;

    ~ReconT() override
    {
        if (exec) cudaGraphExecDestroy(exec);
        cudaStreamSynchronize(ctx->stream);
    }

    void setup(const void *Min, const uint8_t *maskin, const uint8_t *support, const void *initial,
               const double *projs, const double *angles, bool on_device)
    {
        cudaStream_t st = ctx->stream;
        const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        D1 = p.Dim1; D2 = p.Dim2;
        grid_dims(p, n1, n2);
        if (n1 < D1 || n2 < D2) fail(GENFIRE_ERR_ARG, "oversampled size smaller than the projection size.");
        h1 = n1 / 2 + 1;
        ld1 = round_up(h1, 8);
        if (p.constraintSupport) { B1 = D1; B2 = D2; B3 = D1; }
        else { B1 = n1; B2 = n2; B3 = n1; }
        pl1 = plan_or_fail(n1);
        pl2 = plan_or_fail(n2);
        tw1 = twiddles<T>(n1, st);
        tw2 = twiddles<T>(n2, st);
        W1 = tile_width<T>(n1); W2 = tile_width<T>(n2); W3 = W1;
        if (W3 > 16) fail(GENFIRE_ERR_STATE, "internal: tile width too large for the table format.");
        const long long N = (long long)n1 * n2 * n1, NB = (long long)B1 * B2 * B3;

        // delays and change points (GENFIRE_Reconstructor.m:156-165, reconstruct.m:103)
        double delay[32];
        int mm = 0;
        const int mode = p.constraintEnforcementMode;
        if (mode == 1 || mode == 2) {
            for (int k = 0; k < 12; ++k) delay[mm++] = 0.95 + k * -0.1;
            delay[mm++] = -10; delay[mm++] = -10;
            if (mode == 1) {
                delay[mm++] = -10;
                for (int k = 0; k < 12; ++k) delay[mm++] = -0.15 + k * 0.1;
            }
        } else if (mode == 3) {
            for (int k = 0; k < 5; ++k) delay[mm++] = -999;
        } else {
            fail(GENFIRE_ERR_ARG, "ERROR! constraintEnforcementMode value " + std::to_string(mode) + " not understood");
        }
        m = mm;
        std::vector<int> ch(m);
        const int Nit = p.numIterations;
        for (int i = 0; i < m; ++i) {
            double y = (m == 1) ? (double)Nit : 1.0 + ((double)i * (double)(Nit - 1)) / (double)(m - 1);
            if (i == m - 1) y = Nit;
            ch[i] = (int)mround(y);
        }
        changes.alloc(sizeof(int) * m, st);
        GF_CUDA(cudaMemcpyAsync(changes.p, ch.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st));

        // measured data on the device
        M.alloc(sizeof(cplx<T>) * N, st);
        if (on_device) GF_CUDA(cudaMemcpyAsync(M.p, Min, sizeof(cplx<T>) * N, kind, st));
        else copy_host(M.p, Min, sizeof(cplx<T>) * N, kind, st);
        if (maskin) {
            mask.alloc(N, st);
            if (on_device) GF_CUDA(cudaMemcpyAsync(mask.p, maskin, N, kind, st));
            else copy_host(mask.p, maskin, N, kind, st);
        }
        // constraint table
        TabGeom g;
        g.n1 = n1; g.n2 = n2; g.h1 = h1; g.W3 = W3; g.m = m;
        g.always = 0;
        for (int k = 0; k < 32; ++k) {
            g.delay[k] = k < m ? delay[k] : 0.0;
            if (k < m && delay[k] < -0.75) g.always |= 1u << k;
        }
        const int ncol = h1 * n2, nseg = (int)cdiv(n1, kTabSeg);
        const long long nsc = (long long)ncol * nseg;
        DevBuf counts(sizeof(int) * nsc, st), colsum(sizeof(double) * nsc, st), dtot(sizeof(double), st);
        DevBuf segoff(sizeof(int) * (nsc + 1), st);
        taboff.alloc(sizeof(int) * (ncol + 1), st);
        const dim3 tgrid((unsigned)cdiv(ncol, 128), (unsigned)nseg);
        k_tab_count<T><<<tgrid, 128, 0, st>>>(M.as<cplx<T>>(), mask.as<uint8_t>(), g, nseg, counts.as<int>(), colsum.as<double>());
        GF_CHECK_LAUNCH();
        {
            // segment offsets: segoff[0] = 0, segoff[i + 1] = counts[0] + ... + counts[i];
            // denom = the sum of the segments' |M| sums (device-wide reduction)
            GF_CUDA(cudaMemsetAsync(segoff.p, 0, sizeof(int), st));
            size_t tb1 = 0, tb2 = 0;
            GF_CUDA(cub::DeviceScan::InclusiveSum(nullptr, tb1, counts.as<int>(), segoff.as<int>() + 1, (int)nsc, st));
            GF_CUDA(cub::DeviceReduce::Sum(nullptr, tb2, colsum.as<double>(), dtot.as<double>(), (int)nsc, st));
            DevBuf tmp(std::max(tb1, tb2), st);
            GF_CUDA(cub::DeviceScan::InclusiveSum(tmp.p, tb1, counts.as<int>(), segoff.as<int>() + 1, (int)nsc, st));
            GF_CUDA(cub::DeviceReduce::Sum(tmp.p, tb2, colsum.as<double>(), dtot.as<double>(), (int)nsc, st));
        }
        k_tab_coloff<<<cdiv(ncol + 1, 256), 256, 0, st>>>(segoff.as<int>(), ncol, nseg, taboff.as<int>());
        GF_CHECK_LAUNCH();
        ntab = 0;
        GF_CUDA(cudaMemcpyAsync(&ntab, taboff.as<int>() + ncol, sizeof(int), cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaMemcpyAsync(&denom, dtot.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
        tab.alloc(sizeof(TabEntry<T>) * (size_t)std::max(ntab, 1), st);
        k_tab_write<T><<<tgrid, 128, 0, st>>>(M.as<cplx<T>>(), mask.as<uint8_t>(), g, nseg, segoff.as<int>(), tab.as<TabEntry<T>>());
        GF_CHECK_LAUNCH();

        // object buffers, support
        for (int k = 0; k < 2; ++k) xbuf[k].alloc(sizeof(T) * NB, st);
        {
            DevBuf init;
            const T *dinit = nullptr;
            if (initial) {
                const size_t nb = sizeof(T) * (size_t)D1 * D2 * D1;
                if (on_device) dinit = static_cast<const T *>(initial);
                else {
                    init.alloc(nb, st);
                    copy_host(init.p, initial, nb, cudaMemcpyHostToDevice, st);
                    dinit = init.as<T>();
                }
            }
            k_place<T><<<dim3(cdiv(B1, 256), B2, B3), 256, 0, st>>>(dinit, D1, D2, B1, B2, B3, xbuf[0].as<T>());
            GF_CHECK_LAUNCH();
            GF_CUDA(cudaStreamSynchronize(st));
        }
        GF_CUDA(cudaMemsetAsync(xbuf[1].p, 0, xbuf[1].bytes, st));
        T *hp[2] = {xbuf[0].as<T>(), xbuf[1].as<T>()};
        xptrs.alloc(sizeof(hp), st);
        GF_CUDA(cudaMemcpyAsync(xptrs.p, hp, sizeof(hp), cudaMemcpyHostToDevice, st));
        if (p.constraintSupport) {
            const size_t ns = (size_t)D1 * D2 * D1;
            S.alloc(ns, st);
            if (support) GF_CUDA(cudaMemcpyAsync(S.p, support, ns, kind, st));
            else GF_CUDA(cudaMemsetAsync(S.p, 1, ns, st));
            // the row pairs that hold no support voxel, for every row-pass
            // engine (a CTA skips its rows when all of its pairs are empty);
            // the object buffers are finite everywhere (the placement and the
            // clear above), so rows the passes skip stay finite
            if (support) {
                const int nrow = B2 * B3, npairs = (nrow + 1) / 2;
                pairmask.alloc(npairs, st);
                k_row_support_mask<<<npairs, 256, 0, st>>>(S.as<uint8_t>(), B1, nrow, 2, pairmask.as<uint8_t>());
                GF_CHECK_LAUNCH();
                std::vector<uint8_t> hr(npairs);
                GF_CUDA(cudaMemcpyAsync(hr.data(), pairmask.p, npairs, cudaMemcpyDeviceToHost, st));
                // slabs along dim 3 (the radix-32 dim-2 passes' `other`): B2 rows each
                std::vector<uint8_t> hz;
                if (sizeof(T) == 4 && (n1 == 512 || n1 == 1024) && rows_r32_enabled()) {
                    zmask.alloc(B3, st);
                    k_row_support_mask<<<B3, 256, 0, st>>>(S.as<uint8_t>(), B1, nrow, B2, zmask.as<uint8_t>());
                    GF_CHECK_LAUNCH();
                    hz.resize(B3);
                    GF_CUDA(cudaMemcpyAsync(hz.data(), zmask.p, B3, cudaMemcpyDeviceToHost, st));
                }
                GF_CUDA(cudaStreamSynchronize(st));
                // the shares of set entries, for the passes' byte counts (profile)
                frac_rows = (double)std::count(hr.begin(), hr.end(), (uint8_t)1) / npairs;
                if (!hz.empty()) frac_slabs = (double)std::count(hz.begin(), hz.end(), (uint8_t)1) / B3;
            }
        }
        Y1.alloc(sizeof(cplx<T>) * (size_t)ld1 * B2 * B3, st);
        Y2.alloc(sizeof(cplx<T>) * (size_t)ld1 * n2 * B3, st);
        tiles1 = (int)cdiv(h1, W3);
        nparts = tiles1 * n2;
        partial.alloc(sizeof(double) * nparts, st);
        hist.alloc(sizeof(double) * std::max(Nit, 1), st);
        GF_CUDA(cudaMemsetAsync(hist.p, 0, hist.bytes, st));
        errf.alloc(sizeof(int), st);
        GF_CUDA(cudaMemsetAsync(errf.p, 0, sizeof(int), st));
        Ctl c0;
        std::memset(&c0, 0, sizeof(c0));
        c0.m = m; c0.xbest = -1; c0.bestErr = 1e30;
        ctl.alloc(sizeof(Ctl), st);
        GF_CUDA(cudaMemcpyAsync(ctl.p, &c0, sizeof(Ctl), cudaMemcpyHostToDevice, st));

        // R-factor monitor inputs (reconstruct.m:168-185; ZYZ closed-form projector)
        if (p.monitor_R == 1) {
            if (!projs || !angles) fail(GENFIRE_ERR_ARG, "monitor_R needs projections and angles.");
            if (p.monitorR_loopLength < 1) fail(GENFIRE_ERR_ARG, "monitorR_loopLength must be positive.");
            const int P = p.NumProjs;
            const size_t npj = (size_t)D1 * D2 * P;
            dmeas.alloc(sizeof(double) * npj, st);
            GF_CUDA(cudaMemcpyAsync(dmeas.p, projs, sizeof(double) * npj, kind, st));
            std::vector<double> Rs(9 * (size_t)P), ang(3 * (size_t)P);
            if (on_device) GF_CUDA(cudaMemcpyAsync(ang.data(), angles, sizeof(double) * 3 * P, cudaMemcpyDeviceToHost, st));
            else std::memcpy(ang.data(), angles, sizeof(double) * 3 * P);
            GF_CUDA(cudaStreamSynchronize(st));
            for (int i = 0; i < P; ++i) rot_zyz(ang[i], ang[i + P], ang[i + 2 * P], &Rs[9 * (size_t)i]);
            dR.alloc(sizeof(double) * Rs.size(), st);
            GF_CUDA(cudaMemcpyAsync(dR.p, Rs.data(), sizeof(double) * Rs.size(), cudaMemcpyHostToDevice, st));
            dsums.alloc(sizeof(double) * 4 * P, st);
        }
        GF_CUDA(cudaStreamSynchronize(st));
        autotune();
        build_graph();
    }

    // F2: dim 2 forward, box rows in, all n2 frequencies out
    ColPassArgs<T> f2_args()
    {
        ColPassArgs<T> a = colargs<T>(pl2, tw2, W2, h1);
        a.in = Y1.as<cplx<T>>(); a.in_dim = ld1; a.in_other = (long long)ld1 * B2; a.in_cnt = B2; a.in_c = B2 / 2;
        a.out = Y2.as<cplx<T>>(); a.out_dim = ld1; a.out_other = (long long)ld1 * n2; a.out_cnt = n2; a.out_c = 0;
        a.mode = 1;
        a.zmask = zmask.as<uint8_t>();  // zero slabs stay zero (nullptr when not built)
        a.zmask_zero = 1;
        return a;
    }
    // F3: dim 3 forward, constraint, dim 3 inverse (in place)
    ColPassArgs<T> f3_args()
    {
        Ctl *c = ctl.as<Ctl>();
        ColPassArgs<T> b = colargs<T>(pl1, tw1, W3, h1);
        b.in = Y2.as<cplx<T>>(); b.in_dim = (long long)ld1 * n2; b.in_other = ld1; b.in_cnt = B3; b.in_c = B3 / 2;
        b.out = Y2.as<cplx<T>>(); b.out_dim = (long long)ld1 * n2; b.out_other = ld1; b.out_cnt = B3; b.out_c = B3 / 2;
        b.mode = 1 | 2 | 4;
        b.tab_off = taboff.as<int>(); b.tab = tab.as<TabEntry<T>>(); b.h1 = h1; b.partial = partial.as<double>();
        b.err = errf.as<int>();
        b.cidx = &c->cidx;
        if (nshells > 0) {
            b.rtab_off = rtaboff.as<int>();
            b.rtab = rtab.as<uint2>();
            b.rcap = rcap.as<cplx<T>>();
        }
        return b;
    }
    // I2: dim 2 inverse, box rows out; with_ctl: CTA 0 first forms errK from
    // F3's partials and updates the best object and the output buffer
    ColPassArgs<T> i2_args(bool with_ctl = true)
    {
        ColPassArgs<T> d = colargs<T>(pl2, tw2, W2, h1);
        d.in = Y2.as<cplx<T>>(); d.in_dim = ld1; d.in_other = (long long)ld1 * n2; d.in_cnt = n2; d.in_c = 0;
        d.out = Y1.as<cplx<T>>(); d.out_dim = ld1; d.out_other = (long long)ld1 * B2; d.out_cnt = B2; d.out_c = B2 / 2;
        d.mode = 2;
        // slabs without support voxels: their rows are skipped by I1 and masked
        // by the next F1, so they are not transformed back; with the R-factor
        // monitor on, I1 writes every row and reads them all
        d.zmask = p.monitor_R == 1 ? nullptr : zmask.as<uint8_t>();
        d.zmask_zero = 0;
        if (with_ctl) {
            d.ctl = ctl.as<Ctl>();
            d.partial = partial.as<double>();
            d.nparts = nparts;
            d.denom = denom;
            d.hist = hist.as<double>();
        }
        return d;
    }

    // Column-pass variants by measurement on this problem's buffers (the
    // environment variable GENFIRE_AUTOTUNE=0 keeps the default choices).
    void autotune()
    {
        const char *env = std::getenv("GENFIRE_AUTOTUNE");
        if (env && env[0] == '0') return;
        cudaStream_t st = ctx->stream;
        vF2 = autotune_colpass<T>(f2_args(), B3, st);
        vF3 = autotune_colpass<T>(f3_args(), n2, st);
        vI2 = autotune_colpass<T>(i2_args(false), B3, st);  // timed launches leave the control block alone
        GF_CUDA(cudaStreamSynchronize(st));
    }

    // ev (optional) receives an event before each of the 7 kernels and one after
    void enqueue_iteration(cudaStream_t st, cudaEvent_t *ev = nullptr)
    {
        Ctl *c = ctl.as<Ctl>();
        int ek = 0;
        auto mark = [&]() { if (ev) GF_CUDA(cudaEventRecord(ev[ek++], st)); };
        mark();
        // F1: rows (dim 1) real -> half spectrum, with positivity and support;
        // the object of this iteration is the previous iteration's output
        // buffer (xnext; CTA 0 sets xcur to it)
        RowPassArgs<T> r;
        std::memset(&r, 0, sizeof(r));
        r.pl = pl1; r.tw = tw1; r.W = W1; r.nrows = B2 * B3; r.B1 = B1; r.c1 = B1 / 2; r.h1 = h1; r.ld1 = ld1;
        r.xs[0] = xbuf[0].as<T>(); r.xs[1] = xbuf[1].as<T>(); r.xsel = &c->xnext;
        r.ctl = c;
        r.changes = changes.as<int>();
        r.support = p.constraintSupport ? S.as<uint8_t>() : nullptr;
        r.pairmask = pairmask.as<uint8_t>();  // nullptr when not built
        r.positivity = p.constraintPositivity;
        r.Y = Y1.as<cplx<T>>();
        r.scale = (T)1;
        launch_rows<T>(r, true, st);
        mark();
        launch_colpass<T>(f2_args(), B3, st, vF2);
        mark();
        launch_colpass<T>(f3_args(), n2, st, vF3);
        if (nshells > 0) {
            k_rfree_shells<T><<<nshells, 256, 0, st>>>(rcap.as<cplx<T>>(), rvals.as<cplx<T>>(), rshoff.as<long long>(),
                                                       nshells, c, rhist.as<double>());
            GF_CHECK_LAUNCH();
        }
        mark();
        launch_colpass<T>(i2_args(), B3, st, vI2);
        mark();
        // I1: rows half spectrum -> real box, 1/N
        RowPassArgs<T> q = r;
        q.xsel = &c->xnext;
        q.ctl = nullptr;
        q.changes = nullptr;
        q.support = nullptr;
        // the R-factor monitor projects this pass's raw output, so with it on
        // every row is written
        q.pairmask = p.monitor_R == 1 ? nullptr : pairmask.as<uint8_t>();
        q.positivity = 0;
        q.scale = (T)(1.0 / ((double)n1 * n2 * n1));
        launch_rows<T>(q, false, st);
        mark();
    }

    // Algorithmic HBM bytes per launch of each kernel of the iteration.
    void kernel_bytes(double *b) const
    {
        const double S = sizeof(cplx<T>), Rs = sizeof(T);
        const double box = (double)B1 * B2 * B3;
        const double half_box = (double)h1 * B2 * B3, half_mid = (double)h1 * n2 * B3;
        // with the support masks the row and dim-2 passes move only the rows
        // and slabs that hold support voxels (F1 and F2 still write every zero)
        const bool skip = p.monitor_R != 1;
        const double fr = frac_rows, fz = frac_slabs;
        b[0] = (box * Rs + (p.constraintSupport ? box : 0.0)) * fr + half_box * S;
        b[1] = half_box * S * fz + half_mid * S;
        b[2] = 2 * half_mid * S + ntab * (double)sizeof(TabEntry<T>) + (h1 * (double)n2 + 1) * 4 + nparts * 8.0;
        if (nshells > 0) b[2] += nrfree * (8.0 + 3 * S) + (h1 * (double)n2 + 1) * 4;
        b[3] = (half_mid * S + half_box * S) * (skip ? fz : 1.0) + nparts * 8.0;
        b[4] = (half_box * S + box * Rs) * (skip ? fr : 1.0);
    }

    void profile(int count, double *ms, double *bytes) override
    {
        if (count < 1 || it_done + count > p.numIterations)
            fail(GENFIRE_ERR_STATE, "profile: iteration count out of range.");
        cudaStream_t st = ctx->stream;
        constexpr int NK = GENFIRE_PROFILE_KERNELS;
        cudaEvent_t ev[NK + 1];
        for (auto &e : ev) GF_CUDA(cudaEventCreate(&e));
        double acc[NK] = {};
        try {
            for (int i = 0; i < count; ++i) {
                enqueue_iteration(st, ev);
                GF_CUDA(cudaEventSynchronize(ev[NK]));
                for (int k = 0; k < NK; ++k) {
                    float t = 0;
                    GF_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
                    acc[k] += t;
                }
                ++it_done;
                if (p.monitor_R == 1 && it_done % p.monitorR_loopLength == 0) monitor();
            }
        } catch (...) {
            for (auto &e : ev) cudaEventDestroy(e);
            throw;
        }
        for (auto &e : ev) cudaEventDestroy(e);
        if (ms)
            for (int k = 0; k < NK; ++k) ms[k] = acc[k] / count;
        if (bytes) kernel_bytes(bytes);
    }

    void enqueue(cudaStream_t st) override { enqueue_iteration(st); }
    void prepare_capture() override { ensure_smem_attrs<T>(); }
    long long grid_points() const override { return (long long)n1 * n2 * n1; }

    cudaGraph_t capture_iteration() override
    {
        cudaStream_t st = ctx->stream;
        ensure_smem_attrs<T>();  // kernel attributes are set outside the capture
        cudaGraph_t graph = nullptr;
        GF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue_iteration(st);
        } catch (...) {
            cudaStreamEndCapture(st, &graph);
            if (graph) cudaGraphDestroy(graph);
            throw;
        }
        GF_CUDA(cudaStreamEndCapture(st, &graph));
        return graph;
    }

    void build_graph()
    {
        cudaGraph_t graph = capture_iteration();
        cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        GF_CUDA(e);
    }

    // Rfree monitor (reconstruct.m:46-69, :137-146): withheld points of each
    // shell as 0-based linear indices into the centred grid; the caller has
    // removed them from the mask given at creation.  Rebuilds the iteration graph.
    void set_rfree(int nsh, const int64_t *counts, const int64_t *ind) override
    {
        if (it_done != 0) fail(GENFIRE_ERR_STATE, "set_rfree: call before the first iteration.");
        if (nsh < 0 || (nsh > 0 && !counts)) fail(GENFIRE_ERR_ARG, "set_rfree: bad shell count.");
        cudaStream_t st = ctx->stream;
        const long long N = (long long)n1 * n2 * n1;
        std::vector<long long> off((size_t)nsh + 1, 0);
        for (int s = 0; s < nsh; ++s) {
            if (counts[s] < 0) fail(GENFIRE_ERR_ARG, "set_rfree: negative count.");
            off[s + 1] = off[s] + counts[s];
        }
        const long long tot = off[nsh];
        if (tot >= (1LL << 31)) fail(GENFIRE_ERR_ARG, "set_rfree: too many points.");
        if (tot > 0 && !ind) fail(GENFIRE_ERR_ARG, "set_rfree: indices is NULL.");
        // capture entries, CSR by F3 column (stable: slot order within a column)
        const int ncol = h1 * n2;
        std::vector<int> roff((size_t)ncol + 1, 0), colof((size_t)tot);
        std::vector<uint2> ent((size_t)tot);
        for (long long i = 0; i < tot; ++i) {
            const long long li = ind[i];
            if (li < 0 || li >= N) fail(GENFIRE_ERR_ARG, "set_rfree: index out of range.");
            const int c1 = (int)(li % n1), c2 = (int)((li / n1) % n2), c3 = (int)(li / ((long long)n1 * n2));
            // FFT position (ifftshift); the half spectrum stores q1 < h1, else the mirror -q
            int q1 = (c1 - n1 / 2 + n1) % n1, q2 = (c2 - n2 / 2 + n2) % n2, q3 = (c3 - n1 / 2 + n1) % n1;
            uint32_t conj = 0;
            if (q1 >= h1) {
                q1 = (n1 - q1) % n1; q2 = (n2 - q2) % n2; q3 = (n1 - q3) % n1;
                conj = 1;
            }
            colof[(size_t)i] = q2 * h1 + q1;
            ent[(size_t)i] = make_uint2((uint32_t)q3 | ((uint32_t)(q1 % W3) << 16), (uint32_t)i | (conj << 31));
            ++roff[(size_t)colof[(size_t)i] + 1];
        }
        for (int c = 0; c < ncol; ++c) roff[(size_t)c + 1] += roff[(size_t)c];
        std::vector<uint2> sorted((size_t)std::max(tot, 1LL));
        {
            std::vector<int> fill(roff.begin(), roff.end() - 1);
            for (long long i = 0; i < tot; ++i) sorted[(size_t)fill[(size_t)colof[(size_t)i]]++] = ent[(size_t)i];
        }
        std::vector<long long> idx(ind, ind + tot);
        rtaboff.alloc(sizeof(int) * ((size_t)ncol + 1), st);
        rtab.alloc(sizeof(uint2) * sorted.size(), st);
        rcap.alloc(sizeof(cplx<T>) * (size_t)std::max(tot, 1LL), st);
        rvals.alloc(sizeof(cplx<T>) * (size_t)std::max(tot, 1LL), st);
        rshoff.alloc(sizeof(long long) * off.size(), st);
        rhist.alloc(sizeof(double) * (size_t)std::max(nsh, 1) * std::max(p.numIterations, 1), st);
        DevBuf didx(sizeof(long long) * (size_t)std::max(tot, 1LL), st);
        GF_CUDA(cudaMemcpyAsync(rtaboff.p, roff.data(), sizeof(int) * roff.size(), cudaMemcpyHostToDevice, st));
        GF_CUDA(cudaMemcpyAsync(rtab.p, sorted.data(), sizeof(uint2) * sorted.size(), cudaMemcpyHostToDevice, st));
        GF_CUDA(cudaMemcpyAsync(rshoff.p, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice, st));
        GF_CUDA(cudaMemsetAsync(rhist.p, 0, rhist.bytes, st));
        if (tot > 0) {
            GF_CUDA(cudaMemcpyAsync(didx.p, idx.data(), sizeof(long long) * (size_t)tot, cudaMemcpyHostToDevice, st));
            k_rfree_gather<T><<<(unsigned)std::min<long long>(cdiv(tot, 256), 4096), 256, 0, st>>>(
                M.as<cplx<T>>(), didx.as<long long>(), tot, rvals.as<cplx<T>>());
            GF_CHECK_LAUNCH();
        }
        GF_CUDA(cudaStreamSynchronize(st));
        nshells = nsh;
        nrfree = tot;
        if (exec) {
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        build_graph();
    }
    // Rfree(shell, iteration) for the iterations run so far, column-major
    // (nshells x iterations); returns nshells
    int rfree(double *out) const override
    {
        if (nshells > 0 && out && it_done > 0) {
            GF_CUDA(cudaMemcpyAsync(out, rhist.p, sizeof(double) * (size_t)nshells * it_done, cudaMemcpyDeviceToHost,
                                    ctx->stream));
            GF_CUDA(cudaStreamSynchronize(ctx->stream));
        }
        return nshells;
    }

    int remaining() const override { return p.numIterations - it_done; }
    void tuning(int *v) const override
    {
        v[0] = vF2; v[1] = vF3; v[2] = vI2;
    }
    void advance() override
    {
        ++it_done;
        if (p.monitor_R == 1 && it_done % p.monitorR_loopLength == 0) monitor();
    }

    void monitor()
    {
        cudaStream_t st = ctx->stream;
        Ctl hc;
        GF_CUDA(cudaMemcpyAsync(&hc, ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
        // model = fftshift(x)(Vol_ind): the centred D1 x D2 x D1 part of the box
        const int o1 = B1 / 2 - D1 / 2, o2 = B2 / 2 - D2 / 2, o3 = B3 / 2 - D1 / 2;
        const T *base = xbuf[hc.xnext].as<T>() + (o1 + (long long)B1 * (o2 + (long long)B2 * o3));
        const int P = p.NumProjs;
        project_batch(ctx, p.precision, base, D1, D2, D1, B1, (long long)B1 * B2, P, dR.as<double>(), nullptr,
                      dmeas.as<double>(), dsums.as<double>(), st);
        std::vector<double> sums(4 * (size_t)P);
        GF_CUDA(cudaMemcpyAsync(sums.data(), dsums.p, sizeof(double) * 4 * P, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
        double s1 = 0;
        for (int i = 0; i < P; ++i) {
            const double r1 = sums[4 * i] / sums[4 * i + 1];
            const double r2 = std::sqrt(sums[4 * i + 2]) / std::sqrt(sums[4 * i + 3]);
            Rarr.push_back(r1);
            Rarr2.push_back(r2);
            s1 += r1;
        }
        errR.push_back(s1 / P);
    }

    void iterate(int count) override
    {
        if (count < 0 || it_done + count > p.numIterations)
            fail(GENFIRE_ERR_STATE, "iterate: more iterations requested than numIterations.");
        cudaStream_t st = ctx->stream;
        for (int i = 0; i < count; ++i) {
            GF_CUDA(cudaGraphLaunch(exec, st));
            ++it_done;
            if (p.monitor_R == 1 && it_done % p.monitorR_loopLength == 0) monitor();
        }
        GF_CUDA(cudaStreamSynchronize(st));
        check_device_error();
    }

    void check_device_error() override
    {
        int e = 0;
        GF_CUDA(cudaMemcpyAsync(&e, errf.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        GF_CUDA(cudaStreamSynchronize(ctx->stream));
        if (e) fail(GENFIRE_ERR_TIMEOUT, "iteration: a bounded wait of the fused column pass expired.");
    }

    void result(void *rec, double *errK, double *eR, double *RA, double *RA2, bool on_device) override
    {
        cudaStream_t st = ctx->stream;
        const size_t nv = (size_t)D1 * D2 * D1;
        DevBuf out;
        T *dout;
        if (on_device) dout = static_cast<T *>(rec);
        else { out.alloc(sizeof(T) * nv, st); dout = out.as<T>(); }
        if (rec) {
            k_extract<T><<<dim3(cdiv(D1, 256), D2, D1), 256, 0, st>>>(
                xptrs.as<T *>(), ctl.as<Ctl>(), p.constraintSupport ? S.as<uint8_t>() : nullptr,
                p.constraintPositivity, D1, D2, B1, B2, B3, dout);
            GF_CHECK_LAUNCH();
            if (!on_device) copy_host(rec, dout, sizeof(T) * nv, cudaMemcpyDeviceToHost, st);
        }
        if (errK) {
            if (on_device) GF_CUDA(cudaMemcpyAsync(errK, hist.p, sizeof(double) * it_done, cudaMemcpyDeviceToDevice, st));
            else GF_CUDA(cudaMemcpyAsync(errK, hist.p, sizeof(double) * it_done, cudaMemcpyDeviceToHost, st));
        }
        GF_CUDA(cudaStreamSynchronize(st));
        const size_t nm = errR.size(), P = (size_t)p.NumProjs;
        if (eR && nm) std::memcpy(eR, errR.data(), sizeof(double) * nm);
        if (RA && nm) std::memcpy(RA, Rarr.data(), sizeof(double) * nm * P);
        if (RA2 && nm) std::memcpy(RA2, Rarr2.data(), sizeof(double) * nm * P);
    }
};

genfire_recon *recon_create(genfire_ctx *ctx, const genfire_params &p, const void *M, const uint8_t *mask,
                            const uint8_t *support, const void *initial, const double *projs,
                            const double *angles, bool on_device)
{
    check_params(p, p.monitor_R == 1);
    if (p.numIterations < 0) fail(GENFIRE_ERR_ARG, "numIterations must be non-negative.");
    if (!M) fail(GENFIRE_ERR_ARG, "measuredK is NULL.");
    ReconBase *impl;
    if (p.precision == GENFIRE_PREC_FP64) {
        auto *r = new ReconT<double>();
        r->ctx = ctx; r->p = p;
        try { r->setup(M, mask, support, initial, projs, angles, on_device); } catch (...) { delete r; throw; }
        impl = r;
    } else {
        auto *r = new ReconT<float>();
        r->ctx = ctx; r->p = p;
        try { r->setup(M, mask, support, initial, projs, angles, on_device); } catch (...) { delete r; throw; }
        impl = r;
    }
    auto *h = new genfire_recon{ctx, impl};
    ctx->recons.insert(h);
    return h;
}

void recon_iterate(genfire_recon *r, int count) { r->impl->iterate(count); }
void recon_tuning(genfire_recon *r, int *variants) { r->impl->tuning(variants); }
void recon_set_rfree(genfire_recon *r, int nshells, const int64_t *counts, const int64_t *indices)
{
    r->impl->set_rfree(nshells, counts, indices);
}
int recon_rfree(genfire_recon *r, double *out) { return r->impl->rfree(out); }
void recon_profile(genfire_recon *r, int count, double *ms, double *bytes) { r->impl->profile(count, ms, bytes); }
void recon_result(genfire_recon *r, void *rec, double *errK, double *errR, double *Rarr, double *Rarr2, bool on_device)
{
    r->impl->result(rec, errK, errR, Rarr, Rarr2, on_device);
}
void recon_destroy(genfire_recon *r)
{
    for (genfire_recon_batch *b : r->ctx->batches)
        for (genfire_recon *m : b->members)
            if (m == r) fail(GENFIRE_ERR_STATE, "a reconstruction that belongs to a live batch: destroy the batch first.");
    r->ctx->recons.erase(r);
    delete r->impl;
    delete r;
}

// ===========================================================================
// batches: one graph holds one iteration of every member problem as
// independent child graphs, so one launch runs them all concurrently
// ===========================================================================
genfire_recon_batch *recon_batch_create(genfire_ctx *ctx, genfire_recon *const *members, int count)
{
    if (count < 1) fail(GENFIRE_ERR_ARG, "batch: at least one reconstruction.");
    for (int i = 0; i < count; ++i) {
        if (!members[i]) fail(GENFIRE_ERR_ARG, "batch: NULL reconstruction.");
        if (members[i]->ctx != ctx) fail(GENFIRE_ERR_ARG, "batch: every reconstruction must belong to the batch's context.");
        for (int j = 0; j < i; ++j)
            if (members[j] == members[i]) fail(GENFIRE_ERR_ARG, "batch: a reconstruction appears twice.");
    }
    // One graph of one iteration of every member: a fork/join capture in which
    // the members' launches go to up to 8 branch streams (largest grids first,
    // dealt round-robin), so the graph holds parallel chains of kernels and small
    // members run beside the large ones.
    auto *b = new genfire_recon_batch();
    b->ctx = ctx;
    b->members.assign(members, members + count);
    cudaGraph_t graph = nullptr;
    try {
        const int S = std::min(count, 8);
        for (int k = 0; k < S; ++k) {
            cudaStream_t s = nullptr;
            GF_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            b->branches.push_back(s);
        }
        for (int k = 0; k < S + 1; ++k) {
            cudaEvent_t e = nullptr;
            GF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            b->events.push_back(e);
        }
        std::vector<int> order(count);
        for (int i = 0; i < count; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
            return members[x]->impl->grid_points() > members[y]->impl->grid_points();
        });
        for (int i = 0; i < count; ++i) members[i]->impl->prepare_capture();
        cudaStream_t st = ctx->stream;
        GF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            GF_CUDA(cudaEventRecord(b->events[S], st));  // fork
            for (int k = 0; k < S; ++k) GF_CUDA(cudaStreamWaitEvent(b->branches[k], b->events[S], 0));
            for (int n = 0; n < count; ++n) members[order[n]]->impl->enqueue(b->branches[n % S]);
            for (int k = 0; k < S; ++k) {  // join
                GF_CUDA(cudaEventRecord(b->events[k], b->branches[k]));
                GF_CUDA(cudaStreamWaitEvent(st, b->events[k], 0));
            }
        } catch (...) {
            cudaStreamEndCapture(st, &graph);
            if (graph) cudaGraphDestroy(graph);
            graph = nullptr;
            throw;
        }
        GF_CUDA(cudaStreamEndCapture(st, &graph));
        GF_CUDA(cudaGraphInstantiate(&b->exec, graph, 0));
        cudaGraphDestroy(graph);
    } catch (...) {
        if (graph) cudaGraphDestroy(graph);
        if (b->exec) cudaGraphExecDestroy(b->exec);
        for (auto s : b->branches) cudaStreamDestroy(s);
        for (auto e : b->events) cudaEventDestroy(e);
        delete b;
        throw;
    }
    ctx->batches.insert(b);
    return b;
}

void recon_batch_iterate(genfire_recon_batch *b, int count)
{
    if (count < 0) fail(GENFIRE_ERR_ARG, "batch: negative iteration count.");
    for (genfire_recon *r : b->members)
        if (r->impl->remaining() < count)
            fail(GENFIRE_ERR_STATE, "batch: more iterations requested than a member's numIterations allows.");
    cudaStream_t st = b->ctx->stream;
    for (int i = 0; i < count; ++i) {
        GF_CUDA(cudaGraphLaunch(b->exec, st));
        for (genfire_recon *r : b->members) r->impl->advance();
    }
    GF_CUDA(cudaStreamSynchronize(st));
    for (genfire_recon *r : b->members) r->impl->check_device_error();
}

void recon_batch_destroy(genfire_recon_batch *b)
{
    cudaStreamSynchronize(b->ctx->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    for (auto s : b->branches) cudaStreamDestroy(s);
    for (auto e : b->events) cudaEventDestroy(e);
    b->ctx->batches.erase(b);
    delete b;
}

}  // namespace gf
