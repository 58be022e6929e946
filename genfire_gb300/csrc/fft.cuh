// fft.cuh -- Stockham FFT engine on shared-memory tiles, and the pass kernels
// the gridding and the Fourier-constraint iteration are built from.
//
// A CTA holds a tile of W independent length-n columns in shared memory as
// s[i * P + c] (i along the transform, c the column, pitch P = W + 1) and runs
// the mixed-radix Stockham stages of the plan on it.  Each stage reads the
// thread's butterflies into registers, synchronises, and writes them back, so
// one tile buffer suffices.  Twiddles come from a table tw[t] = exp(-2 pi i t / n)
// computed on the host in double precision.
//
// Layout conventions of the 3-D volumes (MATLAB column-major, dim 1 fastest):
//   half spectrum   ld1 x L2 x L3 complex, q1 in [0, h1), h1 = floor(n1/2)+1,
//                   ld1 = h1 rounded up to the tile width
//   box volume      B1 x B2 x B3 real, entry e of a dimension at position
//                   e - floor(B/2), i.e. FFT index (e - floor(B/2)) mod n.
#pragma once

#include "common.cuh"

namespace gf {

// Radix schedule packed 4 bits per stage (the radix itself, 2..13), so the
// kernels read it with shifts instead of indexing a parameter array.
struct FftPlan {
    int n;
    int nst;
    unsigned long long radices;
    __host__ __device__ int radix(int st) const { return (int)((radices >> (4 * st)) & 15ull); }
};

// Radix schedule: 8s first, then 4, 2, then the odd primes 3, 5, 7.
inline bool make_fft_plan(int n, FftPlan &pl)
{
    pl.n = n;
    pl.nst = 0;
    pl.radices = 0;
    int m = n;
    auto push = [&](int r) {
        if (pl.nst >= 16) return false;
        pl.radices |= (unsigned long long)r << (4 * pl.nst);
        ++pl.nst;
        return true;
    };
    while (m % 8 == 0) { if (!push(8)) return false; m /= 8; }
    while (m % 4 == 0) { if (!push(4)) return false; m /= 4; }
    while (m % 2 == 0) { if (!push(2)) return false; m /= 2; }
    const int odd[3] = {3, 5, 7};
    for (int f : odd)
        while (m % f == 0) {
            if (!push(f)) return false;
            m /= f;
        }
    return m == 1 && n >= 1;
}

// ---------------------------------------------------------------------------
// radix-R DFT kernels in registers: X_q = sum_r v_r exp(-+2 pi i q r / R)
// ---------------------------------------------------------------------------
template <typename C> __device__ __forceinline__ C mul_mi(C z) { return mk(z.y, -z.x); }  // -i z
template <typename C> __device__ __forceinline__ C mul_pi(C z) { return mk(-z.y, z.x); }  // +i z

template <int R, typename T> struct Dft;

template <typename T> struct Dft<2, T> {
    static __device__ __forceinline__ void run(cplx<T> *v, bool, const cplx<T> *, int)
    {
        cplx<T> a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

template <typename T> struct Dft<4, T> {
    static __device__ __forceinline__ void run(cplx<T> *v, bool inv, const cplx<T> *, int)
    {
        cplx<T> s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
        cplx<T> s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
        cplx<T> r = inv ? mul_pi(d13) : mul_mi(d13);
        v[0] = cadd(s02, s13);
        v[2] = csub(s02, s13);
        v[1] = cadd(d02, r);
        v[3] = csub(d02, r);
    }
};

template <typename T> struct Dft<8, T> {
    static __device__ __forceinline__ void run(cplx<T> *v, bool inv, const cplx<T> *tw, int n)
    {
        cplx<T> e[4] = {v[0], v[2], v[4], v[6]};
        cplx<T> o[4] = {v[1], v[3], v[5], v[7]};
        Dft<4, T>::run(e, inv, tw, n);
        Dft<4, T>::run(o, inv, tw, n);
        const T c = (T)0.70710678118654752440;
        // o[k] *= w8^k, w8 = exp(-+ i pi / 4)
        cplx<T> o1 = inv ? mk(c * (o[1].x - o[1].y), c * (o[1].x + o[1].y))
                         : mk(c * (o[1].x + o[1].y), c * (o[1].y - o[1].x));
        cplx<T> o2 = inv ? mul_pi(o[2]) : mul_mi(o[2]);
        cplx<T> o3 = inv ? mk(-c * (o[3].x + o[3].y), c * (o[3].x - o[3].y))
                         : mk(c * (o[3].y - o[3].x), -c * (o[3].x + o[3].y));
        v[0] = cadd(e[0], o[0]); v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], o1);   v[5] = csub(e[1], o1);
        v[2] = cadd(e[2], o2);   v[6] = csub(e[2], o2);
        v[3] = cadd(e[3], o3);   v[7] = csub(e[3], o3);
    }
};

// Single-precision radix 4 and 8 in packed FP32 pairs (add/sub/fma/mul
// .rn.f32x2 of sm_100-class parts: one instruction for both halves of a
// complex value).  Each pair operation rounds as the two scalar operations of
// the generic versions above, so the results are the same bit for bit;
// multiplying by -i or +i is a swap of the halves and an exact sign product.
// The twiddle products elsewhere stay scalar: their packed form needs
// (re, re) / (im, im) operand pairs, which cost more than they saved.
typedef unsigned long long f32x2_t;
__device__ __forceinline__ f32x2_t pk2(float2 a)
{
    f32x2_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 upk2(f32x2_t r)
{
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
__device__ __forceinline__ f32x2_t add2(f32x2_t a, f32x2_t b)
{
    f32x2_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2_t sub2(f32x2_t a, f32x2_t b)
{
    f32x2_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2_t mul2(f32x2_t a, f32x2_t b)
{
    f32x2_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2_t fma2(f32x2_t a, f32x2_t b, f32x2_t c)
{
    f32x2_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ f32x2_t swap2(f32x2_t a)
{
    const float2 v = upk2(a);
    return pk2(make_float2(v.y, v.x));
}

// (The order of the operations below is the one that kept the 512-point
// column pass at 91 registers; other orders of the same operations took 128.)
template <> struct Dft<4, float> {
    static __device__ __forceinline__ void run(float2 *v, bool inv, const float2 *, int)
    {
        const f32x2_t a0 = pk2(v[0]), a1 = pk2(v[1]), a2 = pk2(v[2]), a3 = pk2(v[3]);
        const f32x2_t s02 = add2(a0, a2), d02 = sub2(a0, a2), s13 = add2(a1, a3), d13 = sub2(a1, a3);
        // -i d13 (forward) = swap(d13) (1, -1); +i d13 (inverse) = swap(d13) (-1, 1)
        const f32x2_t sw = swap2(d13);
        const f32x2_t sg = inv ? pk2(make_float2(-1.f, 1.f)) : pk2(make_float2(1.f, -1.f));
        v[0] = upk2(add2(s02, s13));
        v[2] = upk2(sub2(s02, s13));
        v[1] = upk2(fma2(sw, sg, d02));
        const f32x2_t ng = inv ? pk2(make_float2(1.f, -1.f)) : pk2(make_float2(-1.f, 1.f));
        v[3] = upk2(fma2(sw, ng, d02));
    }
};

template <> struct Dft<8, float> {
    static __device__ __forceinline__ void run(float2 *v, bool inv, const float2 *tw, int n)
    {
        float2 e[4] = {v[0], v[2], v[4], v[6]};
        float2 o[4] = {v[1], v[3], v[5], v[7]};
        Dft<4, float>::run(e, inv, tw, n);
        Dft<4, float>::run(o, inv, tw, n);
        const float c = 0.70710678118654752440f;
        const f32x2_t pp = pk2(make_float2(1.f, -1.f)), mp = pk2(make_float2(-1.f, 1.f));
        const f32x2_t cc = pk2(make_float2(c, c));
        const f32x2_t o1 = pk2(o[1]), o2 = pk2(o[2]), o3 = pk2(o[3]);
        const f32x2_t s1 = swap2(o1), s2 = swap2(o2), s3 = swap2(o3);
        // o W8 = c (o + swap(o) sg), o W8^2 = swap(o) sg, o W8^3 = c (swap(o) sg - o),
        // sg = (1, -1) forward, (-1, 1) inverse (W8 = exp(-+ i pi / 4))
        const f32x2_t sg = inv ? mp : pp;
        const f32x2_t r1 = mul2(fma2(s1, sg, o1), cc);
        const f32x2_t r2 = mul2(s2, sg);
        const f32x2_t r3 = mul2(sub2(mul2(s3, sg), o3), cc);
        const f32x2_t e0 = pk2(e[0]), e1 = pk2(e[1]), e2 = pk2(e[2]), e3 = pk2(e[3]), o0 = pk2(o[0]);
        v[0] = upk2(add2(e0, o0)); v[4] = upk2(sub2(e0, o0));
        v[1] = upk2(add2(e1, r1)); v[5] = upk2(sub2(e1, r1));
        v[2] = upk2(add2(e2, r2)); v[6] = upk2(sub2(e2, r2));
        v[3] = upk2(add2(e3, r3)); v[7] = upk2(sub2(e3, r3));
    }
};

template <typename T> struct Dft<3, T> {
    static __device__ __forceinline__ void run(cplx<T> *v, bool inv, const cplx<T> *, int)
    {
        const T s3 = (T)0.86602540378443864676;
        cplx<T> t = cadd(v[1], v[2]);
        cplx<T> d = csub(v[1], v[2]);
        cplx<T> a = mk(v[0].x - (T)0.5 * t.x, v[0].y - (T)0.5 * t.y);
        cplx<T> b = mk(s3 * d.x, s3 * d.y);
        cplx<T> rb = inv ? mul_pi(b) : mul_mi(b);
        v[0] = cadd(v[0], t);
        v[1] = cadd(a, rb);
        v[2] = csub(a, rb);
    }
};

template <typename T> struct Dft<5, T> {
    static __device__ __forceinline__ void run(cplx<T> *v, bool inv, const cplx<T> *, int)
    {
        const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
        const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
        cplx<T> p14 = cadd(v[1], v[4]), m14 = csub(v[1], v[4]);
        cplx<T> p23 = cadd(v[2], v[3]), m23 = csub(v[2], v[3]);
        cplx<T> a1 = mk(v[0].x + c1 * p14.x + c2 * p23.x, v[0].y + c1 * p14.y + c2 * p23.y);
        cplx<T> a2 = mk(v[0].x + c2 * p14.x + c1 * p23.x, v[0].y + c2 * p14.y + c1 * p23.y);
        cplx<T> b1 = mk(s1 * m14.x + s2 * m23.x, s1 * m14.y + s2 * m23.y);
        cplx<T> b2 = mk(s2 * m14.x - s1 * m23.x, s2 * m14.y - s1 * m23.y);
        cplx<T> r1 = inv ? mul_pi(b1) : mul_mi(b1);
        cplx<T> r2 = inv ? mul_pi(b2) : mul_mi(b2);
        v[0] = mk(v[0].x + p14.x + p23.x, v[0].y + p14.y + p23.y);
        v[1] = cadd(a1, r1); v[4] = csub(a1, r1);
        v[2] = cadd(a2, r2); v[3] = csub(a2, r2);
    }
};

// Radix 7: direct O(R^2) sum with roots taken from the table.
template <int R, typename T> struct DftGeneric {
    static __device__ __forceinline__ void run(cplx<T> *v, bool inv, const cplx<T> *tw, int n)
    {
        cplx<T> o[R];
        const int step = n / R;
#pragma unroll
        for (int q = 0; q < R; ++q) {
            cplx<T> acc = v[0];
#pragma unroll
            for (int r = 1; r < R; ++r) acc = cadd(acc, ctw(v[r], tw[((q * r) % R) * step], inv));
            o[q] = acc;
        }
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = o[q];
    }
};
template <typename T> struct Dft<7, T> : DftGeneric<7, T> {};

// One Stockham stage on the tile.  Ns is the product of the radices already
// applied.  The host chooses blockDim >= n*W/8, so no thread owns more than
// ceil(8/R) butterflies.
template <int R, typename T>
__device__ __forceinline__ void fft_stage(cplx<T> *s, int n, int W, int P, int Ns,
                                          const cplx<T> *__restrict__ tw, bool inv)
{
    constexpr int MAXB = (8 + R - 1) / R;
    const int m = n / R;
    const int nb = m * W;
    const int nt = blockDim.x;
    cplx<T> v[MAXB][R];
#pragma unroll
    for (int k = 0; k < MAXB; ++k) {
        const int b = threadIdx.x + k * nt;
        if (b < nb) {
            const int j = b / W, c = b - j * W;
#pragma unroll
            for (int r = 0; r < R; ++r) v[k][r] = s[(j + r * m) * P + c];
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < MAXB; ++k) {
        const int b = threadIdx.x + k * nt;
        if (b < nb) {
            const int j = b / W, c = b - j * W;
            const int kk = j % Ns;
            if (Ns > 1) {
                const int step = n / (Ns * R);
#pragma unroll
                for (int r = 1; r < R; ++r) v[k][r] = ctw(v[k][r], tw[kk * r * step], inv);
            }
            Dft<R, T>::run(v[k], inv, tw, n);
            const int base = (j - kk) * R + kk;
#pragma unroll
            for (int r = 0; r < R; ++r) s[(base + r * Ns) * P + c] = v[k][r];
        }
    }
    __syncthreads();
}

template <typename T>
__device__ __noinline__ void fft_tile(cplx<T> *s, const FftPlan pl, int W, int P, const cplx<T> *__restrict__ tw,
                                     bool inv)
{
    int Ns = 1;
    for (int st = 0; st < pl.nst; ++st) {
        const int R = pl.radix(st);
        switch (R) {
        case 8: fft_stage<8, T>(s, pl.n, W, P, Ns, tw, inv); break;
        case 4: fft_stage<4, T>(s, pl.n, W, P, Ns, tw, inv); break;
        case 2: fft_stage<2, T>(s, pl.n, W, P, Ns, tw, inv); break;
        case 3: fft_stage<3, T>(s, pl.n, W, P, Ns, tw, inv); break;
        case 5: fft_stage<5, T>(s, pl.n, W, P, Ns, tw, inv); break;
        default: fft_stage<7, T>(s, pl.n, W, P, Ns, tw, inv); break;
        }
        Ns *= R;
    }
}

__device__ __forceinline__ int wrap(int a, int n)
{
    a %= n;
    return a < 0 ? a + n : a;
}

// Largest CTA of a tile pass: 512 threads for complex64 tiles (n*W <= 4096),
// 256 for complex128 tiles (n*W <= 2048), 8 elements per thread.
template <typename T> constexpr int kTileMaxThreads = sizeof(T) == 4 ? 512 : 256;

// ---------------------------------------------------------------------------
// Fourier-constraint table entry (one per half-spectrum point q that is in E
// or whose Hermitian mate -q is in E).  See the iteration kernel below.
// ---------------------------------------------------------------------------
template <typename T> struct TabEntry {
    uint32_t pos;     // q3 | (q1 - tile*W) << 16
    uint32_t eflags;  // bit0: q in E; bit1: -q in E and -q is not a stored point
    uint32_t cq;      // bit c: q in C while delay index c is in force
    uint32_t cmq;     // bit c: -q in C while delay index c is in force
    cplx<T> Mq;       // measuredK(q)
    cplx<T> Mmq;      // measuredK(-q)
};

// ---------------------------------------------------------------------------
// Control block of the iteration, in device memory, so one iteration is a
// fixed sequence of launches (a CUDA graph).  Its two updates run inside the
// passes, in CTA 0 of a pass where nothing else reads what they change: the
// start of an iteration in the first row pass, the errK reduction and the
// best-object bookkeeping in the dim-2 inverse pass.
// ---------------------------------------------------------------------------
struct Ctl {
    int it;           // iterations completed
    int cur;          // next entry of the change-point list (0-based currentCutoffNum)
    int cidx;         // delay indicator in force
    int xcur;         // buffer holding the current object
    int xnext;        // buffer the next object is written to
    int xbest;        // buffer holding the best object (-1: none yet)
    int m;            // number of delay indicators
    int pad;
    double bestErr;
    double errK;
};

// reconstruct.m:118-124 (one thread)
__device__ __forceinline__ void ctl_begin_update(Ctl *c, const int *__restrict__ changes)
{
    c->xcur = c->xnext;
    const int it = ++c->it;
    if (c->cur < c->m && it == changes[c->cur]) {
        int last = c->cur;
        for (int k = 0; k < c->m; ++k)
            if (changes[k] == it) last = k;
        c->cidx = last;
        c->cur = last + 1;
        c->bestErr = 1e30;
    }
}

// reconstruct.m:135 and :149-153, run by all threads of CTA 0 of the pass
// after the fused dim-3 pass (the dim-2 inverse, which itself needs neither
// errK nor the output buffer; the pass after it does): sums the fused pass's
// per-CTA errK partials in a fixed order (each thread a contiguous slice, then
// a fixed tree) and updates errK, the best object and the output buffer.
static __device__ __noinline__ void ctl_mid_update(Ctl *c, const double *partial, int np, double denom,
                                                   double *hist)
{
    __shared__ double red[32];
    const int nt = blockDim.x;
    const int per = (np + nt - 1) / nt;
    const int b = threadIdx.x * per, e = min(b + per, np);
    double s = 0;
    for (int i = b; i < e; ++i) s += partial[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0;
        for (int w = 0; w < (nt + 31) / 32; ++w) v += red[w];
        const double err = v / denom;
        c->errK = err;
        hist[c->it - 1] = err;
        if (err < c->bestErr) {
            c->bestErr = err;
            c->xbest = c->xcur;
        }
        c->xnext = (c->xbest == c->xcur) ? 1 - c->xcur : c->xcur;
    }
}

// ---------------------------------------------------------------------------
// Column pass: length-n transforms along a strided dimension, W columns per
// CTA.  Column c of tile t is element (t*W + c) * col_stride; entry e along
// the transform is at e * dim_stride; blockIdx.y selects the "other"
// dimension (offset other * other_stride).  Input entries e in [0, in_cnt)
// sit at FFT index (e - in_c) mod n (the rest is zero); output entries are
// read back the same way.
// mode bit 0: forward, bit 1: inverse (after the forward), bit 2: apply the
// Fourier-constraint table between them.
// ---------------------------------------------------------------------------
template <typename T> struct ColPassArgs {
    FftPlan pl;
    const cplx<T> *tw;
    int W, P;
    int ncols;
    long long col_stride;
    const cplx<T> *in;
    long long in_dim, in_other;
    int in_cnt, in_c;
    cplx<T> *out;
    long long out_dim, out_other;
    int out_cnt, out_c;
    int mode;
    T scale;  // multiplies stored values
    // constraint table (mode bit 2)
    const int *tab_off;     // CSR offsets over columns q1 + h1 * other
    const TabEntry<T> *tab;
    int h1;
    double *partial;        // one errK partial sum per CTA
    const int *cidx;        // current delay index (device)
    // with ctl set (the iteration's dim-2 inverse pass): CTA 0 first reduces
    // the fused pass's partials (nparts of them) into errK and updates the
    // best object (ctl_mid_update)
    Ctl *ctl;
    int nparts;
    double denom;
    double *hist;
    // Rfree monitor (mode bit 2 only; NULL when off): entries CSR by column as
    // tab, each {pos as in TabEntry, slot | conj << 31}; the spectrum value at
    // pos (conjugated for a withheld point whose mirror is the stored one) is
    // copied to rcap[slot] before the Fourier constraint changes the tile
    const int *rtab_off;
    const uint2 *rtab;
    cplx<T> *rcap;
    // set to 1 by a pass whose bounded device-side wait expired (NULL: none)
    int *err;
    // radix-32 column passes: per value of `other`, nonzero when that slab of
    // the box holds a support voxel.  For the other slabs a forward pass whose
    // input there is zero (zmask_zero = 1) writes zeros without transforming,
    // and an inverse pass whose output there is never read (zmask_zero = 0)
    // does nothing (nullptr: every CTA works)
    const uint8_t *zmask;
    int zmask_zero;
};

// Copy of the withheld (Rfree) points of one tile of F3, read before the
// constraint; idx maps (q3, column in tile) to the tile's shared-memory slot.
// The caller synchronises before the constraint writes the tile.
template <typename T, class Idx>
__device__ __forceinline__ void capture_rfree(const cplx<T> *s, const ColPassArgs<T> &a, int tile, int W, int other,
                                              Idx idx)
{
    const int cid0 = other * a.h1 + tile * W;
    const int cid1 = min(cid0 + W, other * a.h1 + a.h1);
    const int e1 = a.rtab_off[cid1];
    for (int e = a.rtab_off[cid0] + threadIdx.x; e < e1; e += blockDim.x) {
        const uint2 t = a.rtab[e];
        const cplx<T> k = s[idx((int)(t.x & 0xFFFFu), (int)(t.x >> 16))];
        a.rcap[t.y & 0x7FFFFFFFu] = (t.y >> 31) ? cconj(k) : k;
    }
}

template <typename T>
__global__ void __launch_bounds__(kTileMaxThreads<T>) k_colpass(ColPassArgs<T> a)
{
    if (a.ctl && blockIdx.x == 0 && blockIdx.y == 0) ctl_mid_update(a.ctl, a.partial, a.nparts, a.denom, a.hist);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *s = reinterpret_cast<cplx<T> *>(smem_raw);
    const int n = a.pl.n, W = a.W, P = a.P;
    const int tile = blockIdx.x, other = blockIdx.y;
    const int nt = blockDim.x, tid = threadIdx.x;
    const cplx<T> zero = mk((T)0, (T)0);

    for (int i = tid; i < n * P; i += nt) s[i] = zero;
    __syncthreads();
    const cplx<T> *in = a.in + (long long)other * a.in_other;
    if (a.col_stride == 1) {
        for (int idx = tid; idx < a.in_cnt * W; idx += nt) {
            const int e = idx / W, c = idx - e * W;
            const int col = tile * W + c;
            if (col < a.ncols) s[wrap(e - a.in_c, n) * P + c] = in[(long long)col + (long long)e * a.in_dim];
        }
    } else {
        for (int idx = tid; idx < a.in_cnt * W; idx += nt) {
            const int c = idx / a.in_cnt, e = idx - c * a.in_cnt;
            const int col = tile * W + c;
            if (col < a.ncols)
                s[wrap(e - a.in_c, n) * P + c] = in[(long long)col * a.col_stride + (long long)e * a.in_dim];
        }
    }
    __syncthreads();
    if (a.mode & 1) fft_tile<T>(s, a.pl, W, P, a.tw, false);
    if ((a.mode & 4) && a.rtab) {
        capture_rfree<T>(s, a, tile, W, other, [P](int q3, int cl) { return q3 * P + cl; });
        __syncthreads();
    }
    if (a.mode & 4) {
        // Fourier constraint on the half spectrum (reconstruct.m:135 and :163-165):
        // H(q) = (A(q) + conj(A(-q))) / 2 with A = measuredK on C and the
        // current spectrum elsewhere; A(-q) of a real object's spectrum is
        // conj(k(q)), so H = k outside C.  errK terms use |k(-q)| = |k(q)|.
        const int cid0 = other * a.h1 + tile * W;
        const int cid1 = min(cid0 + W, other * a.h1 + a.h1);
        const int e0 = a.tab_off[cid0], e1 = a.tab_off[cid1];
        const int ci = *a.cidx;
        double acc = 0.0;
        for (int e = e0 + tid; e < e1; e += nt) {
            const TabEntry<T> t = a.tab[e];
            const int q3 = t.pos & 0xFFFF, cl = t.pos >> 16;
            cplx<T> k = s[q3 * P + cl];
            const T mk_ = sqrt(k.x * k.x + k.y * k.y);
            if (t.eflags & 1u) {
                const T mq = sqrt(t.Mq.x * t.Mq.x + t.Mq.y * t.Mq.y);
                acc += fabs((double)mk_ - (double)mq);
            }
            if (t.eflags & 2u) {
                const T mm = sqrt(t.Mmq.x * t.Mmq.x + t.Mmq.y * t.Mmq.y);
                acc += fabs((double)mk_ - (double)mm);
            }
            const bool eq = (t.cq >> ci) & 1u, emq = (t.cmq >> ci) & 1u;
            if (eq || emq) {
                const cplx<T> A = eq ? t.Mq : k;
                const cplx<T> B = emq ? cconj(t.Mmq) : k;
                s[q3 * P + cl] = mk((T)0.5 * (A.x + B.x), (T)0.5 * (A.y + B.y));
            }
        }
        // deterministic block reduction of the errK partial
        __shared__ double red[32];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if ((tid & 31) == 0) red[tid >> 5] = acc;
        __syncthreads();
        if (tid < 32) {
            double v = (tid < (nt + 31) / 32) ? red[tid] : 0.0;
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (tid == 0) a.partial[(long long)other * gridDim.x + tile] = v;
        }
        __syncthreads();
    }
    if (a.mode & 2) fft_tile<T>(s, a.pl, W, P, a.tw, true);
    cplx<T> *out = a.out + (long long)other * a.out_other;
    if (a.col_stride == 1) {
        for (int idx = tid; idx < a.out_cnt * W; idx += nt) {
            const int e = idx / W, c = idx - e * W;
            const int col = tile * W + c;
            if (col < a.ncols) {
                cplx<T> v = s[wrap(e - a.out_c, n) * P + c];
                out[(long long)col + (long long)e * a.out_dim] = mk(v.x * a.scale, v.y * a.scale);
            }
        }
    } else {
        for (int idx = tid; idx < a.out_cnt * W; idx += nt) {
            const int c = idx / a.out_cnt, e = idx - c * a.out_cnt;
            const int col = tile * W + c;
            if (col < a.ncols) {
                cplx<T> v = s[wrap(e - a.out_c, n) * P + c];
                out[(long long)col * a.col_stride + (long long)e * a.out_dim] = mk(v.x * a.scale, v.y * a.scale);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Row passes along dimension 1 between a real box volume and the half
// spectrum.  Two real rows travel in one complex transform (z = x_a + i x_b).
// ---------------------------------------------------------------------------
struct Ctl;  // iteration control block (dr.cu)

template <typename T> struct RowPassArgs {
    FftPlan pl;
    const cplx<T> *tw;
    int W, P;          // row pairs per CTA, smem pitch
    int nrows;         // B2 * B3 real rows
    int B1, c1;        // box length along dim 1 and its centre floor(B1/2)
    int h1, ld1;
    // real side: x = xs[*xsel] when xsel != nullptr, else xs[0]
    T *xs[2];
    const int *xsel;
    const uint8_t *support;  // box-shaped support mask, nullptr for none
    // per row pair, nonzero when one of its two rows holds a support voxel;
    // a CTA whose row pairs are all zero writes zero half spectra (forward) or
    // nothing (inverse: set only when nothing else reads that output)
    const uint8_t *pairmask;
    int positivity;
    cplx<T> *Y;        // ld1 x nrows half spectrum
    T scale;           // inverse only
    // with ctl set (the iteration's first pass): CTA 0 starts the iteration
    // (ctl_begin_update) while every CTA reads the object from xs[ctl->xnext]
    Ctl *ctl;
    const int *changes;
};

// The CTA's row pairs [blockIdx.x W, (blockIdx.x + 1) W) hold no support voxel
// (RowPassArgs::pairmask); every thread reaches the same answer.  The W loads
// are independent (no early exit), so they cost one memory latency.
template <typename T> __device__ __forceinline__ bool row_pairs_empty(const RowPassArgs<T> &a, int W)
{
    if (!a.pairmask) return false;
    const int npairs = (a.nrows + 1) / 2;
    int any = 0;
    for (int c = 0; c < W; ++c) {
        const int p = blockIdx.x * W + c;
        if (p < npairs) any |= a.pairmask[p];
    }
    return any == 0;
}
// A forward row pass's output for such a CTA: its rows are zero after the
// support constraint, and so are their half spectra.
template <typename T> __device__ __forceinline__ void zero_half_rows(const RowPassArgs<T> &a, int W)
{
    const int r0 = blockIdx.x * W * 2;
    for (int i = threadIdx.x; i < 2 * W * a.h1; i += blockDim.x) {
        const int rr = i / a.h1, q = i - rr * a.h1;
        if (r0 + rr < a.nrows) a.Y[(long long)(r0 + rr) * a.ld1 + q] = mk((T)0, (T)0);
    }
}

// forward: real rows (after positivity and support, reconstruct.m:126-131) -> half spectrum
template <typename T>
__global__ void __launch_bounds__(kTileMaxThreads<T>) k_rows_r2c(RowPassArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *s = reinterpret_cast<cplx<T> *>(smem_raw);
    const int n = a.pl.n, W = a.W, P = a.P, tid = threadIdx.x, nt = blockDim.x;
    if (a.ctl && blockIdx.x == 0 && threadIdx.x == 0) ctl_begin_update(a.ctl, a.changes);
    if (row_pairs_empty(a, W)) {
        zero_half_rows(a, W);
        return;
    }
    const T *x = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int r0base = blockIdx.x * W * 2;
    for (int i = tid; i < n * P; i += nt) s[i] = mk((T)0, (T)0);
    __syncthreads();
    for (int idx = tid; idx < W * a.B1; idx += nt) {
        const int c = idx / a.B1, e = idx - c * a.B1;
        const int r0 = r0base + 2 * c, r1 = r0 + 1;
        T va = 0, vb = 0;
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
        s[wrap(e - a.c1, n) * P + c] = mk(va, vb);
    }
    __syncthreads();
    fft_tile<T>(s, a.pl, W, P, a.tw, false);
    for (int idx = tid; idx < W * a.h1; idx += nt) {
        const int c = idx / a.h1, q = idx - c * a.h1;
        const int r0 = r0base + 2 * c, r1 = r0 + 1;
        const cplx<T> Z = s[q * P + c];
        const cplx<T> Zm = s[(q == 0 ? 0 : n - q) * P + c];
        // X_a = (Z + conj(Zm)) / 2,  X_b = (Z - conj(Zm)) / (2i)
        const cplx<T> Xa = mk((T)0.5 * (Z.x + Zm.x), (T)0.5 * (Z.y - Zm.y));
        const cplx<T> Xb = mk((T)0.5 * (Z.y + Zm.y), (T)0.5 * (Zm.x - Z.x));
        if (r0 < a.nrows) a.Y[(long long)r0 * a.ld1 + q] = Xa;
        if (r1 < a.nrows) a.Y[(long long)r1 * a.ld1 + q] = Xb;
    }
}

// inverse: half spectrum -> real rows restricted to the box (C2R; the
// imaginary parts at q1 = 0 and q1 = n1/2 are dropped as real() does)
template <typename T>
__global__ void __launch_bounds__(kTileMaxThreads<T>) k_rows_c2r(RowPassArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *s = reinterpret_cast<cplx<T> *>(smem_raw);
    const int n = a.pl.n, W = a.W, P = a.P, tid = threadIdx.x, nt = blockDim.x;
    if (row_pairs_empty(a, W)) return;
    T *x = (a.xsel && *a.xsel) ? a.xs[1] : a.xs[0];
    const int r0base = blockIdx.x * W * 2;
    for (int idx = tid; idx < W * a.h1; idx += nt) {
        const int c = idx / a.h1, q = idx - c * a.h1;
        const int r0 = r0base + 2 * c, r1 = r0 + 1;
        cplx<T> ha = mk((T)0, (T)0), hb = ha;
        if (r0 < a.nrows) ha = a.Y[(long long)r0 * a.ld1 + q];
        if (r1 < a.nrows) hb = a.Y[(long long)r1 * a.ld1 + q];
        if (q == 0 || 2 * q == n) { ha.y = 0; hb.y = 0; }
        s[q * P + c] = mk(ha.x - hb.y, ha.y + hb.x);
        if (q != 0 && n - q >= a.h1) s[(n - q) * P + c] = mk(ha.x + hb.y, hb.x - ha.y);
    }
    __syncthreads();
    fft_tile<T>(s, a.pl, W, P, a.tw, true);
    for (int idx = tid; idx < W * a.B1; idx += nt) {
        const int c = idx / a.B1, e = idx - c * a.B1;
        const int r0 = r0base + 2 * c, r1 = r0 + 1;
        const cplx<T> z = s[wrap(e - a.c1, n) * P + c];
        if (r0 < a.nrows) x[(long long)r0 * a.B1 + e] = z.x * a.scale;
        if (r1 < a.nrows) x[(long long)r1 * a.B1 + e] = z.y * a.scale;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <typename T> const cplx<T> *twiddles(int n, cudaStream_t s);  // cached per device

// Threads for a tile of W columns of length n: at most 8 elements per thread
// (n * W <= 4096 keeps this within 512 threads).
inline int tile_threads(int n, int W)
{
    int t = (n * W + 7) / 8;
    t = (t + 31) / 32 * 32;
    if (t < 32) t = 32;
    return t;
}
template <typename T> inline size_t tile_smem(int n, int W) { return (size_t)n * (W + 1) * sizeof(cplx<T>); }

// Tile width (columns per CTA) for a transform length: at most
// 8 * kTileMaxThreads elements per tile.
template <typename T> inline int tile_width(int n)
{
    int W = sizeof(T) == 4 ? 8 : 4;
    while (W > 1 && n * W > 8 * kTileMaxThreads<T>) W /= 2;
    return W;
}

}  // namespace gf
