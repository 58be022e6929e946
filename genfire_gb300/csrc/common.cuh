// common.cuh -- shared types and helpers of libgenfire (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <set>
#include <string>
#include <vector>

#include "../../include/genfire.h"

namespace gf {

// ---------------------------------------------------------------------------
// complex arithmetic on float2 / double2
// ---------------------------------------------------------------------------
template <typename T> struct CplxOf;
template <> struct CplxOf<float> { using type = float2; };
template <> struct CplxOf<double> { using type = double2; };
template <typename T> using cplx = typename CplxOf<T>::type;

__host__ __device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
__host__ __device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { return mk(a.x + b.x, a.y + b.y); }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { return mk(a.x - b.x, a.y - b.y); }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b)
{
    return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) { return mk(a.x, -a.y); }
// twiddle application: a * w for a forward transform, a * conj(w) for an inverse one
template <typename C> __host__ __device__ __forceinline__ C ctw(C a, C w, bool inv)
{
    return inv ? mk(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y) : cmul(a, w);
}

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
struct Error {
    genfire_status st;
    std::string msg;
};

#define GF_CUDA(call)                                                                         \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            throw ::gf::Error{e_ == cudaErrorMemoryAllocation ? GENFIRE_ERR_OOM               \
                                                              : GENFIRE_ERR_CUDA,             \
                              std::string("GENFIRE: CUDA error in ") + #call + ": " +         \
                                  cudaGetErrorString(e_)};                                    \
        }                                                                                     \
    } while (0)

#define GF_CHECK_LAUNCH() GF_CUDA(cudaGetLastError())

[[noreturn]] inline void fail(genfire_status st, const std::string &m) { throw Error{st, "GENFIRE: " + m}; }

// ---------------------------------------------------------------------------
// device buffers (stream-ordered allocation on the context stream)
// ---------------------------------------------------------------------------
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaStream_t s = nullptr;
    DevBuf() = default;
    DevBuf(size_t n, cudaStream_t st) { alloc(n, st); }
    void alloc(size_t n, cudaStream_t st)
    {
        release();
        s = st;
        bytes = n;
        if (n) GF_CUDA(cudaMallocAsync(&p, n, st));
    }
    void release()
    {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        bytes = 0;
    }
    ~DevBuf() { release(); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), bytes(o.bytes), s(o.s) { o.p = nullptr; o.bytes = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept
    {
        if (this != &o) { release(); p = o.p; bytes = o.bytes; s = o.s; o.p = nullptr; o.bytes = 0; }
        return *this;
    }
    template <typename T> T *as() const { return static_cast<T *>(p); }
};

inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

// A copy between a caller's host buffer and the device.  Buffers of 64 MB and
// more are page-locked for the copy (cudaHostRegister, undone once the copy
// has completed), so the copy engines read or write them directly: copies of
// the 1 GB measured grid from pageable memory ran at 190 GB/s on some GB300
// boxes and at 8-10 GB/s on others, registration costs 2-5 ms per GB.  When
// registration fails (memory already registered, read-only or foreign
// mappings) the plain pageable copy runs.  The call returns with the copy
// complete.
constexpr size_t kPinBytes = size_t(64) << 20;
inline void copy_host(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st)
{
    void *host = kind == cudaMemcpyHostToDevice ? const_cast<void *>(src) : dst;
    bool reg = false;
    if (bytes >= kPinBytes) {
        if (cudaHostRegister(host, bytes, cudaHostRegisterDefault) == cudaSuccess) reg = true;
        else (void)cudaGetLastError();  // clear the registration error: the plain copy follows
    }
    const cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, st);
    const cudaError_t es = e == cudaSuccess ? cudaStreamSynchronize(st) : e;
    if (reg) cudaHostUnregister(host);
    GF_CUDA(es);
}
inline int floordiv2(int n) { return n / 2; }
inline int imod(long long a, long long n) { long long r = a % n; return (int)(r < 0 ? r + n : r); }

// MATLAB round(): half away from zero.
inline double mround(double x) { return x < 0 ? -std::floor(-x + 0.5) : std::floor(x + 0.5); }

}  // namespace gf

// The context behind genfire_ctx.  It tracks the reconstructions and batches
// created on it: genfire_destroy frees whatever is still alive before it
// destroys the stream they use.
struct genfire_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    int interp = GENFIRE_INTERP_TRILINEAR;  // projector interpolation (genfire_set_projector_interpolation)
    std::string last_error;
    std::set<genfire_recon *> recons;
    std::set<genfire_recon_batch *> batches;
};
