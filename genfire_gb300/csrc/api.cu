// api.cu -- the extern "C" entry points of libgenfire.so (declared in
// include/genfire.h).  Each call validates its arguments the way the
// reference's error() guards do (GENFIRE_Reconstructor.m:87-221), moves host
// data to the device when needed, runs the kernels on the context stream and
// returns a status; exceptions never cross the C boundary.
#include "internal.h"

#include <cstring>
#include <functional>

using gf::DevBuf;
using gf::Error;

namespace {

thread_local std::string g_noctx_error;

genfire_status guarded(genfire_ctx *ctx, const std::function<void()> &fn)
{
    try {
        if (ctx) {
            GF_CUDA(cudaSetDevice(ctx->device));
            ctx->last_error.clear();
        }
        fn();
        return GENFIRE_OK;
    } catch (const Error &e) {
        if (ctx) ctx->last_error = e.msg;
        else g_noctx_error = e.msg;
        return e.st;
    } catch (const std::bad_alloc &) {
        if (ctx) ctx->last_error = "GENFIRE: host memory exhausted";
        return GENFIRE_ERR_OOM;
    } catch (...) {
        if (ctx) ctx->last_error = "GENFIRE: unexpected internal error";
        return GENFIRE_ERR_STATE;
    }
}

void need(const void *ptr, const char *what)
{
    if (!ptr) gf::fail(GENFIRE_ERR_ARG, std::string(what) + " is NULL.");
}

size_t real_size(int precision) { return precision == GENFIRE_PREC_FP64 ? sizeof(double) : sizeof(float); }

}  // namespace

extern "C" {

int32_t genfire_abi_version(void) { return GENFIRE_ABI_VERSION; }

const char *genfire_status_string(genfire_status s)
{
    switch (s) {
    case GENFIRE_OK: return "ok";
    case GENFIRE_ERR_ARG: return "invalid argument";
    case GENFIRE_ERR_OOM: return "out of memory";
    case GENFIRE_ERR_CUDA: return "CUDA error";
    case GENFIRE_ERR_TIMEOUT: return "device wait timed out";
    case GENFIRE_ERR_UNSUPPORTED: return "unsupported size";
    case GENFIRE_ERR_STATE: return "invalid state";
    }
    return "unknown status";
}

genfire_status genfire_params_init(genfire_params *p)
{
    if (!p) return GENFIRE_ERR_ARG;
    std::memset(p, 0, sizeof(*p));
    // GENFIRE_Reconstructor.m:30-70
    p->DFT_CentroSymmetricity = 1;
    p->oversamplingRatio = 3;
    p->interpolationCutoffDistance = 0.7;
    p->vector1[2] = 1;  // [0 0 1]
    p->vector2[1] = 1;  // [0 1 0]
    p->vector3[0] = 1;  // [1 0 0]
    p->numIterations = 50;
    p->constraintEnforcementMode = 1;
    p->constraintPositivity = 1;
    p->constraintSupport = 1;
    p->monitor_R = 0;
    p->monitorR_loopLength = 10;
    p->precision = GENFIRE_PREC_FP64;
    p->griddingMethod = 2;            // the C entry points name their method; sizes default to DFT
    p->allowMultipleGridMatches = 1;  // GENFIRE_Reconstructor.m:46
    return GENFIRE_OK;
}

genfire_status genfire_grid_size(const genfire_params *p, int32_t *n1, int32_t *n2)
{
    if (!p || !n1 || !n2) return GENFIRE_ERR_ARG;
    if (p->griddingMethod == 1) {
        const int m = gf::fft_grid_size(p->Dim2, p->oversamplingRatio);
        if (m < 0) return GENFIRE_ERR_ARG;
        *n1 = *n2 = m;
        return GENFIRE_OK;
    }
    *n1 = gf::oversampled(p->Dim1, p->oversamplingRatio);
    *n2 = gf::oversampled(p->Dim2, p->oversamplingRatio);
    return GENFIRE_OK;
}

genfire_status genfire_create(int32_t device, genfire_ctx **out)
{
    if (!out) return GENFIRE_ERR_ARG;
    *out = nullptr;
    genfire_ctx *c = new genfire_ctx();
    c->device = device;
    genfire_status st = guarded(nullptr, [&] {
        int n = 0;
        GF_CUDA(cudaGetDeviceCount(&n));
        if (device < 0 || device >= n) gf::fail(GENFIRE_ERR_ARG, "device index out of range.");
        GF_CUDA(cudaSetDevice(device));
        GF_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        GF_CUDA(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device));
        // keep memory freed by the library's stream-ordered allocations in the
        // device's pool instead of returning it to the driver at each
        // synchronisation, so repeated calls do not re-map gigabytes
        cudaMemPool_t pool;
        GF_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
        uint64_t keep = UINT64_MAX;
        GF_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    });
    if (st != GENFIRE_OK) {
        delete c;
        return st;
    }
    *out = c;
    return GENFIRE_OK;
}

genfire_status genfire_destroy(genfire_ctx *ctx)
{
    if (!ctx) return GENFIRE_OK;
    cudaSetDevice(ctx->device);
    // batches and reconstructions still alive use this context's stream: free them first
    while (!ctx->batches.empty()) gf::recon_batch_destroy(*ctx->batches.begin());
    // (recon_destroy lives where the reconstruction type is complete, so its
    // destructor runs: a delete here, of an incomplete type, would free the
    // object without releasing its device buffers and graph)
    while (!ctx->recons.empty()) gf::recon_destroy(*ctx->recons.begin());
    if (ctx->stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
    }
    delete ctx;
    return GENFIRE_OK;
}

const char *genfire_last_error(const genfire_ctx *ctx) { return ctx ? ctx->last_error.c_str() : g_noctx_error.c_str(); }

void *genfire_stream(genfire_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

// ---------------------------------------------------------------- gridding
genfire_status genfire_grid_dft_device(genfire_ctx *ctx, const genfire_params *p, const double *d_projections,
                                       const double *angles, void *d_measuredK, void *d_recIFFT, int64_t *nk)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(p, "params");
        need(d_projections, "projections");
        need(angles, "angles");
        need(d_measuredK, "measuredK");
        gf::check_params(*p, true);
        gf::grid_dft(ctx, *p, d_projections, angles, d_measuredK, d_recIFFT, nk);
    });
}

genfire_status genfire_grid_dft(genfire_ctx *ctx, const genfire_params *p, const double *projections,
                                const double *angles, void *measuredK, void *recIFFT, int64_t *nk)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(p, "params");
        need(projections, "projections");
        need(angles, "angles");
        need(measuredK, "measuredK");
        gf::check_params(*p, true);
        cudaStream_t st = ctx->stream;
        const int n1 = gf::oversampled(p->Dim1, p->oversamplingRatio);
        const int n2 = gf::oversampled(p->Dim2, p->oversamplingRatio);
        const size_t npj = (size_t)p->Dim1 * p->Dim2 * p->NumProjs;
        const size_t nM = (size_t)n1 * n2 * n1 * 2 * real_size(p->precision);
        const size_t nR = (size_t)p->Dim1 * p->Dim2 * p->Dim1 * real_size(p->precision);
        DevBuf dp(sizeof(double) * npj, st), dM(nM, st), dR;
        if (recIFFT) dR.alloc(nR, st);
        GF_CUDA(cudaMemcpyAsync(dp.p, projections, sizeof(double) * npj, cudaMemcpyHostToDevice, st));
        gf::grid_dft(ctx, *p, dp.as<double>(), angles, dM.p, recIFFT ? dR.p : nullptr, nk);
        gf::copy_host(measuredK, dM.p, nM, cudaMemcpyDeviceToHost, st);
        if (recIFFT) gf::copy_host(recIFFT, dR.p, nR, cudaMemcpyDeviceToHost, st);
        GF_CUDA(cudaStreamSynchronize(st));
    });
}

genfire_status genfire_grid_profile(genfire_ctx *ctx, const genfire_params *p, const double *d_projections,
                                    const double *angles, void *d_measuredK, double *stage_ms)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(p, "params");
        need(d_projections, "projections");
        need(angles, "angles");
        need(d_measuredK, "measuredK");
        need(stage_ms, "stage_ms");
        gf::check_params(*p, true);
        gf::grid_dft(ctx, *p, d_projections, angles, d_measuredK, nullptr, nullptr, stage_ms);
    });
}

genfire_status genfire_grid_fft_device(genfire_ctx *ctx, const genfire_params *p, const double *d_projections,
                                       const double *angles, void *d_measuredK, void *d_recIFFT, int64_t *npairs)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(p, "params");
        need(d_projections, "projections");
        need(angles, "angles");
        need(d_measuredK, "measuredK");
        gf::check_params(*p, true);
        gf::grid_fft(ctx, *p, d_projections, angles, d_measuredK, d_recIFFT, npairs);
    });
}

genfire_status genfire_grid_fft(genfire_ctx *ctx, const genfire_params *p, const double *projections,
                                const double *angles, void *measuredK, void *recIFFT, int64_t *npairs)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(p, "params");
        need(projections, "projections");
        need(angles, "angles");
        need(measuredK, "measuredK");
        gf::check_params(*p, true);
        const int m = gf::fft_grid_size(p->Dim2, p->oversamplingRatio);
        if (m < 0)
            gf::fail(GENFIRE_ERR_ARG, "FFT gridding: Dim2 * oversamplingRatio (1 + (Dim2-1) * oversamplingRatio "
                                      "for odd Dim2) must be an integer.");
        cudaStream_t st = ctx->stream;
        const size_t npj = (size_t)p->Dim1 * p->Dim2 * p->NumProjs;
        const size_t nM = (size_t)m * m * m * 2 * real_size(p->precision);
        const size_t nR = (size_t)p->Dim1 * p->Dim2 * p->Dim1 * real_size(p->precision);
        DevBuf dp(sizeof(double) * npj, st), dM(nM, st), dR;
        if (recIFFT) dR.alloc(nR, st);
        GF_CUDA(cudaMemcpyAsync(dp.p, projections, sizeof(double) * npj, cudaMemcpyHostToDevice, st));
        gf::grid_fft(ctx, *p, dp.as<double>(), angles, dM.p, recIFFT ? dR.p : nullptr, npairs);
        gf::copy_host(measuredK, dM.p, nM, cudaMemcpyDeviceToHost, st);
        if (recIFFT) gf::copy_host(recIFFT, dR.p, nR, cudaMemcpyDeviceToHost, st);
        GF_CUDA(cudaStreamSynchronize(st));
    });
}

// ---------------------------------------------------------------- iteration
genfire_status genfire_recon_create(genfire_ctx *ctx, const genfire_params *p, const void *measuredK,
                                    const uint8_t *measuredK_mask, const uint8_t *support, const void *initialObject,
                                    const double *projections, const double *angles, int32_t on_device,
                                    genfire_recon **out)
{
    if (!ctx || !out) return GENFIRE_ERR_ARG;
    *out = nullptr;
    return guarded(ctx, [&] {
        need(p, "params");
        *out = gf::recon_create(ctx, *p, measuredK, measuredK_mask, support, initialObject, projections, angles,
                                on_device != 0);
    });
}

genfire_status genfire_recon_iterate(genfire_recon *r, int32_t count)
{
    if (!r) return GENFIRE_ERR_ARG;
    genfire_ctx *ctx = r->ctx;
    return guarded(ctx, [&] { gf::recon_iterate(r, count); });
}

genfire_status genfire_recon_result(genfire_recon *r, void *reconstruction, double *errK, double *errR, double *Rarr,
                                    double *Rarr2, int32_t on_device)
{
    if (!r) return GENFIRE_ERR_ARG;
    genfire_ctx *ctx = r->ctx;
    return guarded(ctx, [&] { gf::recon_result(r, reconstruction, errK, errR, Rarr, Rarr2, on_device != 0); });
}

genfire_status genfire_recon_destroy(genfire_recon *r)
{
    if (!r) return GENFIRE_OK;
    genfire_ctx *ctx = r->ctx;
    return guarded(ctx, [&] { gf::recon_destroy(r); });
}

genfire_status genfire_recon_batch_create(genfire_ctx *ctx, int32_t count, genfire_recon *const *members,
                                          genfire_recon_batch **out)
{
    if (!ctx || !out) return GENFIRE_ERR_ARG;
    *out = nullptr;
    return guarded(ctx, [&] {
        need(members, "members");
        *out = gf::recon_batch_create(ctx, members, count);
    });
}

genfire_status genfire_recon_batch_iterate(genfire_recon_batch *b, int32_t count)
{
    if (!b) return GENFIRE_ERR_ARG;
    return guarded(b->ctx, [&] { gf::recon_batch_iterate(b, count); });
}

genfire_status genfire_recon_batch_destroy(genfire_recon_batch *b)
{
    if (!b) return GENFIRE_OK;
    genfire_ctx *ctx = b->ctx;
    return guarded(ctx, [&] { gf::recon_batch_destroy(b); });
}

genfire_status genfire_recon_tuning(genfire_recon *r, int32_t *variants)
{
    if (!r || !variants) return GENFIRE_ERR_ARG;
    int v[3];
    gf::recon_tuning(r, v);
    for (int i = 0; i < 3; ++i) variants[i] = v[i];
    return GENFIRE_OK;
}

genfire_status genfire_recon_set_rfree(genfire_recon *r, int32_t nshells, const int64_t *counts,
                                      const int64_t *indices)
{
    if (!r) return GENFIRE_ERR_ARG;
    genfire_ctx *ctx = r->ctx;
    return guarded(ctx, [&] { gf::recon_set_rfree(r, nshells, counts, indices); });
}

genfire_status genfire_recon_rfree(genfire_recon *r, int32_t *nshells, double *rfree)
{
    if (!r) return GENFIRE_ERR_ARG;
    genfire_ctx *ctx = r->ctx;
    return guarded(ctx, [&] {
        const int n = gf::recon_rfree(r, rfree);
        if (nshells) *nshells = n;
    });
}

genfire_status genfire_rfree_candidates(genfire_ctx *ctx, const genfire_params *p, const void *measuredK,
                                        int32_t on_device, int32_t nbins, int64_t *counts, int64_t *indices)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(p, "params");
        gf::check_params(*p, false);
        gf::rfree_candidates(ctx, *p, measuredK, on_device != 0, nbins, counts, indices);
    });
}

genfire_status genfire_recon_profile(genfire_recon *r, int32_t iterations, double *ms, double *bytes)
{
    if (!r) return GENFIRE_ERR_ARG;
    genfire_ctx *ctx = r->ctx;
    return guarded(ctx, [&] { gf::recon_profile(r, iterations, ms, bytes); });
}

const char *genfire_profile_kernel_name(int32_t k)
{
    static const char *names[GENFIRE_PROFILE_KERNELS] = {
        "F1 row pass (dim-1 real->half, positivity, support; starts the iteration)",
        "F2 column pass (dim-2 forward)",
        "F3 column pass (dim-3 forward, Fourier constraint, errK, dim-3 inverse)",
        "I2 column pass (dim-2 inverse; errK total and best object)", "I1 row pass (half->real dim-1)"};
    return (k >= 0 && k < GENFIRE_PROFILE_KERNELS) ? names[k] : "";
}

genfire_status genfire_reconstruct(genfire_ctx *ctx, const genfire_params *p, const void *measuredK,
                                   const uint8_t *measuredK_mask, const uint8_t *support, const void *initialObject,
                                   const double *projections, const double *angles, void *reconstruction,
                                   double *errK, double *errR, double *Rarr, double *Rarr2)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    genfire_recon *r = nullptr;
    genfire_status st = genfire_recon_create(ctx, p, measuredK, measuredK_mask, support, initialObject, projections,
                                             angles, 0, &r);
    if (st != GENFIRE_OK) return st;
    st = genfire_recon_iterate(r, p->numIterations);
    if (st == GENFIRE_OK) st = genfire_recon_result(r, reconstruction, errK, errR, Rarr, Rarr2, 0);
    std::string keep = ctx->last_error;
    genfire_recon_destroy(r);
    if (st != GENFIRE_OK) ctx->last_error = keep;
    return st;
}

// ---------------------------------------------------------------- projector
static void host_rotations(int P, const double *angles, const double *vectors, std::vector<double> &Rs)
{
    Rs.resize(9 * (size_t)P);
    for (int i = 0; i < P; ++i) {
        double *R = &Rs[9 * (size_t)i];
        if (vectors) gf::euler_rot(vectors, vectors + 3, vectors + 6, angles[i], angles[i + P], angles[i + 2 * P], R);
        else gf::rot_zyz(angles[i], angles[i + P], angles[i + 2 * P], R);
    }
}

genfire_status genfire_project(genfire_ctx *ctx, int32_t precision, const void *vol, int32_t n1, int32_t n2,
                               int32_t n3, int32_t num_proj, const double *angles, const double *vectors, void *projs)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(vol, "vol");
        need(angles, "angles");
        need(projs, "projs");
        if (precision != GENFIRE_PREC_FP64 && precision != GENFIRE_PREC_MIXED) gf::fail(GENFIRE_ERR_ARG, "bad precision.");
        if (num_proj < 1) gf::fail(GENFIRE_ERR_ARG, "num_proj must be positive.");
        cudaStream_t st = ctx->stream;
        const size_t es = real_size(precision);
        std::vector<double> Rs;
        host_rotations(num_proj, angles, vectors, Rs);
        const size_t nv = (size_t)n1 * n2 * n3, np = (size_t)n1 * n2 * num_proj;
        DevBuf dv(es * nv, st), dp(es * np, st), dR(sizeof(double) * Rs.size(), st);
        GF_CUDA(cudaMemcpyAsync(dv.p, vol, es * nv, cudaMemcpyHostToDevice, st));
        GF_CUDA(cudaMemcpyAsync(dR.p, Rs.data(), sizeof(double) * Rs.size(), cudaMemcpyHostToDevice, st));
        gf::project_batch(ctx, precision, dv.p, n1, n2, n3, n1, (long long)n1 * n2, num_proj, dR.as<double>(), dp.p,
                          nullptr, nullptr, st);
        GF_CUDA(cudaMemcpyAsync(projs, dp.p, es * np, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
    });
}

genfire_status genfire_rfactor(genfire_ctx *ctx, int32_t precision, const void *vol, int32_t n1, int32_t n2,
                               int32_t n3, int32_t num_proj, const double *angles, const double *vectors,
                               const double *measured, double *Rarr, double *Rarr2, double *errR)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(vol, "vol");
        need(angles, "angles");
        need(measured, "measured");
        if (precision != GENFIRE_PREC_FP64 && precision != GENFIRE_PREC_MIXED) gf::fail(GENFIRE_ERR_ARG, "bad precision.");
        if (num_proj < 1) gf::fail(GENFIRE_ERR_ARG, "num_proj must be positive.");
        cudaStream_t st = ctx->stream;
        const size_t es = real_size(precision);
        std::vector<double> Rs;
        host_rotations(num_proj, angles, vectors, Rs);
        const size_t nv = (size_t)n1 * n2 * n3, np = (size_t)n1 * n2 * num_proj;
        DevBuf dv(es * nv, st), dm(sizeof(double) * np, st), dR(sizeof(double) * Rs.size(), st),
            ds(sizeof(double) * 4 * num_proj, st);
        GF_CUDA(cudaMemcpyAsync(dv.p, vol, es * nv, cudaMemcpyHostToDevice, st));
        GF_CUDA(cudaMemcpyAsync(dm.p, measured, sizeof(double) * np, cudaMemcpyHostToDevice, st));
        GF_CUDA(cudaMemcpyAsync(dR.p, Rs.data(), sizeof(double) * Rs.size(), cudaMemcpyHostToDevice, st));
        gf::project_batch(ctx, precision, dv.p, n1, n2, n3, n1, (long long)n1 * n2, num_proj, dR.as<double>(), nullptr,
                          dm.as<double>(), ds.as<double>(), st);
        std::vector<double> sums(4 * (size_t)num_proj);
        GF_CUDA(cudaMemcpyAsync(sums.data(), ds.p, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
        double tot = 0;
        for (int i = 0; i < num_proj; ++i) {
            const double r1 = sums[4 * i] / sums[4 * i + 1];
            const double r2 = std::sqrt(sums[4 * i + 2]) / std::sqrt(sums[4 * i + 3]);
            if (Rarr) Rarr[i] = r1;
            if (Rarr2) Rarr2[i] = r2;
            tot += r1;
        }
        if (errR) *errR = tot / num_proj;
    });
}

genfire_status genfire_set_projector_interpolation(genfire_ctx *ctx, int32_t interp)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    if (interp != GENFIRE_INTERP_TRILINEAR && interp != GENFIRE_INTERP_CUBIC) {
        ctx->last_error = "GENFIRE: interpolation must be GENFIRE_INTERP_TRILINEAR or GENFIRE_INTERP_CUBIC.";
        return GENFIRE_ERR_ARG;
    }
    ctx->interp = interp;
    return GENFIRE_OK;
}

genfire_status genfire_rfactor_realspace(genfire_ctx *ctx, int32_t precision, const void *model, int32_t m1,
                                         int32_t m2, int32_t m3, const double *projs, int32_t p1, int32_t p2,
                                         int32_t num_proj, const double *angles, double *Rarr, double *Rtotal,
                                         float *simuProjs)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(model, "model");
        need(projs, "projs");
        need(angles, "angles");
        if (precision != GENFIRE_PREC_FP64 && precision != GENFIRE_PREC_MIXED) gf::fail(GENFIRE_ERR_ARG, "bad precision.");
        if (num_proj < 1) gf::fail(GENFIRE_ERR_ARG, "num_proj must be positive.");
        if (p1 < 1 || p2 < 1) gf::fail(GENFIRE_ERR_ARG, "projection sizes must be positive.");
        cudaStream_t st = ctx->stream;
        const size_t es = real_size(precision);
        const size_t nv = (size_t)m1 * m2 * m3, np = (size_t)p1 * p2 * num_proj;
        DevBuf dv(es * nv, st), dp(sizeof(double) * np, st), ds;
        if (simuProjs) ds.alloc(sizeof(float) * np, st);
        GF_CUDA(cudaMemcpyAsync(dv.p, model, es * nv, cudaMemcpyHostToDevice, st));
        GF_CUDA(cudaMemcpyAsync(dp.p, projs, sizeof(double) * np, cudaMemcpyHostToDevice, st));
        gf::rfactor_realspace(ctx, precision, dv.p, m1, m2, m3, num_proj, angles, dp.as<double>(), p1, p2, Rarr,
                              Rtotal, simuProjs ? ds.as<float>() : nullptr);
        if (simuProjs) {
            GF_CUDA(cudaMemcpyAsync(simuProjs, ds.p, sizeof(float) * np, cudaMemcpyDeviceToHost, st));
            GF_CUDA(cudaStreamSynchronize(st));
        }
    });
}

// Allocation-free: no std::function wrapper, no heap buffers; errors are
// caught here directly.
genfire_status genfire_rfactor_noalloc(genfire_ctx *ctx, int32_t precision, const void *d_vol, int32_t n1,
                                       int32_t n2, int32_t n3, int32_t num_proj, const double *angles,
                                       const double *vectors, const double *d_measured, double *Rarr,
                                       double *Rarr2, double *errR)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    try {
        GF_CUDA(cudaSetDevice(ctx->device));
        ctx->last_error.clear();
        need(d_vol, "vol");
        need(angles, "angles");
        need(d_measured, "measured");
        if (precision != GENFIRE_PREC_FP64 && precision != GENFIRE_PREC_MIXED) gf::fail(GENFIRE_ERR_ARG, "bad precision.");
        if (num_proj < 1) gf::fail(GENFIRE_ERR_ARG, "num_proj must be positive.");
        if (n1 < 2 || n2 < 2 || n3 < 2) gf::fail(GENFIRE_ERR_ARG, "projector: every volume dimension must be at least 2.");
        gf::rfactor_noalloc(ctx, precision, d_vol, n1, n2, n3, num_proj, angles, vectors, d_measured, Rarr, Rarr2, errR);
        return GENFIRE_OK;
    } catch (const Error &e) {
        ctx->last_error = e.msg;
        return e.st;
    } catch (...) {
        ctx->last_error = "GENFIRE: unexpected internal error";
        return GENFIRE_ERR_STATE;
    }
}

// ---------------------------------------------------------------- index and symmetry kernels
genfire_status genfire_centro_symmetricity(genfire_ctx *ctx, const double *FS, int32_t n1, int32_t n_k1, int32_t n2,
                                           double *measuredK)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(FS, "FS");
        need(measuredK, "measuredK");
        if (n1 < 1 || n2 < 1 || n_k1 != n1 / 2) gf::fail(GENFIRE_ERR_ARG, "CentroSymmetricity: n_k1 must be floor(n1/2).");
        cudaStream_t st = ctx->stream;
        const size_t nfs = (size_t)(n_k1 + 1) * (2 * (n2 / 2) + 1) * (2 * (n1 / 2) + 1);
        const size_t nm = (size_t)n1 * n2 * n1;
        DevBuf a(sizeof(double2) * nfs, st), b(sizeof(double2) * nm, st);
        GF_CUDA(cudaMemcpyAsync(a.p, FS, sizeof(double2) * nfs, cudaMemcpyHostToDevice, st));
        gf::centro_device(ctx, a.as<double2>(), n1, n_k1, n2, b.as<double2>());
        GF_CUDA(cudaMemcpyAsync(measuredK, b.p, sizeof(double2) * nm, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
    });
}

genfire_status genfire_hermitian_symmetrize(genfire_ctx *ctx, const double *in, int32_t d1, int32_t d2, int32_t d3,
                                            double *out)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(in, "in");
        need(out, "out");
        if (d1 < 1 || d2 < 1 || d3 < 1) gf::fail(GENFIRE_ERR_ARG, "hermitianSymmetrize: bad size.");
        cudaStream_t st = ctx->stream;
        const size_t n = (size_t)d1 * d2 * d3;
        DevBuf a(sizeof(double2) * n, st), b(sizeof(double2) * n, st);
        GF_CUDA(cudaMemcpyAsync(a.p, in, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
        gf::hermitian_device(ctx, a.as<double2>(), d1, d2, d3, b.as<double2>());
        GF_CUDA(cudaMemcpyAsync(out, b.p, sizeof(double2) * n, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
    });
}

genfire_status genfire_make_kspace_indices(genfire_ctx *ctx, int32_t d1, int32_t d2, int32_t d3, double *Q)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(Q, "Q");
        if (d1 < 1 || d2 < 1 || d3 < 1) gf::fail(GENFIRE_ERR_ARG, "make_Kspace_indices: bad size.");
        cudaStream_t st = ctx->stream;
        const size_t n = (size_t)d1 * d2 * d3;
        DevBuf a(sizeof(double) * n, st);
        gf::kspace_device(ctx, d1, d2, d3, a.as<double>());
        GF_CUDA(cudaMemcpyAsync(Q, a.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
    });
}

genfire_status genfire_volumn_index(const int32_t big[3], const int32_t ori[3], int32_t out[6])
{
    if (!big || !ori || !out) return GENFIRE_ERR_ARG;
    for (int i = 0; i < 3; ++i) {
        if (ori[i] > big[i] || ori[i] < 0) {
            g_noctx_error = "GENFIRE: paddedsize should be equal to or smaller than original volume in all dimensions!";
            return GENFIRE_ERR_ARG;
        }
        // the four parity cases of My_volumn_index.m:12-28 all equal floor(big/2) - floor(ori/2)
        const int s = big[i] / 2 - ori[i] / 2;
        out[i] = s + 1;
        out[i + 3] = s + ori[i];
    }
    return GENFIRE_OK;
}

genfire_status genfire_iffshift3_ind(genfire_ctx *ctx, const int32_t size[3], int64_t count, const int64_t *inds,
                                     int64_t *out)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(size, "size");
        if (count < 0) gf::fail(GENFIRE_ERR_ARG, "count must be non-negative.");
        if (count == 0) return;
        need(inds, "inds");
        need(out, "out");
        cudaStream_t st = ctx->stream;
        DevBuf a(sizeof(long long) * count, st), b(sizeof(long long) * count, st);
        GF_CUDA(cudaMemcpyAsync(a.p, inds, sizeof(long long) * count, cudaMemcpyHostToDevice, st));
        const int sz[3] = {size[0], size[1], size[2]};
        gf::iffshift_device(ctx, sz, count, a.as<long long>(), b.as<long long>());
        GF_CUDA(cudaMemcpyAsync(out, b.p, sizeof(long long) * count, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
    });
}

genfire_status genfire_select(genfire_ctx *ctx, const genfire_params *p, double phi, double theta, double psi,
                              int64_t cap, int64_t *ind, float *dist, float *u, float *v, int64_t *count)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(p, "params");
        need(count, "count");
        gf::check_params(*p, false);
        if (cap > 0) { need(ind, "ind"); need(dist, "dist"); need(u, "u"); need(v, "v"); }
        *count = gf::select_one(ctx, *p, phi, theta, psi, cap, ind, dist, u, v);
    });
}

genfire_status genfire_fftn(genfire_ctx *ctx, int32_t precision, void *data, int32_t n1, int32_t n2, int32_t n3,
                            int32_t inverse)
{
    if (!ctx) return GENFIRE_ERR_ARG;
    return guarded(ctx, [&] {
        need(data, "data");
        if (n1 < 1 || n2 < 1 || n3 < 1) gf::fail(GENFIRE_ERR_ARG, "fftn: bad size.");
        if (precision != GENFIRE_PREC_FP64 && precision != GENFIRE_PREC_MIXED) gf::fail(GENFIRE_ERR_ARG, "bad precision.");
        cudaStream_t st = ctx->stream;
        const size_t nb = (size_t)n1 * n2 * n3 * 2 * real_size(precision);
        DevBuf a(nb, st);
        GF_CUDA(cudaMemcpyAsync(a.p, data, nb, cudaMemcpyHostToDevice, st));
        gf::fftn_device(ctx, precision, a.p, n1, n2, n3, inverse != 0);
        GF_CUDA(cudaMemcpyAsync(data, a.p, nb, cudaMemcpyDeviceToHost, st));
        GF_CUDA(cudaStreamSynchronize(st));
    });
}

}  // extern "C"
