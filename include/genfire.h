/*
 * genfire.h -- C ABI of libgenfire.so, the GB300 (sm_103a) implementation of
 * the GENFIRE v2 reconstruction hot path.
 *
 * Each entry point replaces one method or function of the MATLAB reference
 * (paths are relative to the GENFIRE source tree).  Arrays use MATLAB's
 * memory layout: column-major (dimension 1 fastest), complex data
 * interleaved (re, im), which is what a MEX gateway receives from
 * mxGetComplexDoubles / mxGetComplexSingles.
 *
 * Conventions
 *   - Every function returns a genfire_status; GENFIRE_OK is 0.  On failure
 *     genfire_last_error(ctx) holds a message of the form "GENFIRE: ...".
 *   - Calls are synchronous: outputs are complete when the call returns.
 *   - A context owns one CUDA stream on one device.  A context is not
 *     thread-safe; use one context per host thread.
 *   - Host-pointer entry points copy inputs to the device and results back.
 *     The *_device variants take device pointers (e.g. from cudaMalloc or a
 *     torch tensor) and leave results on the device.
 *   - precision GENFIRE_PREC_FP64 is the drop-in: gridding DFT, averaging,
 *     FFTs and the iteration in FP64, measuredK complex128.
 *     GENFIRE_PREC_MIXED computes the gridding DFT in reduced precision with
 *     FP32 accumulation and FP64 phase reduction and weight sums, keeps
 *     measuredK as complex64 (as runGridding does, GENFIRE_Reconstructor.m:182)
 *     and runs the iteration on complex64 with FP64 error accumulation.
 */
#ifndef GENFIRE_H
#define GENFIRE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GENFIRE_ABI_VERSION 1

typedef enum genfire_status {
    GENFIRE_OK = 0,
    GENFIRE_ERR_ARG = 1,          /* invalid argument (sizes, NULL, modes) */
    GENFIRE_ERR_OOM = 2,          /* device memory exhausted */
    GENFIRE_ERR_CUDA = 3,         /* CUDA runtime error */
    GENFIRE_ERR_TIMEOUT = 4,      /* a bounded device-side wait gave up */
    GENFIRE_ERR_UNSUPPORTED = 5,  /* e.g. an FFT length with a prime factor > 7 */
    GENFIRE_ERR_STATE = 6         /* handle used out of order */
} genfire_status;

/* Arithmetic of a call.  FP64 is the drop-in (complex128 throughout).  MIXED
 * and FP16_SCALED iterate in complex64 with FP64 error, weight and phase sums;
 * they differ only in the gridding DFT's tensor-core operands: split BF16
 * (hi*hi + hi*lo + lo*hi, ~16 bits per operand) for MIXED, split FP16 (~22
 * bits per operand, each projection scaled by a power of two so its largest
 * value sits below 2^14) for FP16_SCALED.  Wherever a call takes a real
 * volume or grid, FP16_SCALED means float, as MIXED does. */
typedef enum genfire_precision {
    GENFIRE_PREC_FP64 = 0,
    GENFIRE_PREC_MIXED = 1,
    GENFIRE_PREC_FP16_SCALED = 2
} genfire_precision;

/* The GENFIRE_Reconstructor properties read by the hot path
 * (GENFIRE_Reconstructor.m:30-70; names kept).  Dim1, Dim2 and NumProjs are
 * what CheckPrepareData derives from the projection stack
 * (GENFIRE_Reconstructor.m:118-121). */
typedef struct genfire_params {
    int32_t Dim1;
    int32_t Dim2;
    int32_t NumProjs;
    int32_t DFT_CentroSymmetricity;       /* 1: grid the k1<=0 half and mirror */
    double  oversamplingRatio;            /* n = round(Dim * ratio) */
    double  interpolationCutoffDistance;  /* plane-distance cutoff, grid units */
    double  vector1[3];                   /* rotation axes for phi, theta, psi */
    double  vector2[3];
    double  vector3[3];
    int32_t numIterations;
    int32_t constraintEnforcementMode;    /* 1, 2 or 3 */
    int32_t constraintPositivity;
    int32_t constraintSupport;
    int32_t monitor_R;                    /* R-factor every monitorR_loopLength */
    int32_t monitorR_loopLength;
    int32_t precision;                    /* genfire_precision */
    int32_t griddingMethod;               /* 1: FFT gridding grid sizes (an m x m x m cube,
                                             fillInFourierGrid.m:38-42) for genfire_grid_size
                                             and the iteration; else DFT sizes n1 x n2 x n1.
                                             genfire_params_init sets 2 (zero also means DFT) */
    int32_t allowMultipleGridMatches;     /* FFT gridding: also grid to the voxels within
                                             round(cutoff) of the nearest one (class default 1) */
    int32_t reserved[7];                  /* zero */
} genfire_params;

typedef struct genfire_ctx genfire_ctx;
typedef struct genfire_recon genfire_recon;
typedef struct genfire_recon_batch genfire_recon_batch;

/* ---- library ----------------------------------------------------------- */

int32_t genfire_abi_version(void);
const char *genfire_status_string(genfire_status s);

/* Class defaults (GENFIRE_Reconstructor.m:30-70) with precision = FP64. */
genfire_status genfire_params_init(genfire_params *p);

/* Size of measuredK: n1 x n2 x n1 with n1 = round(Dim1*ratio), n2 =
 * round(Dim2*ratio) (CheckPrepareData, GENFIRE_Reconstructor.m:168-169), or,
 * with griddingMethod = 1, the FFT-gridding cube n1 = n2 = m
 * (fillInFourierGrid.m:38-42). */
genfire_status genfire_grid_size(const genfire_params *p, int32_t *n1, int32_t *n2);

/* ---- context ----------------------------------------------------------- */

genfire_status genfire_create(int32_t device, genfire_ctx **out);
/* Frees the context and, first, every reconstruction and batch still alive on
 * it (their handles become invalid). */
genfire_status genfire_destroy(genfire_ctx *ctx);
const char *genfire_last_error(const genfire_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work against the *_device entry points. */
void *genfire_stream(genfire_ctx *ctx);

/* ---- gridding: fillInFourierGrid_DFT ------------------------------------
 * Replaces obj = fillInFourierGrid_DFT(obj)
 * (@GENFIRE_Reconstructor/fillInFourierGrid_DFT.m:85-310) as called by
 * runGridding (GENFIRE_Reconstructor.m:172-186).
 *   projections  Dim1 x Dim2 x NumProjs, double
 *   angles       NumProjs x 3 (phi, theta, psi in degrees), double
 *   measuredK    n1 x n2 x n1 complex, centred (k=0 at floor(n/2)+1):
 *                complex128 for FP64, complex64 for MIXED
 *   recIFFT      Dim1 x Dim2 x Dim1 = My_stripzero(real(my_ifft(measuredK)))
 *                (fillInFourierGrid_DFT.m:304); double for FP64, float for
 *                MIXED; NULL to skip
 *   nk           NumProjs counts of gridded K-points per projection; NULL ok
 * Index sets are bit-exact with the FP32 selection of the reference
 * (:175-192) evaluated with a fixed operation order.  Host buffers of 64 MB
 * and more (measuredK, recIFFT here; measuredK, measuredK_mask and
 * initialObject in genfire_reconstruct and a host genfire_recon_create; the
 * reconstruction of genfire_reconstruct and a host genfire_recon_result) are
 * page-locked with cudaHostRegister for the duration of their copy and
 * released before the call returns; when registration fails the copy runs
 * from pageable memory. */
genfire_status genfire_grid_dft(genfire_ctx *ctx, const genfire_params *p,
                                const double *projections, const double *angles,
                                void *measuredK, void *recIFFT, int64_t *nk);
genfire_status genfire_grid_dft_device(genfire_ctx *ctx, const genfire_params *p,
                                       const double *d_projections, const double *angles,
                                       void *d_measuredK, void *d_recIFFT, int64_t *nk);

/* genfire_grid_dft_device (without recIFFT) with the device time of its
 * stages from CUDA events on the context stream (tracing; the reference
 * prints only the total, fillInFourierGrid_DFT.m:306-308): stage_ms[0]
 * K-point selection, [1] DFT stage (operand preparation and the DFT kernel),
 * [2] the DFT kernel alone, [3] sort, weighted sums, average, centro mirror
 * and cast (written into measuredK), [4] measuredK's zero pattern, [5]
 * recIFFT (0 here). */
genfire_status genfire_grid_profile(genfire_ctx *ctx, const genfire_params *p, const double *d_projections,
                                    const double *angles, void *d_measuredK, double *stage_ms);

/* ---- gridding: fillInFourierGrid (griddingMethod = 1) -------------------
 * Replaces obj = fillInFourierGrid(obj)
 * (@GENFIRE_Reconstructor/fillInFourierGrid.m:27-168), the class's default
 * gridding method in runGridding (GENFIRE_Reconstructor.m:175-177).
 *   projections  Dim1 x Dim2 x NumProjs, double
 *   angles       NumProjs x 3 (phi, theta, psi in degrees; the
 *                GENFIRE/RELION convention of fillInFourierGrid.m:80-82 --
 *                vector1..3 are not used), double
 *   measuredK    m x m x m complex, centred; m = Dim2 * oversamplingRatio for
 *                even Dim2, 1 + (Dim2-1) * oversamplingRatio for odd Dim2 (must
 *                be an integer, and at least Dim1 and Dim2); complex128 for
 *                FP64, complex64 for MIXED.  The values after the weighted
 *                average (w = 1/(d + 1e-5) over the voxels within
 *                interpolationCutoffDistance of each rotated FFT sample) and
 *                hermitianSymmetrize.
 *   recIFFT      Dim1 x Dim2 x Dim1 = My_stripzero(real(my_ifft(measuredK)))
 *                (:165); double / float; NULL to skip
 *   npairs       number of (voxel, value) pairs gridded; NULL ok
 * allowMultipleGridMatches selects the shift search of :108-139.  The sums
 * are FP64 atomic adds (order-independent up to FP64 rounding). */
genfire_status genfire_grid_fft(genfire_ctx *ctx, const genfire_params *p,
                                const double *projections, const double *angles,
                                void *measuredK, void *recIFFT, int64_t *npairs);
genfire_status genfire_grid_fft_device(genfire_ctx *ctx, const genfire_params *p,
                                       const double *d_projections, const double *angles,
                                       void *d_measuredK, void *d_recIFFT, int64_t *npairs);

/* ---- iteration: reconstruct ---------------------------------------------
 * Replaces obj = reconstruct(obj) (@GENFIRE_Reconstructor/reconstruct.m:28-194).
 *   measuredK       n1 x n2 x n1 complex, centred (type as for grid_dft)
 *   measuredK_mask  n1 x n2 x n1 bytes; NULL means measuredK ~= 0 (the value
 *                   runGridding sets, GENFIRE_Reconstructor.m:183)
 *   support         Dim1 x Dim2 x Dim1 bytes; NULL means all ones
 *   initialObject   Dim1 x Dim2 x Dim1 (double for FP64, float for MIXED);
 *                   NULL means zeros
 *   projections, angles   needed only when monitor_R == 1
 *   reconstruction  Dim1 x Dim2 x Dim1 (double for FP64, float for MIXED)
 *   errK            numIterations doubles
 *   errR            floor(numIterations/monitorR_loopLength) doubles (or NULL)
 *   Rarr, Rarr2     NumProjs x that count (or NULL) */
genfire_status genfire_reconstruct(genfire_ctx *ctx, const genfire_params *p,
                                   const void *measuredK, const uint8_t *measuredK_mask,
                                   const uint8_t *support, const void *initialObject,
                                   const double *projections, const double *angles,
                                   void *reconstruction, double *errK,
                                   double *errR, double *Rarr, double *Rarr2);

/* Staged form of genfire_reconstruct for callers that drive the iterations
 * themselves (timing, checkpoints).  on_device selects whether the array
 * pointers are device (1) or host (0) pointers.  iterate() continues the
 * iteration count where the last call stopped; the total may not exceed
 * numIterations.  The loop body of one iteration is replayed as a CUDA
 * graph. */
genfire_status genfire_recon_create(genfire_ctx *ctx, const genfire_params *p,
                                    const void *measuredK, const uint8_t *measuredK_mask,
                                    const uint8_t *support, const void *initialObject,
                                    const double *projections, const double *angles,
                                    int32_t on_device, genfire_recon **out);
genfire_status genfire_recon_iterate(genfire_recon *r, int32_t count);
/* Copies out the best object (after positivity and support, cropped), errK
 * of the iterations run so far, and the R-factor records. */
genfire_status genfire_recon_result(genfire_recon *r, void *reconstruction, double *errK,
                                    double *errR, double *Rarr, double *Rarr2,
                                    int32_t on_device);
/* GENFIRE_ERR_STATE (nothing freed) while r is a member of a live batch:
 * destroy the batch first. */
genfire_status genfire_recon_destroy(genfire_recon *r);

/* Batches of independent reconstructions (problems of different sizes,
 * precisions and projection counts) iterated together: one CUDA graph holds
 * one iteration of every member as independent child graphs, so each launch
 * runs all members' iterations concurrently on the device.  No counterpart in
 * the reference, which reconstructs one object per call.  Every member must
 * have been created on ctx; the batch does not own them: destroy the batch
 * before any member, and do not iterate a member on its own while it is in a
 * live batch.  genfire_recon_batch_iterate advances every member by count
 * iterations (each member's total may not exceed its numIterations); results
 * are read per member with genfire_recon_result. */
genfire_status genfire_recon_batch_create(genfire_ctx *ctx, int32_t count, genfire_recon *const *members,
                                          genfire_recon_batch **out);
genfire_status genfire_recon_batch_iterate(genfire_recon_batch *b, int32_t count);
genfire_status genfire_recon_batch_destroy(genfire_recon_batch *b);

/* Per-kernel timing of the iteration (tracing; the reference only prints
 * wall times, reconstruct.m:74,188-190).  Runs `iterations` further
 * iterations (they count toward numIterations) with each kernel of the
 * iteration launched on its own and bracketed by CUDA events on the context
 * stream.  For kernel k < GENFIRE_PROFILE_KERNELS, ms[k] receives its mean
 * duration and bytes[k] its algorithmic HBM traffic per launch (compulsory
 * reads plus writes); genfire_profile_kernel_name(k) names it. */
/* The FFT-pass variants the autotuner chose for this reconstruction (it times
 * each candidate on the problem's own buffers at creation; the environment
 * variable GENFIRE_AUTOTUNE=0 keeps the built-in choice): variants[0..2] for
 * the dim-2 forward, the fused dim-3 and the dim-2 inverse pass; 0 = generic
 * shared-memory engine, 1 = register-resident radix 8, one column per thread,
 * 2 = the same with two columns per thread, 3 = mixed radix (3 or 5 times a
 * power of two), 4 = radix 32 x 16 or 32 x 32 for 512 or 1024 complex64
 * points (one shared-memory exchange per transform), -1 = built-in choice.
 * GENFIRE_COL_VARIANT=<v>
 * forces variant v wherever it is valid. */
genfire_status genfire_recon_tuning(genfire_recon *r, int32_t *variants);

/* ---- Rfree monitor -------------------------------------------------------
 * reconstruct.m:46-69 (selection) and :137-146 (per iteration).
 * genfire_rfree_candidates: the candidate points of each of nbins shells,
 *   find(measuredK ~= 0 & Q >= edge(s) - 0.05 & Q < edge(s+1)) with
 *   edge = linspace(0, 1, nbins + 1) and Q = make_Kspace_indices of the
 *   measuredK grid (n1 x n2 x n1 from params, as genfire_reconstruct);
 *   counts[s] receives the number of shell s; indices (NULL: counts only)
 *   receives the ascending 0-based linear indices of all shells, concatenated.
 *   measuredK is complex128 (FP64) or complex64 (MIXED), host or device.
 * The random choice of the withheld points (randperm, :53-60) stays with the
 * caller: MATLAB's generator is not reproduced here.
 * genfire_recon_set_rfree: registers the withheld points (0-based centred
 *   linear indices, counts[s] for shell s, concatenated) of a reconstruction
 *   created with them already cleared in measuredK_mask (:65); call before the
 *   first genfire_recon_iterate (and before adding it to a batch).  Each
 *   iteration then records Rfree(s, it) = sum |k - measuredK| / sum |measuredK|
 *   over shell s, k = fftn of the object before the Fourier constraint.
 * genfire_recon_rfree: *nshells, and (rfree not NULL) the values of the
 *   iterations run so far, column-major nshells x iterations (Rfree_complex). */
genfire_status genfire_rfree_candidates(genfire_ctx *ctx, const genfire_params *p, const void *measuredK,
                                        int32_t on_device, int32_t nbins, int64_t *counts, int64_t *indices);
genfire_status genfire_recon_set_rfree(genfire_recon *r, int32_t nshells, const int64_t *counts,
                                      const int64_t *indices);
genfire_status genfire_recon_rfree(genfire_recon *r, int32_t *nshells, double *rfree);

#define GENFIRE_PROFILE_KERNELS 5
genfire_status genfire_recon_profile(genfire_recon *r, int32_t iterations, double *ms, double *bytes);
const char *genfire_profile_kernel_name(int32_t k);

/* ---- projector -----------------------------------------------------------
 * Replaces Proj = calculate3Dprojection_RealSpaceinterp(Vol,phi,theta,psi)
 * (src/calculate3Dprojection_RealSpaceinterp.m:1-57; vectors == NULL: the
 * closed-form ZYZ matrix of :13-15) and
 * calculate3Dprojection_RealSpaceinterp_general(Vol,phi,theta,psi,v1,v2,v3)
 * (src/calculate3Dprojection_RealSpaceinterp_general.m:1-49; vectors = the 9
 * values v1, v2, v3).  Interpolation is trilinear (or cubic, see
 * genfire_set_projector_interpolation), samples outside the volume are 0.  Vol is n1 x n2 x n3; each projection is n1 x n2.  NumProj angle
 * rows (NumProj x 3, column-major like InputAngles).  vol/projs are double
 * for FP64 and float for MIXED. */
genfire_status genfire_project(genfire_ctx *ctx, int32_t precision,
                               const void *vol, int32_t n1, int32_t n2, int32_t n3,
                               int32_t num_proj, const double *angles, const double *vectors,
                               void *projs);
/* Interpolation of the projector (genfire_project, genfire_rfactor,
 * genfire_rfactor_noalloc, genfire_rfactor_realspace and the R-factor monitor
 * of the iteration) for this context.  TRILINEAR (the default) is the
 * projector the benchmark and its R-factors are defined with; CUBIC is the
 * reference's interp3(..., 'cubic', 0) (calculate3Dprojection_RealSpaceinterp.m:45):
 * separable cubic convolution with Keys' kernel (a = -1/2) and Keys' boundary
 * rule, 0 outside the volume; it needs at least 4 samples per dimension.
 * MATLAB's interp3 is closed source, so cubic parity with MATLAB is unpinned. */
#define GENFIRE_INTERP_TRILINEAR 0
#define GENFIRE_INTERP_CUBIC 1
genfire_status genfire_set_projector_interpolation(genfire_ctx *ctx, int32_t interp);

/* Replaces [Rtotal, Rarr, simuProjs] = Tian_calc_Rfactor_realspace(model, Projs,
 * Angles) (src/Tian_calc_Rfactor_realspace.m:1-24).  Its projector,
 * calculate3Dprojection_RealSpaceinterpZYX, is not in the reference tree; it is
 * taken as the general projector with the axes Z, Y, X ([0 0 1], [0 1 0],
 * [1 0 0]) for phi, theta, psi.  Each m1 x m2 projection of the m1 x m2 x m3
 * model is cropped to p1 x p2 (My_stripzero) and compared with the measured
 * projection: Rarr(i) = sum| |bp| - |pj| | / sum|pj|, Rtotal = mean(Rarr).
 *   model      m1 x m2 x m3, double (FP64) / float (MIXED)
 *   projs      p1 x p2 x num_proj double (p1 <= m1, p2 <= m2)
 *   angles     num_proj x 3 double
 *   simuProjs  p1 x p2 x num_proj float (single, as the reference returns
 *              it); NULL to skip */
genfire_status genfire_rfactor_realspace(genfire_ctx *ctx, int32_t precision, const void *model, int32_t m1,
                                         int32_t m2, int32_t m3, const double *projs, int32_t p1, int32_t p2,
                                         int32_t num_proj, const double *angles, double *Rarr, double *Rtotal,
                                         float *simuProjs);

/* R-factors of reconstruct.m:168-185: per projection
 * Rarr = sum|bp - pj| / sum|pj| and Rarr2 = ||bp - pj||_F / ||pj||_F of the
 * projection bp of vol against the measured pj; errR = mean(Rarr).
 * measured is n1 x n2 x num_proj double. */
genfire_status genfire_rfactor(genfire_ctx *ctx, int32_t precision,
                               const void *vol, int32_t n1, int32_t n2, int32_t n3,
                               int32_t num_proj, const double *angles, const double *vectors,
                               const double *measured, double *Rarr, double *Rarr2,
                               double *errR);

/* The R-factors of genfire_rfactor computed without allocating device memory.
 * No counterpart in the reference.  It is for callers whose device memory is
 * owned by someone else and who may not call cudaMalloc: for example a MEX
 * function working on gpuArray data under MATLAB's memory manager, or a
 * service that has reserved the device's memory for its own pool.  vol
 * (n1 x n2 x n3, double for FP64, float for MIXED) and measured (n1 x n2 x
 * num_proj double) are device pointers; angles and vectors are host arrays as
 * for genfire_rfactor; Rarr, Rarr2 and errR are host outputs.  The scratch
 * (rotation matrices and partial sums) is a 4 MiB static device array in the
 * library, so the call allocates nothing; inputs needing more than 4 MiB of
 * scratch (about 9 * num_proj + 4 * num_proj * (ceil(n1*n2/256) + 1) doubles)
 * are rejected with GENFIRE_ERR_ARG.  Every call looks up the array's device
 * address in the current context (cudaGetSymbolAddress, which allocates
 * nothing), so a device reset between calls (reset(gpuDevice) in MATLAB) leaves
 * no stale address behind; the context itself must be recreated after a reset,
 * as for every other call.  vol and measured are read on the context's stream
 * (genfire_stream), with no ordering against the stream that wrote them: the
 * caller finishes writing them first (synchronize, or produce them on that
 * stream).  The call copies the rotation matrices in and the sums out and
 * waits for them, so it must not be called while any stream of the device is
 * being captured into a CUDA graph.  Every call uses the same array: calls
 * whose GPU work overlaps (from two host threads, or on two streams) race on
 * it. */
genfire_status genfire_rfactor_noalloc(genfire_ctx *ctx, int32_t precision, const void *d_vol, int32_t n1,
                                       int32_t n2, int32_t n3, int32_t num_proj, const double *angles,
                                       const double *vectors, const double *d_measured, double *Rarr,
                                       double *Rarr2, double *errR);

/* ---- index and symmetry kernels (host pointers, FP64) -------------------- */

/* CentroSymmetricity(obj, FS, n1, n_k1, n2)
 * (@GENFIRE_Reconstructor/CentroSymmetricity.m:2-72): FS is the
 * (n_k1+1) x (2*floor(n2/2)+1) x (2*floor(n1/2)+1) half grid (k1 <= 0),
 * measuredK the n1 x n2 x n1 full grid. */
genfire_status genfire_centro_symmetricity(genfire_ctx *ctx, const double *FS, int32_t n1,
                                           int32_t n_k1, int32_t n2, double *measuredK);
/* hermitianSymmetrize(in) (src/hermitianSymmetrize.m:22-65). */
genfire_status genfire_hermitian_symmetrize(genfire_ctx *ctx, const double *in, int32_t d1,
                                            int32_t d2, int32_t d3, double *out);
/* Q = make_Kspace_indices(obj) for size(obj) = [d1 d2 d3]
 * (src/make_Kspace_indices.m:16-62). */
genfire_status genfire_make_kspace_indices(genfire_ctx *ctx, int32_t d1, int32_t d2, int32_t d3,
                                           double *Q);
/* My_volumn_index(big_size, ori_size) (src/My_volumn_index.m:3-34): out is
 * 3 x 2 column-major, 1-based [start end]. */
genfire_status genfire_volumn_index(const int32_t big[3], const int32_t ori[3], int32_t out[6]);
/* My_iffshift3_ind(VolSize, Inds) (src/My_iffshift3_ind.m:1-7), 1-based. */
genfire_status genfire_iffshift3_ind(genfire_ctx *ctx, const int32_t size[3], int64_t count,
                                     const int64_t *inds, int64_t *out);
/* K-point selection of one projection (fillInFourierGrid_DFT.m:175-192):
 * the grid points within interpolationCutoffDistance of the rotated plane
 * that pass the in-plane box filter, in ascending 0-based linear index of
 * the half grid (the order of find()).  dist = D, u/v = CP_plane(1:2,:).
 * *count receives the number found; cap bounds the outputs. */
genfire_status genfire_select(genfire_ctx *ctx, const genfire_params *p,
                              double phi, double theta, double psi, int64_t cap,
                              int64_t *ind, float *dist, float *u, float *v, int64_t *count);
/* The library's 3-D FFT (fftn / ifftn semantics: unnormalised forward, 1/N
 * inverse) on an n1 x n2 x n3 complex array, in place; complex128 for FP64,
 * complex64 for MIXED. */
genfire_status genfire_fftn(genfire_ctx *ctx, int32_t precision, void *data, int32_t n1,
                            int32_t n2, int32_t n3, int32_t inverse);

#ifdef __cplusplus
}
#endif

#endif /* GENFIRE_H */
