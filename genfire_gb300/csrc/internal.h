// internal.h -- host-side interfaces shared by the translation units of libgenfire.
#pragma once

#include "common.cuh"

namespace gf {
struct ReconBase;
}

// The handle behind genfire_recon.
struct genfire_recon {
    genfire_ctx *ctx;
    gf::ReconBase *impl;
};

// The handle behind genfire_recon_batch: member reconstructions (not owned)
// and the instantiated graph of one iteration of all of them.
struct genfire_recon_batch {
    genfire_ctx *ctx;
    std::vector<genfire_recon *> members;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaStream_t> branches;  // the capture's branch streams (kept for the graph's lifetime)
    std::vector<cudaEvent_t> events;     // its fork and join events
};

namespace gf {

// ---------------------------------------------------------------- geometry
// FP32 geometry of one projection, computed on the host with a fixed
// operation order (this file is compiled with -ffp-contract=off):
// R = single(Q(v1,phi) Q(v2,theta) Q(v3,psi)) (fillInFourierGrid_DFT.m:108-118),
// nrm = R(:,3) (normVECs), h = nrm / norm(nrm) (distancePointsPlane_YY :332),
// nsq = sum(nrm.*nrm) (closestpoint :347) and the pivoted LU factors of R that
// mldivide uses for R \ CP (:182).
struct ProjGeom {
    float R[9];
    float nrm[3];
    float h[3];
    float nsq;
    float ih;  // 1 / h[0] (IEEE division; used only when |h[0]| >= 0.01)
    float lu[9];
    int piv[3];
};

int oversampled(int dim, double ratio);
void quat_rot(const double v[3], double theta_deg, double R[9]);
void euler_rot(const double v1[3], const double v2[3], const double v3[3], double phi, double theta,
               double psi, double R[9]);
void rot_zyz(double phi, double theta, double psi, double R[9]);
void proj_geometry(const genfire_params &p, double phi, double theta, double psi, ProjGeom &g);

// Gridded index space (fillInFourierGrid_DFT.m:122-144): k1 in [lo1, lo1+l1), ...
struct GridSpec {
    int lo1, lo2, lo3, l1, l2, l3;
    long long total;
};
GridSpec make_grid(int n1, int n2, int centro);

// Validates the parameters; throws Error on failure.
void check_params(const genfire_params &p, bool need_projs);

// ---------------------------------------------------------------- gridding
// fillInFourierGrid_DFT on device buffers: d_proj (D1 x D2 x P double),
// angles on the host (P x 3), d_M (n1 x n2 x n1, centred, complex128 for
// FP64 / complex64 for MIXED), d_rec optional (D1 x D2 x D1 double / float).
// stage_ms (optional, 6 entries): device time of the selection, the DFT stage,
// the DFT kernel alone, the weighted sums, the average/mirror/cast and the
// recIFFT, from CUDA events on the context stream.
void grid_dft(genfire_ctx *ctx, const genfire_params &p, const double *d_proj, const double *angles,
              void *d_M, void *d_rec, int64_t *nk, double *stage_ms = nullptr);

// Grid sizes of measuredK for the params' gridding method: DFT (griddingMethod
// != 1) n1 x n2 x n1 with n = round(Dim * ratio); FFT (griddingMethod 1,
// fillInFourierGrid.m:38-42) an m x m x m cube from Dim2 (n1 = n2 = m).
void grid_dims(const genfire_params &p, int &n1, int &n2);
// Cube size of fillInFourierGrid, -1 when Dim2 * ratio (or 1 + (Dim2-1) * ratio
// for odd Dim2) is not an integer.
int fft_grid_size(int Dim2, double ratio);

// fillInFourierGrid (griddingMethod 1) on device buffers: d_proj (D1 x D2 x P
// double), angles on the host, d_M (m x m x m centred, complex128 / complex64),
// d_rec optional (D1 x D2 x D1); *npairs (optional) = gridded (voxel, value) pairs.
void grid_fft(genfire_ctx *ctx, const genfire_params &p, const double *d_proj, const double *angles,
              void *d_M, void *d_rec, int64_t *npairs);

// Reduced-precision DFT of all selected points on the tensor cores
// (grid_mma.cu): F[j] (complex64) for the points of every projection (counts
// nk, offsets off); split-BF16 operands, or split-FP16 operands with
// per-projection power-of-two scaling when fp16.
// d_off: the points' offsets per projection on the device (P + 1 entries);
// d_err (device, zeroed by the caller) is set when a bounded wait expired.  The
// call does not synchronise; ev_begin / ev_end (may be null) are recorded
// around the DFT kernel.
void dft_tcgen05(genfire_ctx *ctx, const double *d_proj, int D1, int D2, int n1, int n2, int P,
                 const std::vector<long long> &nk, const long long *d_off, const float *d_u, const float *d_v,
                 float2 *d_F, int *d_err, cudaEvent_t ev_begin, cudaEvent_t ev_end, bool fp16);

// Selection of one projection into host arrays (test entry point).
long long select_one(genfire_ctx *ctx, const genfire_params &p, double phi, double theta, double psi,
                     long long cap, int64_t *ind, float *dist, float *u, float *v);

// CentroSymmetricity on device buffers (FS complex128 half grid -> M complex128).
void centro_device(genfire_ctx *ctx, const double2 *d_FS, int n1, int n_k1, int n2, double2 *d_M);
void hermitian_device(genfire_ctx *ctx, const double2 *d_in, int d1, int d2, int d3, double2 *d_out);
void kspace_device(genfire_ctx *ctx, int d1, int d2, int d3, double *d_Q);
void iffshift_device(genfire_ctx *ctx, const int sz[3], long long count, const long long *d_in,
                     long long *d_out);

// ---------------------------------------------------------------- FFT / iteration
// real(ifftn(ifftshift(M))) cropped to the centred D1 x D2 x D1 box
// (the recIFFT of fillInFourierGrid_DFT.m:304).
void rec_ifft(genfire_ctx *ctx, int precision, const void *d_M, int n1, int n2, int D1, int D2, void *d_rec);

// In-place 3-D FFT (fftn/ifftn semantics) of an n1 x n2 x n3 complex array
// along the dimensions set in axes (bit 0 = dim 1; 7 = all three).
void fftn_device(genfire_ctx *ctx, int precision, void *d_data, int n1, int n2, int n3, bool inverse, int axes = 7);

// The staged iteration behind genfire_recon_* (dr.cu).
genfire_recon *recon_create(genfire_ctx *ctx, const genfire_params &p, const void *M, const uint8_t *mask,
                            const uint8_t *support, const void *initial, const double *projs,
                            const double *angles, bool on_device);
void recon_iterate(genfire_recon *r, int count);
void recon_result(genfire_recon *r, void *rec, double *errK, double *errR, double *Rarr, double *Rarr2,
                  bool on_device);
void recon_destroy(genfire_recon *r);
genfire_recon_batch *recon_batch_create(genfire_ctx *ctx, genfire_recon *const *members, int count);
void recon_batch_iterate(genfire_recon_batch *b, int count);
void recon_batch_destroy(genfire_recon_batch *b);
void recon_profile(genfire_recon *r, int iterations, double *ms, double *bytes);
void recon_tuning(genfire_recon *r, int *variants);
void recon_set_rfree(genfire_recon *r, int nshells, const int64_t *counts, const int64_t *indices);
int recon_rfree(genfire_recon *r, double *out);
void rfree_candidates(genfire_ctx *ctx, const genfire_params &p, const void *M, bool on_device, int nbins,
                      int64_t *counts, int64_t *indices);

// ---------------------------------------------------------------- projector
// Trilinear projections of a volume view (base pointer, strides vs1 = stride
// of dim 2, vs2 = stride of dim 3 in elements) for P rotation matrices
// (d_R: P x 9 doubles, column-major each).  d_proj (n1 x n2 x P, may be
// nullptr).  When d_measured is given, d_sums (P x 4 doubles) receives
// sum|bp-pj|, sum|pj|, sum (bp-pj)^2, sum pj^2 per projection.
void project_batch(genfire_ctx *ctx, int precision, const void *d_vol, int n1, int n2, int n3,
                   long long vs1, long long vs2, int P, const double *d_R, void *d_proj,
                   const double *d_measured, double *d_sums, cudaStream_t stream);

// Tian_calc_Rfactor_realspace on device buffers: d_model (m1 x m2 x m3),
// d_projs (p1 x p2 x P double), host angles; Rarr (P) and Rtotal on the host,
// d_simu (p1 x p2 x P float, optional) on the device.
void rfactor_realspace(genfire_ctx *ctx, int precision, const void *d_model, int m1, int m2, int m3, int P,
                       const double *angles, const double *d_projs, int p1, int p2, double *Rarr, double *Rtotal,
                       float *d_simu);

// R-factors with the scratch in a static device array (no allocation); host
// angles/vectors and outputs as genfire_rfactor.
size_t rfactor_noalloc_bytes(int n1, int n2, int P);
void rfactor_noalloc(genfire_ctx *ctx, int precision, const void *d_vol, int n1, int n2, int n3, int P,
                     const double *angles, const double *vectors, const double *d_measured, double *Rarr,
                     double *Rarr2, double *errR);

}  // namespace gf
