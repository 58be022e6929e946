/*
 * genfire_run.c -- standalone C driver of libgenfire.so (no MATLAB, no Python).
 *
 * File mode runs Genfire_test.m without MATLAB: readFiles and CheckPrepareData
 * (GENFIRE_Reconstructor.m:82-170) on MAT files, runGridding (fillInFourierGrid
 * or fillInFourierGrid_DFT), reconstruct, then Tian_calc_Rfactor_realspace and
 * the save of final_Rec, final_errK, final_Rfactor, final_Kfactor,
 * final_Rarray and final_simuProjs (Genfire_test.m:45-64) to a MAT file.
 *
 *   genfire_run --projections pj.mat --angles angles.mat [--support s.mat]
 *               [--initial x0.mat] [--results out.mat] [--oversampling 3]
 *               [--iterations 50] [--cutoff 0.7] [--gridding 1|2] [--mode 1|2|3]
 *               [--positivity 0|1] [--support-constraint 0|1]
 *               [--multiple-matches 0|1] [--centro 0|1] [--vector1 x,y,z]
 *               [--vector2 x,y,z] [--vector3 x,y,z] [--precision fp64|mixed|fp16_scaled]
 *               [--no-rfactor] [--save-temp L [--save-prefix results/temp_rec]]
 *               [--rfree NBINS [--rfree-percent 0.05] [--seed S]]
 *   (defaults: the class defaults of GENFIRE_Reconstructor.m:30-70)
 *
 * Synthetic mode (no --projections) runs fillInFourierGrid_DFT and reconstruct
 * on a seeded synthetic tilt series and prints sizes and timings:
 *
 *   genfire_run [D] [numProjs] [numIterations] [mixed]
 *
 * --mat-info FILE prints the first numeric array of a MAT file (name, size,
 * sum, sum of squares) and exits; --mat-copy IN OUT writes it (as double, or
 * logical) to a new MAT file.
 */
#define _POSIX_C_SOURCE 199309L
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "genfire.h"
#include "matio.h"

static double now(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}

/* host allocations: a failure ends the program with a message */
static void *xmalloc(size_t n)
{
    void *p = malloc(n ? n : 1);
    if (!p) {
        fprintf(stderr, "genfire_run: out of host memory (%zu bytes)\n", n);
        exit(1);
    }
    return p;
}
static void *xcalloc(size_t n, size_t size)
{
    void *p = calloc(n ? n : 1, size ? size : 1);
    if (!p) {
        fprintf(stderr, "genfire_run: out of host memory (%zu x %zu bytes)\n", n, size);
        exit(1);
    }
    return p;
}

static uint64_t rng_state = 88172645463325252ull;
static double urand(void)
{
    rng_state ^= rng_state << 13;
    rng_state ^= rng_state >> 7;
    rng_state ^= rng_state << 17;
    return (rng_state >> 11) * (1.0 / 9007199254740992.0);
}

#define CHECK(call)                                                                      \
    do {                                                                                 \
        genfire_status s_ = (call);                                                      \
        if (s_ != GENFIRE_OK) {                                                          \
            fprintf(stderr, "%s failed: %s (%s)\n", #call, genfire_status_string(s_),    \
                    genfire_last_error(ctx));                                            \
            return 1;                                                                    \
        }                                                                                \
    } while (0)

static int synthetic(int argc, char **argv)
{
    int D = argc > 1 ? atoi(argv[1]) : 32;
    int P = argc > 2 ? atoi(argv[2]) : 20;
    int N = argc > 3 ? atoi(argv[3]) : 50;
    int mixed = argc > 4 && strcmp(argv[4], "mixed") == 0;
    genfire_ctx *ctx = NULL;
    if (genfire_create(0, &ctx) != GENFIRE_OK) {
        fprintf(stderr, "genfire_create: %s\n", genfire_last_error(NULL));
        return 1;
    }
    genfire_params p;
    genfire_params_init(&p);
    p.Dim1 = p.Dim2 = D;
    p.NumProjs = P;
    p.oversamplingRatio = 2;
    p.interpolationCutoffDistance = 0.125;
    p.numIterations = N;
    p.constraintEnforcementMode = 3;
    p.vector3[0] = 0; p.vector3[2] = 1;  /* ZYZ */
    p.precision = mixed ? GENFIRE_PREC_MIXED : GENFIRE_PREC_FP64;
    int32_t n1, n2;
    genfire_grid_size(&p, &n1, &n2);

    /* a few Gaussian blobs, projected with the library's projector */
    size_t nv = (size_t)D * D * D;
    double *vol = xcalloc(nv, sizeof(double));
    for (int b = 0; b < 6; ++b) {
        double cx = (urand() - 0.5) * D * 0.5, cy = (urand() - 0.5) * D * 0.5, cz = (urand() - 0.5) * D * 0.5;
        for (int k = 0; k < D; ++k)
            for (int j = 0; j < D; ++j)
                for (int i = 0; i < D; ++i) {
                    double x = i - D / 2 - cx, y = j - D / 2 - cy, z = k - D / 2 - cz;
                    vol[i + (size_t)D * (j + (size_t)D * k)] += exp(-(x * x + y * y + z * z) / 8.0);
                }
    }
    double *angles = xmalloc(sizeof(double) * 3 * P);
    for (int i = 0; i < P; ++i) {
        angles[i] = 360 * urand();
        angles[i + P] = -70 + 140 * urand();
        angles[i + 2 * P] = 360 * urand();
    }
    double *projs = xmalloc(sizeof(double) * (size_t)D * D * P);
    CHECK(genfire_project(ctx, GENFIRE_PREC_FP64, vol, D, D, D, P, angles, NULL, projs));

    size_t es = mixed ? sizeof(float) : sizeof(double);
    void *M = xmalloc(2 * es * (size_t)n1 * n2 * n1);
    int64_t *nk = xmalloc(sizeof(int64_t) * P);
    double t0 = now();
    CHECK(genfire_grid_dft(ctx, &p, projs, angles, M, NULL, nk));
    double t1 = now();
    int64_t tot = 0;
    for (int i = 0; i < P; ++i) tot += nk[i];

    void *rec = xmalloc(es * nv);
    double *errK = xmalloc(sizeof(double) * N);
    double t2 = now();
    CHECK(genfire_reconstruct(ctx, &p, M, NULL, NULL, NULL, NULL, NULL, rec, errK, NULL, NULL, NULL));
    double t3 = now();
    printf("D=%d P=%d n=%d %s: gridded points %lld in %.3f s; %d iterations in %.3f s (%.1f it/s); errK %.6f\n",
           D, P, n1, mixed ? "mixed" : "fp64", (long long)tot, t1 - t0, N, t3 - t2, N / (t3 - t2), errK[N - 1]);
    free(vol); free(angles); free(projs); free(M); free(nk); free(rec); free(errK);
    genfire_destroy(ctx);
    return 0;
}

static int mat_info(const char *path)
{
    mat_array a;
    char err[256] = {0};
    if (mat_read(path, NULL, &a, err, sizeof err)) {
        fprintf(stderr, "%s\n", err);
        return 1;
    }
    double s = 0, s2 = 0;
    for (int64_t i = 0; i < a.numel; ++i) {
        s += a.re[i];
        s2 += a.re[i] * a.re[i];
    }
    printf("name=%s class=%d logical=%d complex=%d dims=", a.name, a.mx_class, a.is_logical, a.is_complex);
    for (int k = 0; k < a.ndims; ++k) printf(k ? "x%lld" : "%lld", (long long)a.dims[k]);
    printf(" sum=%.17g sumsq=%.17g first=%.17g last=%.17g\n", s, s2, a.numel ? a.re[0] : 0.0,
           a.numel ? a.re[a.numel - 1] : 0.0);
    mat_free(&a);
    return 0;
}

static int mat_copy(const char *in, const char *out)
{
    mat_array a;
    char err[256] = {0};
    if (mat_read(in, NULL, &a, err, sizeof err)) {
        fprintf(stderr, "%s\n", err);
        return 1;
    }
    uint8_t *l = NULL;
    mat_var v = {a.name, a.ndims, a.dims, MAT_DOUBLE, a.re};
    if (a.is_logical) {
        l = xmalloc(a.numel > 0 ? (size_t)a.numel : 1);
        for (int64_t i = 0; i < a.numel; ++i) l[i] = a.re[i] != 0;
        v.mx_class = MAT_LOGICAL;
        v.data = l;
    }
    const int rc = mat_write(out, 1, &v, err, sizeof err);
    if (rc) fprintf(stderr, "%s\n", err);
    free(l);
    mat_free(&a);
    return rc ? 1 : 0;
}

static int vec3(const char *s, double v[3])
{
    return sscanf(s, "%lf,%lf,%lf", &v[0], &v[1], &v[2]) == 3 ? 0 : -1;
}

static int load(const char *what, const char *path, mat_array *a)
{
    char err[256] = {0};
    if (mat_read(path, NULL, a, err, sizeof err)) {
        fprintf(stderr, "GENFIRE: %s file: %s\n", what, err);
        return -1;
    }
    if (a->is_complex) {
        fprintf(stderr, "GENFIRE: %s file holds a complex array\n", what);
        mat_free(a);
        return -1;
    }
    return 0;
}

/* reconstruct through the staged entry points: temporary saves every
 * save_every iterations (reconstruct.m:155-158) and the Rfree monitor
 * (:46-69, :137-146).  The withheld points of each shell are a random
 * permutation of its candidates (Fisher-Yates with this file's xorshift
 * generator, re-seeded before every shell when seed >= 0, as the reference
 * re-seeds rng; MATLAB's randperm stream itself is not reproduced). */
static int staged(genfire_ctx *ctx, const genfire_params *p, const void *M, const uint8_t *support, const void *init,
                  const double *projs, const double *angles, int n1, int n2, int save_every, const char *prefix,
                  int nbins, double pct, long long seed, void *rec, double *errK, double **rfree_out)
{
    const size_t N = (size_t)n1 * n2 * n1, es = p->precision != GENFIRE_PREC_FP64 ? sizeof(float) : sizeof(double);
    uint8_t *mask = NULL;
    int64_t *counts = NULL, *ind = NULL, *wcounts = NULL, *wind = NULL;
    if (nbins > 0) {
        mask = xmalloc(N);
        for (size_t i = 0; i < N; ++i) {
            if (es == sizeof(float)) mask[i] = ((const float *)M)[2 * i] != 0 || ((const float *)M)[2 * i + 1] != 0;
            else mask[i] = ((const double *)M)[2 * i] != 0 || ((const double *)M)[2 * i + 1] != 0;
        }
        counts = xcalloc(nbins, sizeof(int64_t));
        CHECK(genfire_rfree_candidates(ctx, p, M, 0, nbins, counts, NULL));
        int64_t tot = 0;
        for (int s = 0; s < nbins; ++s) tot += counts[s];
        ind = xmalloc(sizeof(int64_t) * (tot > 0 ? tot : 1));
        wind = xmalloc(sizeof(int64_t) * (tot > 0 ? tot : 1));
        wcounts = xcalloc(nbins, sizeof(int64_t));
        CHECK(genfire_rfree_candidates(ctx, p, M, 0, nbins, counts, ind));
        int64_t o = 0, w = 0;
        for (int s = 0; s < nbins; o += counts[s], ++s) {
            if (seed >= 0) {
                rng_state = 88172645463325252ull ^ (uint64_t)seed;
                if (!rng_state) rng_state = 1;  /* xorshift needs a nonzero state */
            }
            int64_t *c = ind + o;
            for (int64_t i = counts[s] - 1; i > 0; --i) {  /* Fisher-Yates */
                const int64_t j = (int64_t)(urand() * (double)(i + 1));
                const int64_t t = c[i]; c[i] = c[j]; c[j] = t;
            }
            int64_t cut = (int64_t)floor((double)counts[s] * pct);
            if (cut == 0) cut = 1;
            if (counts[s] < cut) {
                fprintf(stderr, "GENFIRE: Rfree shell %d has no measured points to withhold.\n", s + 1);
                return 1;
            }
            for (int64_t k = 0; k < cut; ++k) {
                wind[w + k] = c[k];
                mask[c[k]] = 0;
            }
            wcounts[s] = cut;
            w += cut;
        }
    }
    genfire_recon *r = NULL;
    CHECK(genfire_recon_create(ctx, p, M, mask, support, init, projs, angles, 0, &r));
    genfire_status st = nbins > 0 ? genfire_recon_set_rfree(r, nbins, wcounts, wind) : GENFIRE_OK;
    const int D1 = p->Dim1, D2 = p->Dim2, Nit = p->numIterations;
    const int64_t dv[3] = {D1, D2, D1};
    for (int done = 0; st == GENFIRE_OK && done < Nit;) {
        int step = Nit - done;
        if (save_every > 0 && step > save_every - done % save_every) step = save_every - done % save_every;
        st = genfire_recon_iterate(r, step);
        done += step;
        if (st == GENFIRE_OK && save_every > 0 && done % save_every == 0) {
            st = genfire_recon_result(r, rec, NULL, NULL, NULL, NULL, 0);
            char fn[1024], err[256] = {0};
            snprintf(fn, sizeof fn, "%s%d.mat", prefix, done);
            mat_var v = {"temp_reconstruction", 3, dv, es == sizeof(float) ? MAT_SINGLE : MAT_DOUBLE, rec};
            if (st == GENFIRE_OK && mat_write(fn, 1, &v, err, sizeof err)) {
                fprintf(stderr, "GENFIRE: %s\n", err);
                genfire_recon_destroy(r);
                return 1;
            }
        }
    }
    if (st == GENFIRE_OK) st = genfire_recon_result(r, rec, errK, NULL, NULL, NULL, 0);
    if (st == GENFIRE_OK && nbins > 0) {
        *rfree_out = xmalloc(sizeof(double) * (size_t)nbins * (Nit > 0 ? Nit : 1));
        st = genfire_recon_rfree(r, NULL, *rfree_out);
    }
    genfire_recon_destroy(r);
    CHECK(st);
    free(mask); free(counts); free(ind); free(wcounts); free(wind);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc > 2 && !strcmp(argv[1], "--mat-info")) return mat_info(argv[2]);
    if (argc > 3 && !strcmp(argv[1], "--mat-copy")) return mat_copy(argv[2], argv[3]);
    if (argc < 2 || argv[1][0] != '-') return synthetic(argc, argv);

    const char *fproj = NULL, *fang = NULL, *fsup = NULL, *finit = NULL, *fres = "Factor_GENFIRE_test_gdref.mat";
    int want_r = 1, save_every = 0, nbins = 0;
    double rfree_pct = 0.05;
    long long seed = -1;
    const char *save_prefix = "./results/temp_rec";
    genfire_params p;
    genfire_params_init(&p);
    p.griddingMethod = 1;  /* the class default (GENFIRE_Reconstructor.m:44) */
    for (int i = 1; i < argc; ++i) {
        const char *k = argv[i], *v = i + 1 < argc ? argv[i + 1] : NULL;
        int used = 1;
        if (!strcmp(k, "--no-rfactor")) { want_r = 0; used = 0; }
        else if (!v) { fprintf(stderr, "GENFIRE: %s needs a value\n", k); return 2; }
        else if (!strcmp(k, "--projections")) fproj = v;
        else if (!strcmp(k, "--angles")) fang = v;
        else if (!strcmp(k, "--support")) fsup = v;
        else if (!strcmp(k, "--initial")) finit = v;
        else if (!strcmp(k, "--results")) fres = v;
        else if (!strcmp(k, "--oversampling")) p.oversamplingRatio = atof(v);
        else if (!strcmp(k, "--iterations")) p.numIterations = atoi(v);
        else if (!strcmp(k, "--cutoff")) p.interpolationCutoffDistance = atof(v);
        else if (!strcmp(k, "--gridding")) p.griddingMethod = atoi(v);
        else if (!strcmp(k, "--mode")) p.constraintEnforcementMode = atoi(v);
        else if (!strcmp(k, "--positivity")) p.constraintPositivity = atoi(v);
        else if (!strcmp(k, "--support-constraint")) p.constraintSupport = atoi(v);
        else if (!strcmp(k, "--multiple-matches")) p.allowMultipleGridMatches = atoi(v);
        else if (!strcmp(k, "--centro")) p.DFT_CentroSymmetricity = atoi(v);
        else if (!strcmp(k, "--vector1") && !vec3(v, p.vector1)) {}
        else if (!strcmp(k, "--vector2") && !vec3(v, p.vector2)) {}
        else if (!strcmp(k, "--vector3") && !vec3(v, p.vector3)) {}
        else if (!strcmp(k, "--precision")) p.precision = !strcmp(v, "mixed") ? GENFIRE_PREC_MIXED
                                                           : !strcmp(v, "fp16_scaled") ? GENFIRE_PREC_FP16_SCALED : GENFIRE_PREC_FP64;
        else if (!strcmp(k, "--save-temp")) save_every = atoi(v);
        else if (!strcmp(k, "--save-prefix")) save_prefix = v;
        else if (!strcmp(k, "--rfree")) nbins = atoi(v);
        else if (!strcmp(k, "--rfree-percent")) rfree_pct = atof(v);
        else if (!strcmp(k, "--seed")) seed = atoll(v);
        else { fprintf(stderr, "GENFIRE: Invalid option %s provided.\n", k); return 2; }
        i += used;
    }

    /* readFiles (GENFIRE_Reconstructor.m:82-112) */
    if (!fproj) { fprintf(stderr, "GENFIRE: Projections file does not exist!\n"); return 1; }
    if (!fang) { fprintf(stderr, "GENFIRE: Angles file does not exist!\n"); return 1; }
    mat_array pj, an, sp, x0;
    memset(&sp, 0, sizeof sp);
    memset(&x0, 0, sizeof x0);
    if (load("Projections", fproj, &pj) || load("Angles", fang, &an)) return 1;
    if (fsup && load("Support", fsup, &sp)) return 1;
    if (finit && load("Initial Model", finit, &x0)) return 1;

    /* CheckPrepareData (:114-170) */
    p.Dim1 = (int32_t)pj.dims[0];
    p.Dim2 = (int32_t)pj.dims[1];
    p.NumProjs = pj.ndims > 2 ? (int32_t)pj.dims[2] : 1;
    const int P = p.NumProjs, D1 = p.Dim1, D2 = p.Dim2;
    if (an.dims[0] != P) { fprintf(stderr, "GENFIRE: Number of projections and Angles does not match!\n"); return 1; }
    if (an.dims[1] > 3) { fprintf(stderr, "GENFIRE: Input Angle 2nd dimenstions larger than three!\n"); return 1; }
    double *angles = xcalloc(3 * (size_t)P, sizeof(double));
    if (an.dims[1] == 1) memcpy(angles + P, an.re, sizeof(double) * P);  /* [0, theta, 0] */
    else memcpy(angles, an.re, sizeof(double) * 3 * P);
    const size_t nv = (size_t)D1 * D2 * D1;
    if (x0.re && (x0.dims[0] != D1 || x0.dims[1] != D2 || (x0.ndims > 2 ? x0.dims[2] : 1) != D1)) {
        fprintf(stderr, "GENFIRE: Initial Model size does not match with projections!\n");
        return 1;
    }
    if (sp.re && (int64_t)nv != sp.numel) {
        fprintf(stderr, "GENFIRE: Support size does not match with projections!\n");
        return 1;
    }
    if (p.griddingMethod > 2) { fprintf(stderr, "GENFIRE: Unrecognized gridding method.\n"); return 1; }
    const int mixed = p.precision != GENFIRE_PREC_FP64;
    const size_t es = mixed ? sizeof(float) : sizeof(double);
    uint8_t *support = xmalloc(nv);
    for (size_t i = 0; i < nv; ++i) support[i] = sp.re ? sp.re[i] != 0 : 1;
    void *init = NULL;
    if (x0.re) {
        init = xmalloc(es * nv);
        for (size_t i = 0; i < nv; ++i) {
            if (mixed) ((float *)init)[i] = (float)x0.re[i];
            else ((double *)init)[i] = x0.re[i];
        }
    }

    genfire_ctx *ctx = NULL;
    if (genfire_create(0, &ctx) != GENFIRE_OK) {
        fprintf(stderr, "genfire_create: %s\n", genfire_last_error(NULL));
        return 1;
    }
    int32_t n1, n2;
    CHECK(genfire_grid_size(&p, &n1, &n2));

    /* runGridding (:172-186): measuredK (complex64 for MIXED, as the single
     * cast; complex128 in the FP64 drop-in) */
    printf("GENFIRE: Assembling Fourier grid...\n\n");
    void *M = xmalloc(2 * es * (size_t)n1 * n2 * n1);
    double t0 = now();
    if (p.griddingMethod == 1) CHECK(genfire_grid_fft(ctx, &p, pj.re, angles, M, NULL, NULL));
    else CHECK(genfire_grid_dft(ctx, &p, pj.re, angles, M, NULL, NULL));
    double t1 = now();

    /* reconstruct (reconstruct.m:28-194) */
    printf("GENFIRE: Reconstructing... \n\n");
    const int N = p.numIterations;
    void *rec = xmalloc(es * nv);
    double *errK = xmalloc(sizeof(double) * (N > 0 ? N : 1));
    double *rfree = NULL;
    if (save_every <= 0 && nbins <= 0) {
        CHECK(genfire_reconstruct(ctx, &p, M, NULL, support, init, pj.re, angles, rec, errK, NULL, NULL, NULL));
    } else if (staged(ctx, &p, M, support, init, pj.re, angles, n1, n2, save_every, save_prefix, nbins, rfree_pct,
                      seed, rec, errK, &rfree)) {
        return 1;
    }
    double t2 = now();
    printf("GENFIRE: Reconstruction completed in %.12g seconds.\n\n", round(10 * (t2 - t1)) / 10);

    /* Tian_calc_Rfactor_realspace (Genfire_test.m:47-48) and the saved results */
    double *recd = xmalloc(sizeof(double) * nv);
    for (size_t i = 0; i < nv; ++i) recd[i] = mixed ? ((float *)rec)[i] : ((double *)rec)[i];
    double Rtot = 0, Kmin = N > 0 ? errK[0] : 0;
    for (int i = 1; i < N; ++i) Kmin = errK[i] < Kmin ? errK[i] : Kmin;
    double *Rarr = xcalloc(P, sizeof(double));
    float *simu = xcalloc((size_t)D1 * D2 * P, sizeof(float));
    if (want_r)
        CHECK(genfire_rfactor_realspace(ctx, GENFIRE_PREC_FP64, recd, D1, D2, D1, pj.re, D1, D2, P, angles, Rarr, &Rtot,
                                        simu));
    const int64_t dv[3] = {D1, D2, D1}, dk[2] = {1, N}, d1[2] = {1, 1}, dr[2] = {P, 1}, ds[3] = {D1, D2, P};
    const int64_t dfree[2] = {nbins, N};
    mat_var vars[7] = {
        {"final_Rec", 3, dv, mixed ? MAT_SINGLE : MAT_DOUBLE, rec},
        {"final_errK", 2, dk, MAT_DOUBLE, errK},
        {"final_Kfactor", 2, d1, MAT_DOUBLE, &Kmin},
        {"final_Rfactor", 2, d1, MAT_DOUBLE, &Rtot},
        {"final_Rarray", 2, dr, MAT_DOUBLE, Rarr},
        {"final_simuProjs", 3, ds, MAT_SINGLE, simu},
        {"final_Rfree", 2, dfree, MAT_DOUBLE, rfree},
    };
    int nvar = want_r ? 6 : 3;
    if (rfree) vars[nvar++] = vars[6];
    char err[256] = {0};
    if (mat_write(fres, nvar, vars, err, sizeof err)) {
        fprintf(stderr, "GENFIRE: %s\n", err);
        return 1;
    }
    printf("D=%dx%d P=%d n=%dx%d %s gridding %d: %.3f s; %d iterations: %.3f s; errK min %.6f; Rfactor %.6f; saved %s\n",
           D1, D2, P, n1, n2, mixed ? "mixed" : "fp64", p.griddingMethod, t1 - t0, N, t2 - t1, Kmin, Rtot, fres);
    free(angles); free(support); free(init); free(M); free(rec); free(errK); free(recd); free(Rarr); free(simu);
    free(rfree);
    mat_free(&pj); mat_free(&an); mat_free(&sp); mat_free(&x0);
    genfire_destroy(ctx);
    return 0;
}
