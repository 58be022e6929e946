/*
 * genfire_run.c -- standalone C driver of libgenfire.so (no MATLAB, no Python).
 *
 * Runs fillInFourierGrid_DFT and reconstruct through the C ABI on a seeded
 * synthetic tilt series (a few Gaussian blobs, projected analytically) and
 * prints sizes, the gridded K-point count, timings and the last errK.
 *
 *   genfire_run [D] [numProjs] [numIterations] [mixed]
 */
#define _POSIX_C_SOURCE 199309L
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "genfire.h"

static double now(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
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

int main(int argc, char **argv)
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

    /* a few Gaussian blobs projected analytically along the rotated axis is
     * approximated here by projecting a voxelised volume with the library */
    size_t nv = (size_t)D * D * D;
    double *vol = calloc(nv, sizeof(double));
    for (int b = 0; b < 6; ++b) {
        double cx = (urand() - 0.5) * D * 0.5, cy = (urand() - 0.5) * D * 0.5, cz = (urand() - 0.5) * D * 0.5;
        for (int k = 0; k < D; ++k)
            for (int j = 0; j < D; ++j)
                for (int i = 0; i < D; ++i) {
                    double x = i - D / 2 - cx, y = j - D / 2 - cy, z = k - D / 2 - cz;
                    vol[i + (size_t)D * (j + (size_t)D * k)] += exp(-(x * x + y * y + z * z) / 8.0);
                }
    }
    double *angles = malloc(sizeof(double) * 3 * P);
    for (int i = 0; i < P; ++i) {
        angles[i] = 360 * urand();
        angles[i + P] = -70 + 140 * urand();
        angles[i + 2 * P] = 360 * urand();
    }
    double *projs = malloc(sizeof(double) * (size_t)D * D * P);
    CHECK(genfire_project(ctx, GENFIRE_PREC_FP64, vol, D, D, D, P, angles, NULL, projs));

    size_t es = mixed ? sizeof(float) : sizeof(double);
    void *M = malloc(2 * es * (size_t)n1 * n2 * n1);
    int64_t *nk = malloc(sizeof(int64_t) * P);
    double t0 = now();
    CHECK(genfire_grid_dft(ctx, &p, projs, angles, M, NULL, nk));
    double t1 = now();
    int64_t tot = 0;
    for (int i = 0; i < P; ++i) tot += nk[i];

    void *rec = malloc(es * nv);
    double *errK = malloc(sizeof(double) * N);
    double t2 = now();
    CHECK(genfire_reconstruct(ctx, &p, M, NULL, NULL, NULL, NULL, NULL, rec, errK, NULL, NULL, NULL));
    double t3 = now();
    printf("D=%d P=%d n=%d %s: gridded points %lld in %.3f s; %d iterations in %.3f s (%.1f it/s); errK %.6f\n",
           D, P, n1, mixed ? "mixed" : "fp64", (long long)tot, t1 - t0, N, t3 - t2, N / (t3 - t2), errK[N - 1]);
    free(vol); free(angles); free(projs); free(M); free(nk); free(rec); free(errK);
    genfire_destroy(ctx);
    return 0;
}
