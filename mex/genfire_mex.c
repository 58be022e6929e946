/* genfire_mex.c -- MEX gateway: genfire_mex(cmd, obj, ...) over libgenfire.so
 * mex -R2018a genfire_mex.c -I<repo>/include -L<repo>/genfire_gb300/_build -lgenfire */
#include <string.h>
#include "mex.h"
#include "genfire.h"

static genfire_ctx *g_ctx = NULL;
static void at_exit(void) { if (g_ctx) genfire_destroy(g_ctx); g_ctx = NULL; }
static genfire_ctx *ctx(void)
{
    if (!g_ctx) {
        if (genfire_create(0, &g_ctx) != GENFIRE_OK)
            mexErrMsgIdAndTxt("GENFIRE:device", "%s", genfire_last_error(NULL));
        mexAtExit(at_exit);
    }
    return g_ctx;
}
static double prop(const mxArray *obj, const char *name) { return mxGetScalar(mxGetProperty(obj, 0, name)); }
static void vec(const mxArray *obj, const char *name, double v[3])
{
    const double *p = mxGetDoubles(mxGetProperty(obj, 0, name));
    v[0] = p[0]; v[1] = p[1]; v[2] = p[2];
}
static void params(const mxArray *obj, genfire_params *p)
{
    genfire_params_init(p);
    p->Dim1 = (int32_t)prop(obj, "Dim1");
    p->Dim2 = (int32_t)prop(obj, "Dim2");
    p->NumProjs = (int32_t)prop(obj, "NumProjs");
    p->DFT_CentroSymmetricity = (int32_t)prop(obj, "DFT_CentroSymmetricity");
    p->oversamplingRatio = prop(obj, "oversamplingRatio");
    p->interpolationCutoffDistance = prop(obj, "interpolationCutoffDistance");
    vec(obj, "vector1", p->vector1); vec(obj, "vector2", p->vector2); vec(obj, "vector3", p->vector3);
    p->numIterations = (int32_t)prop(obj, "numIterations");
    p->constraintEnforcementMode = (int32_t)prop(obj, "constraintEnforcementMode");
    p->constraintPositivity = (int32_t)prop(obj, "constraintPositivity");
    p->constraintSupport = (int32_t)prop(obj, "constraintSupport");
    p->monitor_R = (int32_t)prop(obj, "monitor_R");
    p->monitorR_loopLength = (int32_t)prop(obj, "monitorR_loopLength");
    p->precision = GENFIRE_PREC_MIXED;   /* single measuredK, as runGridding stores it */
}
static void check(genfire_status s)
{
    if (s != GENFIRE_OK) mexErrMsgIdAndTxt("GENFIRE:lib", "%s", genfire_last_error(g_ctx));
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    char cmd[32];
    genfire_params p;
    if (nrhs < 2 || mxGetString(prhs[0], cmd, sizeof cmd)) mexErrMsgTxt("GENFIRE: genfire_mex(cmd, obj)");
    params(prhs[1], &p);
    int32_t n1, n2;
    genfire_grid_size(&p, &n1, &n2);
    if (!strcmp(cmd, "grid_dft")) {                      /* fillInFourierGrid_DFT */
        mwSize dm[3] = {n1, n2, n1}, dr[3] = {p.Dim1, p.Dim2, p.Dim1};
        plhs[0] = mxCreateNumericArray(3, dm, mxSINGLE_CLASS, mxCOMPLEX);
        plhs[1] = mxCreateNumericArray(3, dr, mxSINGLE_CLASS, mxREAL);
        check(genfire_grid_dft(ctx(), &p, mxGetDoubles(mxGetProperty(prhs[1], 0, "InputProjections")),
                               mxGetDoubles(mxGetProperty(prhs[1], 0, "InputAngles")),
                               mxGetComplexSingles(plhs[0]), mxGetSingles(plhs[1]), NULL));
    } else if (!strcmp(cmd, "grid_fft")) {               /* fillInFourierGrid (griddingMethod 1) */
        int32_t m, m2;
        p.griddingMethod = 1;
        p.allowMultipleGridMatches = (int32_t)prop(prhs[1], "allowMultipleGridMatches");
        check(genfire_grid_size(&p, &m, &m2));
        mwSize dm[3] = {m, m, m}, dr[3] = {p.Dim1, p.Dim2, p.Dim1};
        plhs[0] = mxCreateNumericArray(3, dm, mxSINGLE_CLASS, mxCOMPLEX);
        plhs[1] = mxCreateNumericArray(3, dr, mxSINGLE_CLASS, mxREAL);
        check(genfire_grid_fft(ctx(), &p, mxGetDoubles(mxGetProperty(prhs[1], 0, "InputProjections")),
                               mxGetDoubles(mxGetProperty(prhs[1], 0, "InputAngles")),
                               mxGetComplexSingles(plhs[0]), mxGetSingles(plhs[1]), NULL));
    } else if (!strcmp(cmd, "reconstruct")) {            /* reconstruct */
        mxArray *M = mxGetProperty(prhs[1], 0, "measuredK");
        mxArray *mask = mxGetProperty(prhs[1], 0, "measuredK_mask");
        mxArray *S = mxGetProperty(prhs[1], 0, "Support");
        mxArray *x0 = mxGetProperty(prhs[1], 0, "initialObject");
        mwSize dr[3] = {p.Dim1, p.Dim2, p.Dim1};
        p.griddingMethod = (int32_t)prop(prhs[1], "griddingMethod");   /* grid = size(measuredK) */
        int nm = p.monitor_R == 1 ? p.numIterations / p.monitorR_loopLength : 0;
        plhs[0] = mxCreateNumericArray(3, dr, mxSINGLE_CLASS, mxREAL);
        plhs[1] = mxCreateDoubleMatrix(1, p.numIterations, mxREAL);
        plhs[2] = mxCreateDoubleMatrix(1, nm, mxREAL);
        plhs[3] = mxCreateDoubleMatrix(p.NumProjs, nm, mxREAL);
        plhs[4] = mxCreateDoubleMatrix(p.NumProjs, nm, mxREAL);
        check(genfire_reconstruct(ctx(), &p, mxGetComplexSingles(M),
                                  mxIsEmpty(mask) ? NULL : (const uint8_t *)mxGetLogicals(mask),
                                  mxIsEmpty(S) ? NULL : (const uint8_t *)mxGetLogicals(S),
                                  mxIsEmpty(x0) ? NULL : mxGetSingles(x0),
                                  mxGetDoubles(mxGetProperty(prhs[1], 0, "InputProjections")),
                                  mxGetDoubles(mxGetProperty(prhs[1], 0, "InputAngles")),
                                  mxGetSingles(plhs[0]), mxGetDoubles(plhs[1]), mxGetDoubles(plhs[2]),
                                  mxGetDoubles(plhs[3]), mxGetDoubles(plhs[4])));
    } else if (!strcmp(cmd, "rfree_candidates")) {       /* reconstruct.m:47-50, all shells */
        int32_t nb = (int32_t)prop(prhs[1], "numBinsRfree");
        mxArray *M = mxGetProperty(prhs[1], 0, "measuredK");
        p.griddingMethod = (int32_t)prop(prhs[1], "griddingMethod");
        int64_t *counts = (int64_t *)mxCalloc(nb, sizeof(int64_t)), tot = 0;
        check(genfire_rfree_candidates(ctx(), &p, mxGetComplexSingles(M), 0, nb, counts, NULL));
        for (int s = 0; s < nb; ++s) tot += counts[s];
        int64_t *ind = (int64_t *)mxCalloc(tot > 0 ? tot : 1, sizeof(int64_t));
        check(genfire_rfree_candidates(ctx(), &p, mxGetComplexSingles(M), 0, nb, counts, ind));
        plhs[0] = mxCreateCellMatrix(1, nb);
        for (int s = 0, o = 0; s < nb; o += (int)counts[s], ++s) {
            mxArray *v = mxCreateDoubleMatrix(counts[s], 1, mxREAL);
            double *d = mxGetDoubles(v);
            for (int64_t k = 0; k < counts[s]; ++k) d[k] = (double)(ind[o + k] + 1);   /* 1-based, as find */
            mxSetCell(plhs[0], s, v);
        }
    } else if (!strcmp(cmd, "reconstruct_rfree")) {      /* reconstruct with withheld shells */
        const mxArray *cells = prhs[2];                   /* 1 x nshells cell of 1-based indices */
        int32_t ns = (int32_t)mxGetNumberOfElements(cells);
        int64_t *counts = (int64_t *)mxCalloc(ns > 0 ? ns : 1, sizeof(int64_t)), tot = 0;
        for (int s = 0; s < ns; ++s) tot += (counts[s] = (int64_t)mxGetNumberOfElements(mxGetCell(cells, s)));
        int64_t *ind = (int64_t *)mxCalloc(tot > 0 ? tot : 1, sizeof(int64_t));
        for (int s = 0, o = 0; s < ns; o += (int)counts[s], ++s) {
            const double *d = mxGetDoubles(mxGetCell(cells, s));
            for (int64_t k = 0; k < counts[s]; ++k) ind[o + k] = (int64_t)d[k] - 1;
        }
        mxArray *M = mxGetProperty(prhs[1], 0, "measuredK");
        mxArray *mask = mxGetProperty(prhs[1], 0, "measuredK_mask");   /* withheld points cleared */
        mxArray *S = mxGetProperty(prhs[1], 0, "Support");
        mxArray *x0 = mxGetProperty(prhs[1], 0, "initialObject");
        mwSize dr[3] = {p.Dim1, p.Dim2, p.Dim1};
        p.griddingMethod = (int32_t)prop(prhs[1], "griddingMethod");
        int nm = p.monitor_R == 1 ? p.numIterations / p.monitorR_loopLength : 0;
        genfire_recon *r = NULL;
        check(genfire_recon_create(ctx(), &p, mxGetComplexSingles(M), (const uint8_t *)mxGetLogicals(mask),
                                   mxIsEmpty(S) ? NULL : (const uint8_t *)mxGetLogicals(S),
                                   mxIsEmpty(x0) ? NULL : mxGetSingles(x0),
                                   mxGetDoubles(mxGetProperty(prhs[1], 0, "InputProjections")),
                                   mxGetDoubles(mxGetProperty(prhs[1], 0, "InputAngles")), 0, &r));
        plhs[0] = mxCreateNumericArray(3, dr, mxSINGLE_CLASS, mxREAL);
        plhs[1] = mxCreateDoubleMatrix(1, p.numIterations, mxREAL);
        plhs[2] = mxCreateDoubleMatrix(1, nm, mxREAL);
        plhs[3] = mxCreateDoubleMatrix(p.NumProjs, nm, mxREAL);
        plhs[4] = mxCreateDoubleMatrix(p.NumProjs, nm, mxREAL);
        plhs[5] = mxCreateDoubleMatrix(ns, p.numIterations, mxREAL);     /* Rfree_complex */
        genfire_status st = genfire_recon_set_rfree(r, ns, counts, ind);
        if (st == GENFIRE_OK) st = genfire_recon_iterate(r, p.numIterations);
        if (st == GENFIRE_OK)
            st = genfire_recon_result(r, mxGetSingles(plhs[0]), mxGetDoubles(plhs[1]), mxGetDoubles(plhs[2]),
                                      mxGetDoubles(plhs[3]), mxGetDoubles(plhs[4]), 0);
        if (st == GENFIRE_OK) st = genfire_recon_rfree(r, NULL, mxGetDoubles(plhs[5]));
        genfire_recon_destroy(r);
        check(st);
    } else {
        mexErrMsgIdAndTxt("GENFIRE:cmd", "GENFIRE: unknown command %s", cmd);
    }
}
