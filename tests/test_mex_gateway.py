"""The MEX gateway mex/genfire_mex.c compiles against include/genfire.h.

MATLAB and its mex.h are not available here, so the gateway is compiled
with gcc against a minimal stand-in
mex.h that declares the MATLAB C API names the gateway uses, with their
published signatures.  A change of a genfire.h entry point that the
documented gateway no longer matches (a renamed function, a changed argument
list or type) fails this test.  CPU only: nothing is linked or run."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MEX_H = r"""
#ifndef MEX_STANDIN_H
#define MEX_STANDIN_H
#include <stddef.h>
#include <stdbool.h>
typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef size_t mwIndex;
typedef enum { mxREAL, mxCOMPLEX } mxComplexity;
typedef enum { mxUNKNOWN_CLASS, mxCELL_CLASS, mxSTRUCT_CLASS, mxLOGICAL_CLASS, mxCHAR_CLASS, mxVOID_CLASS,
               mxDOUBLE_CLASS, mxSINGLE_CLASS, mxINT8_CLASS, mxUINT8_CLASS, mxINT16_CLASS, mxUINT16_CLASS,
               mxINT32_CLASS, mxUINT32_CLASS, mxINT64_CLASS, mxUINT64_CLASS } mxClassID;
typedef bool mxLogical;
typedef double mxDouble;
typedef float mxSingle;
typedef struct { mxSingle real, imag; } mxComplexSingle;
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
int mexAtExit(void (*exit_fcn)(void));
void mexErrMsgIdAndTxt(const char *identifier, const char *err_msg, ...);
void mexErrMsgTxt(const char *error_msg);
void *mxCalloc(size_t n, size_t size);
mxArray *mxCreateCellMatrix(mwSize m, mwSize n);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity complexFlag);
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID classid, mxComplexity ComplexFlag);
mxArray *mxGetCell(const mxArray *pm, mwIndex index);
void mxSetCell(mxArray *pm, mwIndex index, mxArray *value);
mxComplexSingle *mxGetComplexSingles(const mxArray *pa);
mxDouble *mxGetDoubles(const mxArray *pa);
mxSingle *mxGetSingles(const mxArray *pa);
mxLogical *mxGetLogicals(const mxArray *pa);
size_t mxGetNumberOfElements(const mxArray *pm);
mxArray *mxGetProperty(const mxArray *pa, mwIndex index, const char *propname);
double mxGetScalar(const mxArray *pm);
int mxGetString(const mxArray *pm, char *str, mwSize strlen);
bool mxIsEmpty(const mxArray *pm);
#endif
"""


GATEWAY = os.path.join(ROOT, "mex", "genfire_mex.c")
SHIMS = ["fillInFourierGrid_DFT.m", "fillInFourierGrid.m", "reconstruct.m"]


def test_gateway_compiles_against_the_abi(tmp_path):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not available")
    (tmp_path / "mex.h").write_text(MEX_H)
    src = GATEWAY
    r = subprocess.run([gcc, "-std=c11", "-fsyntax-only", "-Wall", "-Werror=implicit-function-declaration",
                        "-Werror=incompatible-pointer-types", "-Werror=int-conversion",
                        "-I", str(tmp_path), "-I", os.path.join(ROOT, "include"), src],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr


def test_shims_call_the_gateway():
    """Each .m shim keeps the reference method's signature and calls genfire_mex."""
    for name in SHIMS:
        text = open(os.path.join(ROOT, "mex", "@GENFIRE_Reconstructor", name)).read()
        assert text.startswith("function obj = %s(obj)" % name[:-2])
        assert "genfire_mex(" in text
