"""The C ABI without a GPU: the library loads, exports every entry point of
include/genfire.h, its parameter struct matches the header, and the host-only
entry points behave.  No compute entry point is called here."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "genfire.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(genfire_[a-z0-9_]+)\s*\(", txt)))


def test_every_declared_symbol_is_exported(lib):
    from genfire_gb300 import _lib
    L = _lib.load()
    names = declared_functions()
    assert names, "no declarations parsed"
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(_lib.EXPORTS) == names
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    for n in names:
        assert re.search(r"\sT\s%s$" % n, out, flags=re.M), n


def test_params_layout_matches_header(lib):
    from genfire_gb300 import _lib
    fields = [f[0] for f in _lib.Params._fields_]
    src = "#include <stdio.h>\n#include <stddef.h>\n#include \"genfire.h\"\nint main(void){printf(\"%zu\\n\", sizeof(genfire_params));"
    for f in fields:
        src += 'printf("%%zu\\n", offsetof(genfire_params, %s));' % f
    src += "return 0;}\n"
    with tempfile.TemporaryDirectory() as d:
        cf = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(cf, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), cf, "-o", exe], check=True)
        vals = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == C.sizeof(_lib.Params)
    for f, off in zip(fields, vals[1:]):
        assert getattr(_lib.Params, f).offset == off, f


def declared_prototypes():
    """name -> (return type, [parameter types]) for every prototype of the header."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    out = {}
    for ret, name, args in re.findall(r"([A-Za-z_][A-Za-z0-9_ \*]*?)\b(genfire_[a-z0-9_]+)\s*\(([^)]*)\)\s*;",
                                      txt, flags=re.S):
        params = [a.strip() for a in args.split(",") if a.strip() and a.strip() != "void"]
        # drop the parameter name, keep array brackets as a pointer
        types = []
        for a in params:
            is_array = "[" in a
            a = re.sub(r"\[[^\]]*\]", "", a).strip()
            t = re.sub(r"\b[A-Za-z_][A-Za-z0-9_]*$", "", a).strip()
            types.append(t + (" *" if is_array else ""))
        out[name] = (ret.strip(), types)
    return out


def _c_class(t):
    """The calling-convention class of a C type of the header."""
    t = t.replace("const", "").strip()
    if "*" in t:
        return "ptr"
    return {"int32_t": "i32", "int": "i32", "genfire_status": "i32", "int64_t": "i64", "double": "f64"}[t]


def _c_pointee(t):
    """The pointee of a pointer type: a base type name, or 'ptr' for a pointer to a pointer."""
    t = t.replace("const", "").strip()
    assert t.endswith("*")
    t = t[:-1].strip()
    return "ptr" if "*" in t else t


def test_ctypes_signatures_match_header(lib):
    """The Python binding's ctypes table declares every entry point with the
    header's parameter count and classes (pointer, 32-bit integer, 64-bit
    integer, double), and a typed ctypes pointer points to the header's type."""
    from genfire_gb300 import _lib
    L = _lib.load()
    protos = declared_prototypes()
    assert sorted(protos) == declared_functions()
    scalar = {C.c_int32: "i32", C.c_int: "i32", C.c_int64: "i64", C.c_double: "f64"}
    pointee = {C.c_double: "double", C.c_float: "float", C.c_uint8: "uint8_t", C.c_int64: "int64_t",
               C.c_int32: "int32_t", _lib.Params: "genfire_params", C.c_void_p: "ptr"}

    def py_class(ct):
        if ct in (C.c_void_p, C.c_char_p) or (isinstance(ct, type) and issubclass(ct, C._Pointer)):
            return "ptr"
        return scalar[ct]

    for name, (ret, params) in protos.items():
        f = getattr(L, name)
        assert f.argtypes is not None, name
        assert len(f.argtypes) == len(params), name
        want_ret = "i32" if ret == "genfire_status" else _c_class(ret)
        assert py_class(f.restype) == want_ret, name
        for i, (ct, t) in enumerate(zip(f.argtypes, params)):
            assert py_class(ct) == _c_class(t), (name, i, t)
            if isinstance(ct, type) and issubclass(ct, C._Pointer):
                assert pointee[ct._type_] == _c_pointee(t), (name, i, t)


def test_abi_version_and_status_strings(lib):
    from genfire_gb300 import _lib
    L = _lib.load()
    assert L.genfire_abi_version() == 1
    for s in range(7):
        assert L.genfire_status_string(s)
    assert L.genfire_status_string(0) == b"ok"


def test_params_init_defaults(lib):
    """GENFIRE_Reconstructor.m:30-70."""
    p = lib.default_params()
    assert p.oversamplingRatio == 3 and p.interpolationCutoffDistance == 0.7
    assert list(p.vector1) == [0, 0, 1] and list(p.vector2) == [0, 1, 0] and list(p.vector3) == [1, 0, 0]
    assert p.numIterations == 50 and p.constraintEnforcementMode == 1
    assert p.constraintPositivity == 1 and p.constraintSupport == 1 and p.DFT_CentroSymmetricity == 1
    assert p.monitor_R == 0 and p.monitorR_loopLength == 10 and p.precision == lib.PREC_FP64


@pytest.mark.parametrize("D,os_", [(64, 4), (64, 2), (63, 2), (65, 1.5), (7, 2.5)])
def test_grid_size(lib, oracle, D, os_):
    p = lib.default_params()
    p.Dim1, p.Dim2, p.oversamplingRatio = D, D + 1, os_
    assert lib.grid_size(p) == (oracle.oversampled(D, os_), oracle.oversampled(D + 1, os_))


@pytest.mark.parametrize("big,ori", [((16, 16, 16), (8, 8, 8)), ((17, 16, 15), (8, 9, 7)), ((9, 9, 9), (9, 9, 9))])
def test_volumn_index_host(lib, oracle, big, ori):
    assert np.array_equal(lib.volumn_index(big, ori), oracle.volumn_index(big, ori))


def test_volumn_index_rejects_larger_crop(lib):
    with pytest.raises(lib.GenfireError) as e:
        lib.volumn_index((8, 8, 8), (9, 8, 8))
    assert e.value.status == 1 and "GENFIRE:" in str(e.value)


def test_create_reports_errors_without_crashing(lib):
    """No device (or a bad index) is an error status with a message, never a crash."""
    from genfire_gb300 import _lib
    L = _lib.load()
    h = C.c_void_p()
    st = L.genfire_create(4096, C.byref(h))
    assert st in (_lib.GENFIRE_ERR_ARG, _lib.GENFIRE_ERR_CUDA)
    assert not h.value
    assert L.genfire_last_error(None)


def test_null_handles_are_rejected(lib):
    from genfire_gb300 import _lib
    L = _lib.load()
    assert L.genfire_grid_dft(None, None, None, None, None, None, None) == _lib.GENFIRE_ERR_ARG
    assert L.genfire_recon_iterate(None, 1) == _lib.GENFIRE_ERR_ARG
    assert L.genfire_destroy(None) == 0
