"""MAT-file (Level 5) reading and writing of the standalone C harness
(genfire_gb300/harness/matio.c), against scipy.io: plain and zlib-compressed
variables of every numeric class, logical arrays, small and long names,
non-numeric variables skipped, malformed files rejected.  CPU only: the
harness's --mat-info / --mat-copy modes call no GPU function."""
import os
import subprocess

import numpy as np
import pytest

scipy_io = pytest.importorskip("scipy.io")


@pytest.fixture(scope="module")
def harness():
    from genfire_gb300 import build
    build.build()
    return build.HARNESS


def _info(harness, path):
    r = subprocess.run([harness, "--mat-info", path], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    out = {}
    for tok in r.stdout.split():
        k, v = tok.split("=", 1)
        out[k] = v
    return out


def _seq_sum(a):
    """Sum in column-major order, one term after another (the harness's order)."""
    f = np.asarray(a, dtype=np.float64).ravel(order="F")
    return float(np.cumsum(f)[-1]) if f.size else 0.0


CLASSES = [np.float64, np.float32, np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64, np.uint64]


@pytest.mark.parametrize("compress", [False, True])
@pytest.mark.parametrize("dt", CLASSES)
def test_read_numeric_classes(harness, tmp_path, compress, dt):
    rng = np.random.default_rng(3)
    a = np.asfortranarray((rng.random((5, 7, 3)) * 100).astype(dt))
    f = str(tmp_path / "a.mat")
    scipy_io.savemat(f, {"pj": a}, do_compression=compress)
    info = _info(harness, f)
    assert info["name"] == "pj" and info["dims"] == "5x7x3" and info["complex"] == "0"
    flat = a.astype(np.float64).ravel(order="F")
    assert float(info["sum"]) == _seq_sum(a)
    assert float(info["first"]) == flat[0] and float(info["last"]) == flat[-1]


@pytest.mark.parametrize("compress", [False, True])
def test_first_numeric_after_other_variables(harness, tmp_path, compress):
    """importdata of a one-array file is that array; text and cells are skipped."""
    f = str(tmp_path / "b.mat")
    x = np.arange(12.0).reshape(3, 4, order="F")
    scipy_io.savemat(f, {"a_note": "projections of the test", "b_cell": np.array([[1.0, "x"]], dtype=object),
                         "c": x}, do_compression=compress)
    info = _info(harness, f)
    assert info["name"] == "c" and info["dims"] == "3x4" and float(info["sum"]) == 66.0


@pytest.mark.parametrize("compress", [False, True])
def test_copy_round_trip(harness, tmp_path, compress):
    rng = np.random.default_rng(5)
    src, dst = str(tmp_path / "s.mat"), str(tmp_path / "d.mat")
    a = np.asfortranarray(rng.standard_normal((64, 64, 9)))
    scipy_io.savemat(src, {"projections_with_a_long_name": a}, do_compression=compress)
    r = subprocess.run([harness, "--mat-copy", src, dst], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    back = scipy_io.loadmat(dst)
    assert np.array_equal(back["projections_with_a_long_name"], a)


def test_logical_round_trip(harness, tmp_path):
    src, dst = str(tmp_path / "s.mat"), str(tmp_path / "d.mat")
    m = np.asfortranarray(np.random.default_rng(1).random((6, 5, 6)) > 0.5)
    scipy_io.savemat(src, {"sup": m}, do_compression=True)
    assert _info(harness, src)["logical"] == "1"
    r = subprocess.run([harness, "--mat-copy", src, dst], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    # scipy reads logical arrays (its own included) as uint8; the flag is checked on our side
    back = scipy_io.loadmat(dst)["sup"]
    assert np.array_equal(back.astype(bool), m) and back.max() == 1
    assert _info(harness, dst)["logical"] == "1"


def test_rejects_bad_files(harness, tmp_path):
    f = str(tmp_path / "t.mat")
    scipy_io.savemat(f, {"x": np.arange(1000.0)}, do_compression=True)
    raw = open(f, "rb").read()
    for k, data in enumerate([raw[:60], raw[:200], raw[:128] + bytes(40), b"MATLAB 7.3 MAT-file" + bytes(200)]):
        g = str(tmp_path / ("bad%d.mat" % k))
        open(g, "wb").write(data)
        r = subprocess.run([harness, "--mat-info", g], capture_output=True, text=True, timeout=60)
        assert r.returncode == 1 and r.stderr.strip(), (k, r.stdout)
    # a flipped byte inside the compressed stream fails its checksum or its codes
    bad = bytearray(raw)
    bad[len(bad) // 2] ^= 0x5A
    g = str(tmp_path / "flip.mat")
    open(g, "wb").write(bytes(bad))
    r = subprocess.run([harness, "--mat-info", g], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1


# the reference's data_turb3 folder, found through GENFIRE_REFERENCE (the reference tree)
REF_DATA = os.path.join(os.environ.get("GENFIRE_REFERENCE", ""), "data_turb3")


@pytest.mark.skipif(not os.environ.get("GENFIRE_REFERENCE") or not os.path.isdir(REF_DATA),
                    reason="GENFIRE_REFERENCE does not name a reference tree with data_turb3 on this machine")
def test_reference_data_files(harness):
    """The reference's own compressed MAT files read as scipy reads them."""
    for fn in sorted(os.listdir(REF_DATA)):
        if not fn.endswith(".mat"):
            continue
        path = os.path.join(REF_DATA, fn)
        d = {k: v for k, v in scipy_io.loadmat(path).items() if not k.startswith("__")}
        (name, arr), = d.items()
        info = _info(harness, path)
        assert info["name"] == name
        assert info["dims"] == "x".join(str(s) for s in arr.shape)
        assert float(info["sum"]) == _seq_sum(arr)


def test_read_randomized(harness, tmp_path):
    """Random shapes (including empty and large ones that compress into many
    DEFLATE blocks), numeric classes, value ranges, names and compression,
    written by scipy and read back by the harness's reader and inflater."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=40, deadline=None, derandomize=True)
    @hyp.given(shape=st.lists(st.integers(0, 40), min_size=2, max_size=4), dt=st.sampled_from(CLASSES),
               compress=st.booleans(), scale=st.sampled_from([1.0, 100.0, 1e6]), runs=st.booleans(),
               name=st.from_regex(r"[a-z][a-z0-9_]{0,30}", fullmatch=True), seed=st.integers(0, 2 ** 16))
    def check(shape, dt, compress, scale, runs, name, seed):
        rng = np.random.default_rng(seed)
        n = int(np.prod(shape))
        if runs:   # long runs of repeated values: back-references in the compressed stream
            v = np.repeat(rng.random(max(1, n // 50 + 1)), 50)[:n]
        else:
            v = rng.random(n)
        if np.issubdtype(dt, np.integer):
            lo, hi = np.iinfo(dt).min, np.iinfo(dt).max
            v = np.clip(np.round(v * scale * (1 if lo == 0 else 2) - (0 if lo == 0 else scale)), max(lo, -2 ** 52),
                        min(hi, 2 ** 52))
        else:
            v = v * scale
        a = np.asfortranarray(v.astype(dt).reshape(shape, order="F"))
        f = str(tmp_path / "r.mat")
        scipy_io.savemat(f, {name: a}, do_compression=compress)
        d = {k: x for k, x in scipy_io.loadmat(f).items() if not k.startswith("__")}
        (nm, arr), = d.items()
        info = _info(harness, f)
        assert info["name"] == nm
        assert info["dims"] == "x".join(str(s) for s in arr.shape)
        assert float(info["sum"]) == _seq_sum(arr)

    check()


def test_copy_randomized(harness, tmp_path):
    """Random arrays of every numeric class through --mat-copy (reader, then
    the Level-5 writer of double arrays): scipy reads back the same values."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=25, deadline=None, derandomize=True)
    @hyp.given(shape=st.lists(st.integers(1, 30), min_size=2, max_size=4), dt=st.sampled_from(CLASSES),
               compress=st.booleans(), seed=st.integers(0, 2 ** 16))
    def check(shape, dt, compress, seed):
        rng = np.random.default_rng(seed)
        v = rng.standard_normal(int(np.prod(shape))) * 1000
        if np.issubdtype(dt, np.integer):
            v = np.abs(v) if np.iinfo(dt).min == 0 else v
            v = np.clip(np.round(v), np.iinfo(dt).min, np.iinfo(dt).max)
        a = np.asfortranarray(v.astype(dt).reshape(shape, order="F"))
        src, dst = str(tmp_path / "s.mat"), str(tmp_path / "d.mat")
        scipy_io.savemat(src, {"v": a}, do_compression=compress)
        r = subprocess.run([harness, "--mat-copy", src, dst], capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stderr
        back = scipy_io.loadmat(dst)["v"]
        want = scipy_io.loadmat(src)["v"].astype(np.float64)
        assert back.shape == want.shape and np.array_equal(back.astype(np.float64), want)

    check()
