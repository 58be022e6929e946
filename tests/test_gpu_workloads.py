"""The benchmark's synthetic workloads at their full sizes (genfire_gb300.synth).

* tilt64 (64^3 object, 31 single-axis tilts -75:5:75, 128^3 grid, 200
  iterations): FP64 on the GPU against the oracle end to end -- gridded
  values, recIFFT, reconstruction and errK within relative L2 1e-10, equal
  per-projection point counts -- and the mixed path against FP64 (gridding
  within 1e-4, R-factor within 0.001).
* euler128 (128^3 object, 60 random Euler triples, 256^3 grid, 500
  iterations): the FP64 GPU gridding of a subset of projections against the
  oracle, then mixed against FP64 over the whole series and loop.
* euler256 (the headline: 256^3 object, 90 projections with 0.3 degree angle
  jitter, 512^3 grid, 1000 iterations): selection of all 90 projections
  bit-exact against the oracle, the FP64 gridding of 6 projections within
  1e-10 of the oracle at the full grid, mixed gridding of the whole series
  within 1e-4 of FP64, and mixed and FP64 reaching the same final R-factor
  within 0.001 (and errK within 0.1 %) after the configuration's 1000
  iterations.
* euler512 (512^3 object, 120 projections, 1024^3 grid, 300 iterations, the
  largest workload): selection bit-exact against the oracle on two
  projections, mixed gridding within 1e-4 of FP64, the mixed loop keeps
  positivity and support and lowers errK, and mixed and FP64 reach the same
  final R-factor within 0.001 after the configuration's 300 iterations.
  Everything stays in device memory (the FP64 grid alone is 17 GB).
"""
import numpy as np
import pytest

from genfire_gb300 import synth
from tests.conftest import params, rel

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_GRID_TOL = 1e-4
RFACTOR_TOL = 1e-3
CUTOFF = 0.125


def _workload(ctx, name):
    def proj(vol, angles, vectors):
        return ctx.project(vol.astype(np.float64), angles, vectors=np.asarray(vectors, float).reshape(-1))
    return synth.make_workload(name, proj)


def _params(lib, w, iters, precision, P=None):
    D = w["D"]
    v1, v2, v3 = w["vectors"]
    return params(lib, D, D, P if P is not None else w["projections"].shape[2], oversamplingRatio=w["os"],
                  interpolationCutoffDistance=CUTOFF, vector1=v1, vector2=v2, vector3=v3, numIterations=iters,
                  constraintEnforcementMode=3, constraintPositivity=1, constraintSupport=1, precision=precision)


def _oparams(oracle, w, iters, P=None):
    D = w["D"]
    v1, v2, v3 = w["vectors"]
    return oracle.make_params(D, D, P if P is not None else w["projections"].shape[2], oversamplingRatio=w["os"],
                              interpolationCutoffDistance=CUTOFF, vector1=v1, vector2=v2, vector3=v3,
                              numIterations=iters, constraintEnforcementMode=3, constraintPositivity=1,
                              constraintSupport=1)


def test_tilt64_fp64_against_oracle(lib, ctx, oracle):
    w = _workload(ctx, "tilt64")
    N = w["iters"]
    projs, ang = w["projections"], w["angles_in"]
    assert projs.shape == (64, 64, 31)
    p = _params(lib, w, N, "fp64")
    op = _oparams(oracle, w, N)
    M, rec0, nk = ctx.grid_dft(p, projs, ang)
    Mo, rec0o, nko = oracle.grid_dft(op, projs, ang)
    assert np.array_equal(nk, nko)
    assert rel(M, Mo) < FP64_TOL
    assert rel(rec0, rec0o) < FP64_TOL
    rec, errK, _, _, _ = ctx.reconstruct(p, M, support=w["support"])
    reco, errKo, _, _, _ = oracle.reconstruct(op, Mo, support=w["support"])
    assert errK.shape == (N,)
    assert rel(rec, reco) < FP64_TOL
    assert np.abs(errK - errKo).max() < FP64_TOL * np.abs(errKo).max()
    R, _, _ = ctx.rfactor(rec, ang, projs, vectors=np.asarray(w["vectors"], float).reshape(-1))
    Ro, _, _ = ctx.rfactor(reco, ang, projs, vectors=np.asarray(w["vectors"], float).reshape(-1))
    assert abs(R - Ro) < 1e-10
    # mixed: gridding and the equal-iteration R-factor
    pm = _params(lib, w, N, "mixed")
    M32, _, nk32 = ctx.grid_dft(pm, projs, ang, want_rec=False)
    assert np.array_equal(nk32, nk)
    assert rel(M32, M) < MIXED_GRID_TOL
    rec32, errK32, _, _, _ = ctx.reconstruct(pm, M32, support=w["support"])
    R32, _, _ = ctx.rfactor(rec32.astype(np.float64), ang, projs, vectors=np.asarray(w["vectors"], float).reshape(-1))
    assert abs(R32 - R) < RFACTOR_TOL
    assert rel(rec32, rec) < 1e-3
    # the loop moves towards the ground truth (single-axis tilt: a 30-degree missing wedge remains)
    assert rel(rec, w["vol"]) < 0.6


def test_euler128_mixed_against_fp64(lib, ctx, oracle):
    w = _workload(ctx, "euler128")
    N = w["iters"]
    projs, ang = w["projections"], w["angles_in"]
    assert projs.shape == (128, 128, 60)
    # the FP64 gridding of 6 projections against the oracle at the full grid size
    sub = [0, 11, 23, 35, 47, 59]
    ps = _params(lib, w, 1, "fp64", P=len(sub))
    Ms, rs, nks = ctx.grid_dft(ps, projs[:, :, sub], ang[sub])
    Mso, rso, nkso = oracle.grid_dft(_oparams(oracle, w, 1, P=len(sub)), projs[:, :, sub], ang[sub])
    assert np.array_equal(nks, nkso)
    assert rel(Ms, Mso) < FP64_TOL
    assert rel(rs, rso) < FP64_TOL
    # the whole series and loop, mixed against FP64
    p64, p32 = _params(lib, w, N, "fp64"), _params(lib, w, N, "mixed")
    M64, _, nk64 = ctx.grid_dft(p64, projs, ang, want_rec=False)
    M32, _, nk32 = ctx.grid_dft(p32, projs, ang, want_rec=False)
    assert np.array_equal(nk32, nk64)
    assert rel(M32, M64) < MIXED_GRID_TOL
    vec = np.asarray(w["vectors"], float).reshape(-1)
    rec64, errK64, _, _, _ = ctx.reconstruct(p64, M64, support=w["support"])
    rec32, errK32, _, _, _ = ctx.reconstruct(p32, M32, support=w["support"])
    R64, _, _ = ctx.rfactor(rec64, ang, projs, vectors=vec)
    R32, _, _ = ctx.rfactor(rec32.astype(np.float64), ang, projs, vectors=vec)
    assert abs(R32 - R64) < RFACTOR_TOL
    assert abs(errK32[-1] - errK64[-1]) < 1e-3 * errK64[-1]
    assert errK64[-1] < errK64[0]


def test_euler256_headline_full_length(lib, ctx, oracle):
    torch = pytest.importorskip("torch")
    w = _workload(ctx, "euler256")
    projs, ang = w["projections"], w["angles_in"]
    D, P, N = w["D"], projs.shape[2], w["iters"]
    assert (D, P, N) == (256, 90, 1000)
    p32, p64 = _params(lib, w, N, "mixed"), _params(lib, w, N, "fp64")
    n1, n2 = lib.grid_size(p32)
    assert (n1, n2) == (512, 512)
    # selection of every projection, bit-exact against the oracle (index, D, u, v)
    op1 = _oparams(oracle, w, 1, P=1)
    ps1 = _params(lib, w, 1, "fp64", P=1)
    for i in range(P):
        g = ctx.select(ps1, *ang[i], cap=4 * n1 * n2)
        Rf, nrm = oracle.proj_geometry(op1, *ang[i])
        o = oracle.select(n1, n2, 1, CUTOFF, Rf, nrm, cap=4 * n1 * n2)
        assert len(g[0]) > n1 * n2 // 16
        for a, b in zip(g, o[:4]):
            assert np.array_equal(a, b), i
    # the FP64 gridding (and recIFFT) of 6 spread projections against the oracle at the full grid
    sub = [0, 17, 35, 53, 71, 89]
    Ms, rs, nks = ctx.grid_dft(_params(lib, w, 1, "fp64", P=len(sub)), projs[:, :, sub], ang[sub])
    Mso, rso, nkso = oracle.grid_dft(_oparams(oracle, w, 1, P=len(sub)), projs[:, :, sub], ang[sub])
    assert np.array_equal(nks, nkso)
    assert rel(Ms, Mso) < FP64_TOL
    assert rel(rs, rso) < FP64_TOL
    del Ms, rs, Mso, rso
    # the whole series on the device: mixed gridding against FP64
    dev = torch.device("cuda")
    d_proj = torch.from_numpy(np.ascontiguousarray(projs.reshape(-1, order="F"))).to(dev)
    d_sup = torch.from_numpy(np.ascontiguousarray(w["support"].reshape(-1, order="F").astype(np.uint8))).to(dev)
    N3 = n1 * n2 * n1
    d_M32 = torch.empty(N3, dtype=torch.complex64, device=dev)
    d_M64 = torch.empty(N3, dtype=torch.complex128, device=dev)
    nk32 = ctx.grid_dft_device(p32, d_proj.data_ptr(), ang, d_M32.data_ptr())
    nk64 = ctx.grid_dft_device(p64, d_proj.data_ptr(), ang, d_M64.data_ptr())
    assert np.array_equal(nk32, nk64) and nk32.min() > 0
    err = float(torch.linalg.vector_norm(d_M32.to(torch.complex128) - d_M64) / torch.linalg.vector_norm(d_M64))
    assert err < MIXED_GRID_TOL
    # the configuration's 1000 iterations in both precisions: the same final R-factor
    vec = np.asarray(w["vectors"], float).reshape(-1)
    out = {}
    for name, p, dM in (("mixed", p32, d_M32), ("fp64", p64, d_M64)):
        r = ctx.recon(p, dM.data_ptr(), support=d_sup.data_ptr(), on_device=True)
        r.iterate(N)
        rec, errK, _, _, _ = r.result()
        r.close()
        assert errK.shape == (N,) and np.all(np.isfinite(errK))
        R, _, _ = ctx.rfactor(rec.astype(np.float64), ang, projs, vectors=vec)
        out[name] = (R, errK, rec)
    (R32, e32, rec32), (R64, e64, rec64) = out["mixed"], out["fp64"]
    assert abs(R32 - R64) < RFACTOR_TOL
    assert abs(e32[-1] - e64[-1]) < 1e-3 * e64[-1]
    assert e64[-1] < e64[0]
    assert rec32.min() >= 0.0 and not np.any(rec32[~w["support"]])
    assert rel(rec32, rec64) < 1e-3


def test_euler512_largest_workload(lib, ctx, oracle):
    torch = pytest.importorskip("torch")
    w = _workload(ctx, "euler512")
    projs, ang = w["projections"], w["angles_in"]
    D, P = w["D"], projs.shape[2]
    assert (D, P) == (512, 120)
    p32 = _params(lib, w, w["iters"], "mixed")
    p64 = _params(lib, w, w["iters"], "fp64")
    n1, n2 = lib.grid_size(p32)
    assert (n1, n2) == (1024, 1024)
    # selection of two projections, bit-exact against the oracle at the full grid size
    # (a slab of half-width 0.125 through the cube holds far fewer than 4 n1 n2 points)
    op = _oparams(oracle, w, 1, P=1)
    for i in (0, 77):
        g = ctx.select(_params(lib, w, 1, "fp64", P=1), *ang[i], cap=4 * n1 * n2)
        Rf, nrm = oracle.proj_geometry(op, *ang[i])
        o = oracle.select(n1, n2, 1, CUTOFF, Rf, nrm, cap=4 * n1 * n2)
        assert len(g[0]) > n1 * n2 // 16
        for a, b in zip(g, o[:4]):
            assert np.array_equal(a, b)
    dev = torch.device("cuda")
    d_proj = torch.from_numpy(np.ascontiguousarray(projs.reshape(-1, order="F"))).to(dev)
    d_sup = torch.from_numpy(np.ascontiguousarray(w["support"].reshape(-1, order="F").astype(np.uint8))).to(dev)
    N3 = n1 * n2 * n1
    d_M32 = torch.empty(N3, dtype=torch.complex64, device=dev)
    d_M64 = torch.empty(N3, dtype=torch.complex128, device=dev)
    nk32 = ctx.grid_dft_device(p32, d_proj.data_ptr(), ang, d_M32.data_ptr())
    nk64 = ctx.grid_dft_device(p64, d_proj.data_ptr(), ang, d_M64.data_ptr())
    assert np.array_equal(nk32, nk64) and nk32.min() > 0
    err = float(torch.linalg.vector_norm(d_M32.to(torch.complex128) - d_M64) / torch.linalg.vector_norm(d_M64))
    assert err < MIXED_GRID_TOL
    vec = np.asarray(w["vectors"], float).reshape(-1)
    sup = w["support"]
    # the workload's 300 mixed iterations
    r = ctx.recon(p32, d_M32.data_ptr(), support=d_sup.data_ptr(), on_device=True)
    r.iterate(20)
    rec20, errK20, _, _, _ = r.result()
    r.iterate(w["iters"] - 20)
    rec, errK, _, _, _ = r.result()
    r.close()
    assert errK.shape == (w["iters"],) and np.all(np.isfinite(errK))
    assert errK[-1] < errK[0]
    assert rec.min() >= 0.0
    assert not np.any(rec[~sup])
    R300, _, _ = ctx.rfactor(rec.astype(np.float64), ang, projs, vectors=vec)
    # mixed and FP64 after 20 iterations and after the configuration's 300
    r64 = ctx.recon(p64, d_M64.data_ptr(), support=d_sup.data_ptr(), on_device=True)
    r64.iterate(20)
    rec64_20, errK64_20, _, _, _ = r64.result()
    r64.iterate(w["iters"] - 20)
    rec64, errK64, _, _, _ = r64.result()
    r64.close()
    R20, _, _ = ctx.rfactor(rec20.astype(np.float64), ang, projs, vectors=vec)
    R64_20, _, _ = ctx.rfactor(rec64_20, ang, projs, vectors=vec)
    assert abs(R20 - R64_20) < RFACTOR_TOL
    assert abs(errK20[-1] - errK64_20[-1]) < 1e-3 * errK64_20[-1]
    R64, _, _ = ctx.rfactor(rec64, ang, projs, vectors=vec)
    assert abs(R300 - R64) < RFACTOR_TOL
    assert abs(errK[-1] - errK64[-1]) < 1e-3 * errK64[-1]
    assert 0.0 < R300 < 0.8
