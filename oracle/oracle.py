"""ctypes front end of the CPU oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker.  Arrays follow the
reference's MATLAB layout: column-major (Fortran order), complex128 for
Fourier data.  Parity against the reference's own outputs is unpinned (the
reference ships no golden vectors); see the header of genfire_oracle.c.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


class OrcParams(C.Structure):
    """Mirror of ``orc_params`` (the GENFIRE_Reconstructor properties on the path)."""
    _fields_ = [
        ("Dim1", C.c_int), ("Dim2", C.c_int), ("NumProjs", C.c_int),
        ("oversamplingRatio", C.c_double),
        ("interpolationCutoffDistance", C.c_double),
        ("DFT_CentroSymmetricity", C.c_int),
        ("vector1", C.c_double * 3), ("vector2", C.c_double * 3), ("vector3", C.c_double * 3),
        ("numIterations", C.c_int),
        ("constraintEnforcementMode", C.c_int),
        ("constraintPositivity", C.c_int),
        ("constraintSupport", C.c_int),
        ("monitor_R", C.c_int),
        ("monitorR_loopLength", C.c_int),
    ]


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        dp, fp, ip, lp, up = (C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int),
                              C.POINTER(C.c_int64), C.POINTER(C.c_ubyte))
        L.orc_oversampled_size.restype = C.c_int
        L.orc_oversampled_size.argtypes = [C.c_int, C.c_double]
        L.orc_volumn_index.argtypes = [ip, ip, ip]
        L.orc_iffshift3_ind.argtypes = [ip, C.c_int64, lp, lp]
        L.orc_paddzero.argtypes = [dp, ip, ip, dp]
        L.orc_stripzero.argtypes = [dp, ip, ip, dp]
        L.orc_make_kspace_indices.argtypes = [ip, dp]
        L.orc_quat_rot.argtypes = [dp, C.c_double, dp]
        L.orc_euler_rot.argtypes = [dp, dp, dp, C.c_double, C.c_double, C.c_double, dp]
        L.orc_rot_zyz.argtypes = [C.c_double, C.c_double, C.c_double, dp]
        L.orc_proj_geometry.argtypes = [C.POINTER(OrcParams), C.c_double, C.c_double, C.c_double, fp, fp]
        L.orc_grid_extent.argtypes = [C.c_int, C.c_int, C.c_int, ip]
        L.orc_select.restype = C.c_int64
        L.orc_select.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, fp, fp, C.c_int64,
                                 lp, fp, fp, fp, lp]
        L.orc_dft.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64, fp, fp, dp]
        L.orc_centro.argtypes = [dp, C.c_int, C.c_int, C.c_int, dp]
        L.orc_hermitian_symmetrize.argtypes = [dp, C.c_int, C.c_int, C.c_int, dp]
        L.orc_fftn.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_grid_fs.restype = C.c_int64
        L.orc_grid_fs.argtypes = [C.POINTER(OrcParams), dp, dp, dp, lp]
        L.orc_grid_dft.restype = C.c_int64
        L.orc_grid_dft.argtypes = [C.POINTER(OrcParams), dp, dp, dp, dp, lp]
        L.orc_rec_ifft.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int, dp]
        L.orc_fft_grid_size.restype = C.c_int
        L.orc_fft_grid_size.argtypes = [C.c_int, C.c_double]
        L.orc_grid_fft.restype = C.c_int64
        L.orc_grid_fft.argtypes = [C.POINTER(OrcParams), C.c_int, dp, dp, dp, dp]
        L.orc_project_R.argtypes = [dp, C.c_int, C.c_int, C.c_int, dp, dp]
        L.orc_project.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, dp, dp]
        L.orc_rfactor.argtypes = [dp, dp, C.c_int64, dp, dp]
        L.orc_project_interp.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, dp,
                                         C.c_int, dp]
        L.orc_rfactor_realspace.restype = C.c_double
        L.orc_rfactor_realspace.argtypes = [dp, C.c_int, C.c_int, C.c_int, dp, C.c_int, C.c_int, C.c_int, dp,
                                            C.c_int, dp, dp]
        L.orc_delay_indicators.restype = C.c_int
        L.orc_delay_indicators.argtypes = [C.c_int, dp]
        L.orc_change_points.argtypes = [C.c_int, C.c_int, ip]
        L.orc_reconstruct.restype = C.c_int
        L.orc_reconstruct.argtypes = [C.POINTER(OrcParams), dp, up, up, dp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_reconstruct_rfree.restype = C.c_int
        L.orc_reconstruct_rfree.argtypes = [C.POINTER(OrcParams), dp, up, up, dp, dp, dp, dp, dp, dp, dp, dp,
                                            C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64), dp]
        L.orc_rfree_candidates.restype = C.c_int64
        L.orc_rfree_candidates.argtypes = [C.c_int, C.c_int, dp, C.c_int, C.c_int, C.POINTER(C.c_int64)]
        L.orc_num_threads.restype = C.c_int
        L.orc_last_loop_seconds.restype = C.c_double
        L.orc_last_loop_seconds_from.restype = C.c_double
        L.orc_last_loop_seconds_from.argtypes = [C.c_int]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def _f64(a):
    return np.asfortranarray(a, dtype=np.float64)


def _c128_view(a):
    """Fortran-ordered complex128 array viewed as interleaved doubles."""
    a = np.asfortranarray(a, dtype=np.complex128)
    return a, a.reshape(-1, order="F").view(np.float64)


def make_params(Dim1, Dim2, NumProjs, oversamplingRatio=3.0, interpolationCutoffDistance=0.7,
                DFT_CentroSymmetricity=1, vector1=(0, 0, 1), vector2=(0, 1, 0), vector3=(1, 0, 0),
                numIterations=50, constraintEnforcementMode=1, constraintPositivity=1,
                constraintSupport=1, monitor_R=0, monitorR_loopLength=10):
    p = OrcParams()
    p.Dim1, p.Dim2, p.NumProjs = Dim1, Dim2, NumProjs
    p.oversamplingRatio = oversamplingRatio
    p.interpolationCutoffDistance = interpolationCutoffDistance
    p.DFT_CentroSymmetricity = DFT_CentroSymmetricity
    for name, v in (("vector1", vector1), ("vector2", vector2), ("vector3", vector3)):
        getattr(p, name)[:] = [float(x) for x in v]
    p.numIterations = numIterations
    p.constraintEnforcementMode = constraintEnforcementMode
    p.constraintPositivity = constraintPositivity
    p.constraintSupport = constraintSupport
    p.monitor_R = monitor_R
    p.monitorR_loopLength = monitorR_loopLength
    return p


def oversampled(dim, ratio):
    return lib().orc_oversampled_size(dim, ratio)


def grid_extent(n1, n2, centro):
    out = np.zeros(6, dtype=np.int32)
    lib().orc_grid_extent(n1, n2, centro, _p(out, C.c_int))
    return out


def volumn_index(big, ori):
    b = np.asarray(big, dtype=np.int32); o = np.asarray(ori, dtype=np.int32)
    out = np.zeros(6, dtype=np.int32)
    lib().orc_volumn_index(_p(b, C.c_int), _p(o, C.c_int), _p(out, C.c_int))
    return out.reshape(3, 2, order="F")


def iffshift3_ind(size, inds):
    s = np.asarray(size, dtype=np.int32)
    i = np.ascontiguousarray(inds, dtype=np.int64)
    out = np.zeros_like(i)
    lib().orc_iffshift3_ind(_p(s, C.c_int), i.size, _p(i, C.c_int64), _p(out, C.c_int64))
    return out


def paddzero(vol, size):
    v = _f64(vol); vs = np.asarray(v.shape, dtype=np.int32); ps = np.asarray(size, dtype=np.int32)
    out = np.zeros(tuple(size), dtype=np.float64, order="F")
    lib().orc_paddzero(_p(v, C.c_double), _p(vs, C.c_int), _p(ps, C.c_int), _p(out, C.c_double))
    return out


def stripzero(pad, size):
    v = _f64(pad); ps = np.asarray(v.shape, dtype=np.int32); os_ = np.asarray(size, dtype=np.int32)
    out = np.zeros(tuple(size), dtype=np.float64, order="F")
    lib().orc_stripzero(_p(v, C.c_double), _p(ps, C.c_int), _p(os_, C.c_int), _p(out, C.c_double))
    return out


def make_kspace_indices(size):
    s = np.asarray(size, dtype=np.int32)
    Q = np.zeros(tuple(size), dtype=np.float64, order="F")
    lib().orc_make_kspace_indices(_p(s, C.c_int), _p(Q, C.c_double))
    return Q


def quat_rot(v, theta):
    v = np.asarray(v, dtype=np.float64); R = np.zeros(9)
    lib().orc_quat_rot(_p(v, C.c_double), theta, _p(R, C.c_double))
    return R.reshape(3, 3, order="F")


def euler_rot(v1, v2, v3, phi, theta, psi):
    a, b, c = (np.asarray(x, dtype=np.float64) for x in (v1, v2, v3))
    R = np.zeros(9)
    lib().orc_euler_rot(_p(a, C.c_double), _p(b, C.c_double), _p(c, C.c_double), phi, theta, psi,
                        _p(R, C.c_double))
    return R.reshape(3, 3, order="F")


def rot_zyz(phi, theta, psi):
    R = np.zeros(9)
    lib().orc_rot_zyz(phi, theta, psi, _p(R, C.c_double))
    return R.reshape(3, 3, order="F")


def proj_geometry(prm, phi, theta, psi):
    Rf = np.zeros(9, dtype=np.float32); nrm = np.zeros(3, dtype=np.float32)
    lib().orc_proj_geometry(C.byref(prm), phi, theta, psi, _p(Rf, C.c_float), _p(nrm, C.c_float))
    return Rf, nrm


def select(n1, n2, centro, cutoff, Rf, nrm, cap=None):
    """One projection's selected K-points: (ind0, dist, u, v, offplane); cap
    bounds the count (default: the whole gridded extent)."""
    if cap is None:
        ext = grid_extent(n1, n2, centro)
        cap = int(ext[3]) * int(ext[4]) * int(ext[5])
    ind = np.zeros(cap, dtype=np.int64)
    dist = np.zeros(cap, dtype=np.float32); u = np.zeros(cap, dtype=np.float32)
    v = np.zeros(cap, dtype=np.float32); off = np.zeros(1, dtype=np.int64)
    Rf = np.ascontiguousarray(Rf, dtype=np.float32); nrm = np.ascontiguousarray(nrm, dtype=np.float32)
    n = lib().orc_select(n1, n2, centro, cutoff, _p(Rf, C.c_float), _p(nrm, C.c_float), cap,
                         _p(ind, C.c_int64), _p(dist, C.c_float), _p(u, C.c_float), _p(v, C.c_float),
                         _p(off, C.c_int64))
    assert n >= 0
    return ind[:n].copy(), dist[:n].copy(), u[:n].copy(), v[:n].copy(), int(off[0])


def dft(proj, n1, n2, u, v):
    P = _f64(proj); D1, D2 = P.shape
    u = np.ascontiguousarray(u, dtype=np.float32); v = np.ascontiguousarray(v, dtype=np.float32)
    F = np.zeros(u.size, dtype=np.complex128)
    lib().orc_dft(_p(P, C.c_double), D1, D2, n1, n2, u.size, _p(u, C.c_float), _p(v, C.c_float),
                  _p(F.view(np.float64), C.c_double))
    return F


def centro(FS, n1, n_k1, n2):
    FSc, FSv = _c128_view(FS)
    M = np.zeros((n1, n2, n1), dtype=np.complex128, order="F")
    lib().orc_centro(_p(FSv, C.c_double), n1, n_k1, n2, _p(M.reshape(-1, order="F").view(np.float64), C.c_double))
    return M


def hermitian_symmetrize(a):
    ac, av = _c128_view(a)
    out = np.zeros(ac.shape, dtype=np.complex128, order="F")
    d = ac.shape
    lib().orc_hermitian_symmetrize(_p(av, C.c_double), d[0], d[1], d[2],
                                   _p(out.reshape(-1, order="F").view(np.float64), C.c_double))
    return out


def fftn(a, inverse=False):
    ac = np.array(a, dtype=np.complex128, order="F", copy=True)
    d = ac.shape + (1,) * (3 - ac.ndim)
    lib().orc_fftn(_p(ac.reshape(-1, order="F").view(np.float64), C.c_double), d[0], d[1], d[2],
                   1 if inverse else 0)
    return ac


def grid_fs(prm, projs, angles):
    """Weighted-average grid FS (before CentroSymmetricity) and per-projection counts."""
    P = _f64(projs); A = _f64(angles)
    n1 = oversampled(prm.Dim1, prm.oversamplingRatio); n2 = oversampled(prm.Dim2, prm.oversamplingRatio)
    ext = grid_extent(n1, n2, prm.DFT_CentroSymmetricity)
    FS = np.zeros(tuple(int(x) for x in ext[3:]), dtype=np.complex128, order="F")
    nk = np.zeros(prm.NumProjs, dtype=np.int64)
    lib().orc_grid_fs(C.byref(prm), _p(P, C.c_double), _p(A, C.c_double),
                      _p(FS.reshape(-1, order="F").view(np.float64), C.c_double), _p(nk, C.c_int64))
    return FS, nk


def grid_dft(prm, projs, angles, want_rec=True):
    """fillInFourierGrid_DFT: (measuredK centred complex128, recIFFT or None, nk per projection)."""
    P = _f64(projs); A = _f64(angles)
    n1 = oversampled(prm.Dim1, prm.oversamplingRatio); n2 = oversampled(prm.Dim2, prm.oversamplingRatio)
    M = np.zeros((n1, n2, n1), dtype=np.complex128, order="F")
    rec = np.zeros((prm.Dim1, prm.Dim2, prm.Dim1), dtype=np.float64, order="F") if want_rec else None
    nk = np.zeros(prm.NumProjs, dtype=np.int64)
    lib().orc_grid_dft(C.byref(prm), _p(P, C.c_double), _p(A, C.c_double),
                       _p(M.reshape(-1, order="F").view(np.float64), C.c_double),
                       _p(rec, C.c_double), _p(nk, C.c_int64))
    return M, rec, nk


def fft_grid_size(Dim2, ratio):
    """Cube size m of fillInFourierGrid (-1 when not an integer)."""
    return lib().orc_fft_grid_size(int(Dim2), float(ratio))


def grid_fft(prm, projs, angles, allow_multiple=1, want_rec=True):
    """fillInFourierGrid (griddingMethod 1): (measuredK m^3 centred complex128,
    recIFFT or None, number of gridded pairs)."""
    P = _f64(projs); A = _f64(angles)
    m = fft_grid_size(prm.Dim2, prm.oversamplingRatio)
    if m < 0:
        raise ValueError("fillInFourierGrid: Dim2 * oversamplingRatio is not an integer")
    M = np.zeros((m, m, m), dtype=np.complex128, order="F")
    rec = np.zeros((prm.Dim1, prm.Dim2, prm.Dim1), dtype=np.float64, order="F") if want_rec else None
    n = lib().orc_grid_fft(C.byref(prm), int(allow_multiple), _p(P, C.c_double), _p(A, C.c_double),
                           _p(M.reshape(-1, order="F").view(np.float64), C.c_double), _p(rec, C.c_double))
    if n < 0:
        raise ValueError("fillInFourierGrid: grid smaller than the projections")
    return M, rec, n


def rec_ifft(M, D1, D2):
    Mc, Mv = _c128_view(M)
    n1, n2, _ = Mc.shape
    rec = np.zeros((D1, D2, D1), dtype=np.float64, order="F")
    lib().orc_rec_ifft(_p(Mv, C.c_double), n1, n2, D1, D2, _p(rec, C.c_double))
    return rec


def project_interp(vol, phi, theta, psi, vectors=None, cubic=False):
    """Projector with trilinear (cubic=False) or Keys cubic-convolution (cubic=True) sampling."""
    V = _f64(vol); n1, n2, n3 = V.shape
    out = np.zeros((n1, n2), dtype=np.float64, order="F")
    vec = None
    if vectors is not None:
        vec = np.ascontiguousarray(np.asarray(vectors, dtype=np.float64).reshape(9))
    lib().orc_project_interp(_p(V, C.c_double), n1, n2, n3, phi, theta, psi, _p(vec, C.c_double), int(cubic),
                             _p(out, C.c_double))
    return out


def rfactor_realspace(model, projs, angles, cubic=False):
    """Tian_calc_Rfactor_realspace: (Rtotal, Rarr, simuProjs)."""
    V = _f64(model); m1, m2, m3 = V.shape
    Pj = _f64(projs); p1, p2, P = Pj.shape
    A = _f64(np.atleast_2d(angles))
    R = np.zeros(P)
    simu = np.zeros((p1, p2, P), dtype=np.float64, order="F")
    tot = lib().orc_rfactor_realspace(_p(V, C.c_double), m1, m2, m3, _p(Pj, C.c_double), p1, p2, P,
                                      _p(A, C.c_double), int(cubic), _p(R, C.c_double), _p(simu, C.c_double))
    return tot, R, simu


def project(vol, phi, theta, psi, vectors=None):
    V = _f64(vol); n1, n2, n3 = V.shape
    out = np.zeros((n1, n2), dtype=np.float64, order="F")
    vec = None
    if vectors is not None:
        vec = np.ascontiguousarray(np.asarray(vectors, dtype=np.float64).reshape(9))
    lib().orc_project(_p(V, C.c_double), n1, n2, n3, phi, theta, psi, _p(vec, C.c_double),
                      _p(out, C.c_double))
    return out


def rfactor(bp, pj):
    a = np.ascontiguousarray(bp, dtype=np.float64).reshape(-1)
    b = np.ascontiguousarray(pj, dtype=np.float64).reshape(-1)
    r1 = C.c_double(); r2 = C.c_double()
    lib().orc_rfactor(_p(a, C.c_double), _p(b, C.c_double), a.size, C.byref(r1), C.byref(r2))
    return r1.value, r2.value


def delay_indicators(mode):
    out = np.zeros(64)
    m = lib().orc_delay_indicators(mode, _p(out, C.c_double))
    return out[:m].copy()


def change_points(N, m):
    out = np.zeros(m, dtype=np.int32)
    lib().orc_change_points(N, m, _p(out, C.c_int))
    return out


def rfree_candidates(measuredK, nbins, shell):
    """Candidate points of Rfree shell `shell` (0-based) of `nbins`
    (reconstruct.m:47-50): ascending 0-based linear indices (int64)."""
    Mc, Mv = _c128_view(measuredK)
    n1, n2 = Mc.shape[0], Mc.shape[1]
    cnt = lib().orc_rfree_candidates(n1, n2, _p(Mv, C.c_double), nbins, shell, None)
    out = np.zeros(max(cnt, 1), dtype=np.int64)
    lib().orc_rfree_candidates(n1, n2, _p(Mv, C.c_double), nbins, shell, _p(out, C.c_int64))
    return out[:cnt]


def reconstruct_rfree(prm, measuredK, shells, support=None, initial=None, mask=None):
    """reconstruct.m with the Rfree monitor (:137-146) for the withheld sets
    `shells` (a list of int64 arrays of 0-based centred linear indices, already
    removed from `mask`).  Returns (reconstruction, errK, Rfree) with Rfree of
    shape (len(shells), numIterations)."""
    Mc, Mv = _c128_view(measuredK)
    D1, D2 = prm.Dim1, prm.Dim2
    sup = None if support is None else np.asfortranarray(support, dtype=np.uint8)
    msk = None if mask is None else np.asfortranarray(mask, dtype=np.uint8)
    ini = None if initial is None else _f64(initial)
    N = prm.numIterations
    counts = np.array([len(s) for s in shells], dtype=np.int64)
    ind = np.ascontiguousarray(np.concatenate([np.asarray(s, dtype=np.int64) for s in shells])
                               if len(shells) else np.zeros(1, dtype=np.int64))
    rec = np.zeros((D1, D2, D1), dtype=np.float64, order="F")
    errK = np.zeros(N)
    rfree = np.zeros((len(shells), max(N, 1)), order="F")
    rc = lib().orc_reconstruct_rfree(C.byref(prm), _p(Mv, C.c_double), _p(msk, C.c_ubyte), _p(sup, C.c_ubyte),
                                     _p(ini, C.c_double), None, None, _p(rec, C.c_double), _p(errK, C.c_double),
                                     None, None, None, len(shells), _p(counts, C.c_int64), _p(ind, C.c_int64),
                                     _p(rfree, C.c_double))
    if rc != 0:
        raise ValueError("oracle reconstruct failed (%d)" % rc)
    return rec, errK, rfree[:, :N]


def reconstruct(prm, measuredK, support=None, initial=None, mask=None, projs=None, angles=None):
    """reconstruct.m end to end.  Returns (reconstruction, errK, errR, Rarr, Rarr2)."""
    Mc, Mv = _c128_view(measuredK)
    D1, D2 = prm.Dim1, prm.Dim2
    sup = None if support is None else np.asfortranarray(support, dtype=np.uint8)
    msk = None if mask is None else np.asfortranarray(mask, dtype=np.uint8)
    ini = None if initial is None else _f64(initial)
    P = None if projs is None else _f64(projs)
    A = None if angles is None else _f64(angles)
    N = prm.numIterations
    nmon = N // prm.monitorR_loopLength if (prm.monitor_R == 1 and prm.monitorR_loopLength > 0) else 0
    rec = np.zeros((D1, D2, D1), dtype=np.float64, order="F")
    errK = np.zeros(N)
    errR = np.zeros(max(nmon, 1)); Rarr = np.zeros((prm.NumProjs, max(nmon, 1)), order="F")
    Rarr2 = np.zeros((prm.NumProjs, max(nmon, 1)), order="F")
    rc = lib().orc_reconstruct(C.byref(prm), _p(Mv, C.c_double), _p(msk, C.c_ubyte), _p(sup, C.c_ubyte),
                               _p(ini, C.c_double), _p(P, C.c_double), _p(A, C.c_double),
                               _p(rec, C.c_double), _p(errK, C.c_double), _p(errR, C.c_double),
                               _p(Rarr, C.c_double), _p(Rarr2, C.c_double))
    if rc != 0:
        raise ValueError("oracle reconstruct failed (%d)" % rc)
    return rec, errK, errR[:nmon], Rarr[:, :nmon], Rarr2[:, :nmon]


def num_threads():
    return lib().orc_num_threads()


def last_loop_seconds():
    """Wall time of the iteration loop of the last reconstruct() call."""
    return lib().orc_last_loop_seconds()


def last_loop_seconds_from(first):
    """Wall time of the iterations after the first `first` (a warm-up) of the
    last reconstruct() call; 0 when `first` is not below its iteration count."""
    return lib().orc_last_loop_seconds_from(int(first))


__all__ = [n for n in dir() if not n.startswith("_")]
