"""ctypes binding of libgenfire.so (the C ABI declared in include/genfire.h).

The library is built in-tree (``genfire_gb300/_build/libgenfire.so``); if it
is missing the loader raises instead of falling back to anything else.
Arrays are passed in MATLAB layout: Fortran-ordered numpy arrays, complex
data interleaved.
"""
import ctypes as C
import weakref
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgenfire.so")

GENFIRE_OK = 0
GENFIRE_ERR_ARG = 1
GENFIRE_ERR_OOM = 2
GENFIRE_ERR_CUDA = 3
GENFIRE_ERR_TIMEOUT = 4
GENFIRE_ERR_UNSUPPORTED = 5
GENFIRE_ERR_STATE = 6

PREC_FP64 = 0
PREC_MIXED = 1
PREC_FP16_SCALED = 2

PROFILE_KERNELS = 5   # GENFIRE_PROFILE_KERNELS: kernels of one iteration

INTERP_TRILINEAR = 0
INTERP_CUBIC = 1

# every entry point of include/genfire.h
EXPORTS = [
    "genfire_abi_version", "genfire_status_string", "genfire_params_init", "genfire_grid_size",
    "genfire_create", "genfire_destroy", "genfire_last_error", "genfire_stream",
    "genfire_grid_dft", "genfire_grid_dft_device", "genfire_grid_fft", "genfire_grid_fft_device",
    "genfire_grid_profile",
    "genfire_reconstruct", "genfire_recon_create", "genfire_recon_iterate", "genfire_recon_result",
    "genfire_recon_destroy", "genfire_recon_profile", "genfire_profile_kernel_name",
    "genfire_recon_batch_create", "genfire_recon_batch_iterate", "genfire_recon_batch_destroy",
    "genfire_recon_tuning", "genfire_rfree_candidates", "genfire_recon_set_rfree", "genfire_recon_rfree",
    "genfire_project", "genfire_rfactor", "genfire_rfactor_noalloc", "genfire_set_projector_interpolation",
    "genfire_rfactor_realspace",
    "genfire_centro_symmetricity", "genfire_hermitian_symmetrize", "genfire_make_kspace_indices",
    "genfire_volumn_index", "genfire_iffshift3_ind", "genfire_select", "genfire_fftn",
]


class GenfireError(RuntimeError):
    """Error raised for a non-zero genfire_status; the message is the library's."""

    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


class Params(C.Structure):
    """Mirror of ``genfire_params``."""
    _fields_ = [
        ("Dim1", C.c_int32), ("Dim2", C.c_int32), ("NumProjs", C.c_int32),
        ("DFT_CentroSymmetricity", C.c_int32),
        ("oversamplingRatio", C.c_double), ("interpolationCutoffDistance", C.c_double),
        ("vector1", C.c_double * 3), ("vector2", C.c_double * 3), ("vector3", C.c_double * 3),
        ("numIterations", C.c_int32), ("constraintEnforcementMode", C.c_int32),
        ("constraintPositivity", C.c_int32), ("constraintSupport", C.c_int32),
        ("monitor_R", C.c_int32), ("monitorR_loopLength", C.c_int32),
        ("precision", C.c_int32), ("griddingMethod", C.c_int32), ("allowMultipleGridMatches", C.c_int32),
        ("reserved", C.c_int32 * 7),
    ]


_lib = None


def load():
    """Load libgenfire.so (built by genfire_gb300.build); raise if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libgenfire.so is not built (%s); run genfire_gb300.build.build() first" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, dp, fp, up, i64p, i32p = (C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_float),
                                  C.POINTER(C.c_uint8), C.POINTER(C.c_int64), C.POINTER(C.c_int32))
    pp = C.POINTER(Params)
    sig = {
        "genfire_abi_version": (C.c_int32, []),
        "genfire_status_string": (C.c_char_p, [C.c_int]),
        "genfire_params_init": (C.c_int, [pp]),
        "genfire_grid_size": (C.c_int, [pp, i32p, i32p]),
        "genfire_create": (C.c_int, [C.c_int32, C.POINTER(C.c_void_p)]),
        "genfire_destroy": (C.c_int, [vp]),
        "genfire_last_error": (C.c_char_p, [vp]),
        "genfire_stream": (C.c_void_p, [vp]),
        "genfire_grid_dft": (C.c_int, [vp, pp, dp, dp, vp, vp, i64p]),
        "genfire_grid_dft_device": (C.c_int, [vp, pp, vp, dp, vp, vp, i64p]),
        "genfire_grid_fft": (C.c_int, [vp, pp, dp, dp, vp, vp, i64p]),
        "genfire_grid_profile": (C.c_int, [vp, pp, vp, dp, vp, dp]),
        "genfire_grid_fft_device": (C.c_int, [vp, pp, vp, dp, vp, vp, i64p]),
        "genfire_reconstruct": (C.c_int, [vp, pp, vp, up, up, vp, dp, dp, vp, dp, dp, dp, dp]),
        "genfire_recon_create": (C.c_int, [vp, pp, vp, vp, vp, vp, vp, vp, C.c_int32, C.POINTER(C.c_void_p)]),
        "genfire_recon_iterate": (C.c_int, [vp, C.c_int32]),
        "genfire_recon_result": (C.c_int, [vp, vp, vp, dp, dp, dp, C.c_int32]),
        "genfire_recon_destroy": (C.c_int, [vp]),
        "genfire_recon_batch_create": (C.c_int, [vp, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
        "genfire_recon_batch_iterate": (C.c_int, [vp, C.c_int32]),
        "genfire_recon_tuning": (C.c_int, [vp, i32p]),
        "genfire_rfree_candidates": (C.c_int, [vp, pp, vp, C.c_int32, C.c_int32, i64p, i64p]),
        "genfire_recon_set_rfree": (C.c_int, [vp, C.c_int32, i64p, i64p]),
        "genfire_recon_rfree": (C.c_int, [vp, i32p, dp]),
        "genfire_recon_batch_destroy": (C.c_int, [vp]),
        "genfire_recon_profile": (C.c_int, [vp, C.c_int32, dp, dp]),
        "genfire_profile_kernel_name": (C.c_char_p, [C.c_int32]),
        "genfire_project": (C.c_int, [vp, C.c_int32, vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, dp, dp, vp]),
        "genfire_rfactor": (C.c_int, [vp, C.c_int32, vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, dp, dp, dp,
                                      dp, dp, dp]),
        "genfire_rfactor_noalloc": (C.c_int, [vp, C.c_int32, vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, dp,
                                              dp, vp, dp, dp, dp]),
        "genfire_set_projector_interpolation": (C.c_int, [vp, C.c_int32]),
        "genfire_rfactor_realspace": (C.c_int, [vp, C.c_int32, vp, C.c_int32, C.c_int32, C.c_int32, dp, C.c_int32,
                                                C.c_int32, C.c_int32, dp, dp, dp, fp]),
        "genfire_centro_symmetricity": (C.c_int, [vp, dp, C.c_int32, C.c_int32, C.c_int32, dp]),
        "genfire_hermitian_symmetrize": (C.c_int, [vp, dp, C.c_int32, C.c_int32, C.c_int32, dp]),
        "genfire_make_kspace_indices": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int32, dp]),
        "genfire_volumn_index": (C.c_int, [i32p, i32p, i32p]),
        "genfire_iffshift3_ind": (C.c_int, [vp, i32p, C.c_int64, i64p, i64p]),
        "genfire_select": (C.c_int, [vp, pp, C.c_double, C.c_double, C.c_double, C.c_int64, i64p, fp, fp, fp,
                                     i64p]),
        "genfire_fftn": (C.c_int, [vp, C.c_int32, vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return _lib


def default_params():
    p = Params()
    load().genfire_params_init(C.byref(p))
    return p


def ptr(a, t=None):
    """Data pointer of a numpy array (or None)."""
    if a is None:
        return None
    if t is None:
        return C.c_void_p(a.ctypes.data)
    return a.ctypes.data_as(C.POINTER(t))


def fortran(a, dtype):
    return np.asfortranarray(a, dtype=dtype)


class Context:
    """A genfire_ctx: one device, one stream.  Methods mirror the C entry points."""

    def __init__(self, device=0):
        L = load()
        h = C.c_void_p()
        st = L.genfire_create(device, C.byref(h))
        if st != GENFIRE_OK:
            msg = L.genfire_last_error(None)
            raise GenfireError(st, (msg or b"").decode() or "GENFIRE: could not create a context")
        self._h = h
        self.device = device
        self._children = weakref.WeakSet()  # live Recon / ReconBatch objects of this context

    @property
    def handle(self):
        return self._h

    def _adopt(self, child):
        self._children.add(child)

    def close(self):
        if getattr(self, "_h", None):
            # batches before their members, then the reconstructions, then the context
            kids = list(getattr(self, "_children", []))
            for k in [k for k in kids if isinstance(k, ReconBatch)] + [k for k in kids if not isinstance(k, ReconBatch)]:
                k.close()
            load().genfire_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def check(self, st):
        if st != GENFIRE_OK:
            msg = load().genfire_last_error(self._h)
            raise GenfireError(st, (msg or b"").decode() or "GENFIRE: error %d" % st)

    @property
    def stream(self):
        return load().genfire_stream(self._h)

    # ---------------------------------------------------------------- gridding
    def grid_dft(self, p, projections, angles, want_rec=True):
        L = load()
        prec = p.precision
        cdt = np.complex128 if prec == PREC_FP64 else np.complex64
        rdt = np.float64 if prec == PREC_FP64 else np.float32
        n1, n2 = grid_size(p, method=2)
        P = fortran(projections, np.float64)
        A = fortran(angles, np.float64)
        M = np.zeros((n1, n2, n1), dtype=cdt, order="F")
        rec = np.zeros((p.Dim1, p.Dim2, p.Dim1), dtype=rdt, order="F") if want_rec else None
        nk = np.zeros(p.NumProjs, dtype=np.int64)
        self.check(L.genfire_grid_dft(self._h, C.byref(p), ptr(P, C.c_double), ptr(A, C.c_double), ptr(M),
                                      ptr(rec), ptr(nk, C.c_int64)))
        return M, rec, nk

    def grid_dft_device(self, p, d_proj_ptr, angles, d_M_ptr, d_rec_ptr=None):
        A = fortran(angles, np.float64)
        nk = np.zeros(p.NumProjs, dtype=np.int64)
        self.check(load().genfire_grid_dft_device(self._h, C.byref(p), C.c_void_p(d_proj_ptr), ptr(A, C.c_double),
                                                  C.c_void_p(d_M_ptr),
                                                  C.c_void_p(d_rec_ptr) if d_rec_ptr else None,
                                                  ptr(nk, C.c_int64)))
        return nk

    def grid_profile(self, p, d_proj_ptr, angles, d_M_ptr):
        """Device ms of the gridding stages: selection, DFT stage, DFT kernel, sums (sort, weighted sums,
        average, centro mirror, cast, written into measuredK), zero_fill (measuredK's zero pattern),
        recIFFT."""
        A = fortran(angles, np.float64)
        ms = np.zeros(6)
        self.check(load().genfire_grid_profile(self._h, C.byref(p), C.c_void_p(d_proj_ptr), ptr(A, C.c_double),
                                               C.c_void_p(d_M_ptr), ptr(ms, C.c_double)))
        return dict(zip(("selection", "dft_stage", "dft_kernel", "sums", "zero_fill", "rec_ifft"), ms.tolist()))

    def grid_fft(self, p, projections, angles, want_rec=True):
        """fillInFourierGrid (griddingMethod 1): (measuredK m^3, recIFFT or None, gridded pairs)."""
        L = load()
        prec = p.precision
        cdt = np.complex128 if prec == PREC_FP64 else np.complex64
        rdt = np.float64 if prec == PREC_FP64 else np.float32
        m, _ = grid_size(p, method=1)
        P = fortran(projections, np.float64)
        A = fortran(angles, np.float64)
        M = np.zeros((m, m, m), dtype=cdt, order="F")
        rec = np.zeros((p.Dim1, p.Dim2, p.Dim1), dtype=rdt, order="F") if want_rec else None
        n = C.c_int64()
        self.check(L.genfire_grid_fft(self._h, C.byref(p), ptr(P, C.c_double), ptr(A, C.c_double), ptr(M),
                                      ptr(rec), C.byref(n)))
        return M, rec, n.value

    def grid_fft_device(self, p, d_proj_ptr, angles, d_M_ptr, d_rec_ptr=None):
        A = fortran(angles, np.float64)
        n = C.c_int64()
        self.check(load().genfire_grid_fft_device(self._h, C.byref(p), C.c_void_p(d_proj_ptr), ptr(A, C.c_double),
                                                  C.c_void_p(d_M_ptr),
                                                  C.c_void_p(d_rec_ptr) if d_rec_ptr else None, C.byref(n)))
        return n.value

    def select(self, p, phi, theta, psi, cap=None):
        """One projection's selected points (ind, dist, u, v).  cap bounds the
        count (default: the whole gridded extent); more points are an error."""
        n1, n2 = grid_size(p, method=2)
        if cap is not None:
            cap = int(cap)
        elif p.DFT_CentroSymmetricity:
            cap = (n1 // 2 + 1) * (2 * (n2 // 2) + 1) * (2 * (n1 // 2) + 1)
        else:
            cap = n1 * n2 * n1
        ind = np.zeros(cap, dtype=np.int64)
        dist = np.zeros(cap, dtype=np.float32)
        u = np.zeros(cap, dtype=np.float32)
        v = np.zeros(cap, dtype=np.float32)
        cnt = C.c_int64()
        self.check(load().genfire_select(self._h, C.byref(p), phi, theta, psi, cap, ptr(ind, C.c_int64),
                                         ptr(dist, C.c_float), ptr(u, C.c_float), ptr(v, C.c_float),
                                         C.byref(cnt)))
        n = cnt.value
        return ind[:n].copy(), dist[:n].copy(), u[:n].copy(), v[:n].copy()

    # ---------------------------------------------------------------- iteration
    def reconstruct(self, p, measuredK, support=None, initial=None, mask=None, projections=None, angles=None):
        L = load()
        prec = p.precision
        cdt = np.complex128 if prec == PREC_FP64 else np.complex64
        rdt = np.float64 if prec == PREC_FP64 else np.float32
        M = fortran(measuredK, cdt)
        sup = None if support is None else fortran(support, np.uint8)
        msk = None if mask is None else fortran(mask, np.uint8)
        ini = None if initial is None else fortran(initial, rdt)
        pj = None if projections is None else fortran(projections, np.float64)
        an = None if angles is None else fortran(angles, np.float64)
        N = p.numIterations
        nmon = N // p.monitorR_loopLength if (p.monitor_R == 1 and p.monitorR_loopLength > 0) else 0
        rec = np.zeros((p.Dim1, p.Dim2, p.Dim1), dtype=rdt, order="F")
        errK = np.zeros(max(N, 1))
        errR = np.zeros(max(nmon, 1))
        Rarr = np.zeros((p.NumProjs, max(nmon, 1)), order="F")
        Rarr2 = np.zeros((p.NumProjs, max(nmon, 1)), order="F")
        self.check(L.genfire_reconstruct(self._h, C.byref(p), ptr(M), ptr(msk, C.c_uint8), ptr(sup, C.c_uint8),
                                         ptr(ini), ptr(pj, C.c_double), ptr(an, C.c_double), ptr(rec),
                                         ptr(errK, C.c_double), ptr(errR, C.c_double), ptr(Rarr, C.c_double),
                                         ptr(Rarr2, C.c_double)))
        return rec, errK[:N], errR[:nmon], Rarr[:, :nmon], Rarr2[:, :nmon]

    def recon(self, p, measuredK, support=None, initial=None, mask=None, projections=None, angles=None,
              on_device=False):
        return Recon(self, p, measuredK, support, initial, mask, projections, angles, on_device)

    # ---------------------------------------------------------------- projector
    def project(self, vol, angles, vectors=None, precision=PREC_FP64):
        rdt = np.float64 if precision == PREC_FP64 else np.float32
        V = fortran(vol, rdt)
        A = fortran(np.atleast_2d(angles), np.float64)
        P = A.shape[0]
        n1, n2, n3 = V.shape
        out = np.zeros((n1, n2, P), dtype=rdt, order="F")
        vec = None if vectors is None else np.ascontiguousarray(np.asarray(vectors, dtype=np.float64).reshape(9))
        self.check(load().genfire_project(self._h, precision, ptr(V), n1, n2, n3, P, ptr(A, C.c_double),
                                          ptr(vec, C.c_double), ptr(out)))
        return out

    def rfactor(self, vol, angles, measured, vectors=None, precision=PREC_FP64):
        rdt = np.float64 if precision == PREC_FP64 else np.float32
        V = fortran(vol, rdt)
        A = fortran(np.atleast_2d(angles), np.float64)
        P = A.shape[0]
        n1, n2, n3 = V.shape
        Mj = fortran(measured, np.float64)
        vec = None if vectors is None else np.ascontiguousarray(np.asarray(vectors, dtype=np.float64).reshape(9))
        R1 = np.zeros(P)
        R2 = np.zeros(P)
        eR = C.c_double()
        self.check(load().genfire_rfactor(self._h, precision, ptr(V), n1, n2, n3, P, ptr(A, C.c_double),
                                          ptr(vec, C.c_double), ptr(Mj, C.c_double), ptr(R1, C.c_double),
                                          ptr(R2, C.c_double), C.byref(eR)))
        return eR.value, R1, R2

    def set_projector_interpolation(self, interp):
        """INTERP_TRILINEAR (default) or INTERP_CUBIC for every projector use of this context."""
        self.check(load().genfire_set_projector_interpolation(self._h, int(interp)))

    def rfactor_realspace(self, model, projs, angles, precision=PREC_FP64):
        """Tian_calc_Rfactor_realspace: (Rtotal, Rarr, simuProjs float32)."""
        rdt = np.float64 if precision == PREC_FP64 else np.float32
        V = fortran(model, rdt)
        Pj = fortran(projs if np.ndim(projs) == 3 else np.asarray(projs)[:, :, None], np.float64)
        A = fortran(np.atleast_2d(angles), np.float64)
        m1, m2, m3 = V.shape
        p1, p2, P = Pj.shape
        R = np.zeros(P)
        tot = C.c_double()
        simu = np.zeros((p1, p2, P), dtype=np.float32, order="F")
        self.check(load().genfire_rfactor_realspace(self._h, precision, ptr(V), m1, m2, m3, ptr(Pj, C.c_double),
                                                    p1, p2, P, ptr(A, C.c_double), ptr(R, C.c_double),
                                                    C.byref(tot), ptr(simu, C.c_float)))
        return tot.value, R, simu

    # ---------------------------------------------------------------- index / symmetry
    def centro_symmetricity(self, FS, n1, n_k1, n2):
        F = fortran(FS, np.complex128)
        M = np.zeros((n1, n2, n1), dtype=np.complex128, order="F")
        self.check(load().genfire_centro_symmetricity(self._h, ptr(F, C.c_double), n1, n_k1, n2,
                                                      ptr(M, C.c_double)))
        return M

    def hermitian_symmetrize(self, a):
        A = fortran(a, np.complex128)
        out = np.zeros(A.shape, dtype=np.complex128, order="F")
        d = A.shape
        self.check(load().genfire_hermitian_symmetrize(self._h, ptr(A, C.c_double), d[0], d[1], d[2],
                                                       ptr(out, C.c_double)))
        return out

    def rfree_candidates(self, p, measuredK, nbins):
        """Candidate points of the nbins Rfree shells (reconstruct.m:47-50): a
        list of ascending 0-based linear index arrays (int64), one per shell."""
        cdt = np.complex128 if p.precision == PREC_FP64 else np.complex64
        M = fortran(measuredK, cdt)
        counts = np.zeros(nbins, dtype=np.int64)
        self.check(load().genfire_rfree_candidates(self._h, C.byref(p), ptr(M), 0, nbins, ptr(counts, C.c_int64),
                                                   None))
        ind = np.zeros(max(int(counts.sum()), 1), dtype=np.int64)
        self.check(load().genfire_rfree_candidates(self._h, C.byref(p), ptr(M), 0, nbins, ptr(counts, C.c_int64),
                                                   ptr(ind, C.c_int64)))
        off = np.concatenate([[0], np.cumsum(counts)])
        return [ind[off[s]:off[s + 1]].copy() for s in range(nbins)]

    def make_kspace_indices(self, shape):
        Q = np.zeros(tuple(shape), dtype=np.float64, order="F")
        self.check(load().genfire_make_kspace_indices(self._h, shape[0], shape[1], shape[2], ptr(Q, C.c_double)))
        return Q

    def iffshift3_ind(self, size, inds):
        s = np.asarray(size, dtype=np.int32)
        i = np.ascontiguousarray(inds, dtype=np.int64)
        out = np.zeros_like(i)
        self.check(load().genfire_iffshift3_ind(self._h, ptr(s, C.c_int32), i.size, ptr(i, C.c_int64),
                                                ptr(out, C.c_int64)))
        return out

    def fftn(self, a, inverse=False, precision=PREC_FP64):
        cdt = np.complex128 if precision == PREC_FP64 else np.complex64
        A = np.array(a, dtype=cdt, order="F", copy=True)
        d = A.shape + (1,) * (3 - A.ndim)
        self.check(load().genfire_fftn(self._h, precision, ptr(A), d[0], d[1], d[2], 1 if inverse else 0))
        return A


class Recon:
    """A genfire_recon: the staged iteration (create, iterate, result)."""

    def __init__(self, ctx, p, measuredK, support=None, initial=None, mask=None, projections=None, angles=None,
                 on_device=False):
        self.ctx = ctx
        self.p = p
        h = C.c_void_p()
        if on_device:
            # raw device pointers (ints) are passed through
            def dv(x):
                return None if x is None else C.c_void_p(int(x))
            st = load().genfire_recon_create(ctx.handle, C.byref(p), dv(measuredK), dv(mask), dv(support),
                                             dv(initial), dv(projections), dv(angles), 1, C.byref(h))
            self._keep = ()
        else:
            prec = p.precision
            cdt = np.complex128 if prec == PREC_FP64 else np.complex64
            rdt = np.float64 if prec == PREC_FP64 else np.float32
            M = fortran(measuredK, cdt)
            sup = None if support is None else fortran(support, np.uint8)
            msk = None if mask is None else fortran(mask, np.uint8)
            ini = None if initial is None else fortran(initial, rdt)
            pj = None if projections is None else fortran(projections, np.float64)
            an = None if angles is None else fortran(angles, np.float64)
            self._keep = (M, sup, msk, ini, pj, an)
            st = load().genfire_recon_create(ctx.handle, C.byref(p), ptr(M), ptr(msk), ptr(sup), ptr(ini),
                                             ptr(pj), ptr(an), 0, C.byref(h))
        ctx.check(st)
        self._h = h
        ctx._adopt(self)
        self.done = 0

    def iterate(self, count):
        self.ctx.check(load().genfire_recon_iterate(self._h, count))
        self.done += count

    def result(self):
        p = self.p
        rdt = np.float64 if p.precision == PREC_FP64 else np.float32
        rec = np.zeros((p.Dim1, p.Dim2, p.Dim1), dtype=rdt, order="F")
        errK = np.zeros(max(self.done, 1))
        nmon = self.done // p.monitorR_loopLength if (p.monitor_R == 1 and p.monitorR_loopLength > 0) else 0
        errR = np.zeros(max(nmon, 1))
        Rarr = np.zeros((p.NumProjs, max(nmon, 1)), order="F")
        Rarr2 = np.zeros((p.NumProjs, max(nmon, 1)), order="F")
        self.ctx.check(load().genfire_recon_result(self._h, ptr(rec), ptr(errK), ptr(errR, C.c_double),
                                                   ptr(Rarr, C.c_double), ptr(Rarr2, C.c_double), 0))
        return rec, errK[:self.done], errR[:nmon], Rarr[:, :nmon], Rarr2[:, :nmon]

    def set_rfree(self, shells):
        """Withheld Rfree points (list of 0-based centred linear index arrays,
        one per shell, already cleared in the mask given at creation)."""
        counts = np.array([len(x) for x in shells], dtype=np.int64)
        ind = np.ascontiguousarray(np.concatenate([np.asarray(x, dtype=np.int64) for x in shells])
                                   if len(shells) else np.zeros(1, dtype=np.int64))
        self.ctx.check(load().genfire_recon_set_rfree(self._h, len(shells), ptr(counts, C.c_int64),
                                                      ptr(ind, C.c_int64)))
        self._rfree_keep = (counts, ind)

    def rfree(self):
        """Rfree_complex so far: array (nshells, iterations)."""
        ns = C.c_int32(0)
        self.ctx.check(load().genfire_recon_rfree(self._h, C.byref(ns), None))
        out = np.zeros((max(ns.value, 1), max(self.done, 1)), order="F")
        self.ctx.check(load().genfire_recon_rfree(self._h, C.byref(ns), ptr(out, C.c_double)))
        return out[:ns.value, :self.done]

    def profile(self, iterations):
        """Per-kernel mean ms and algorithmic bytes per launch over `iterations` iterations."""
        ms = np.zeros(PROFILE_KERNELS)
        by = np.zeros(PROFILE_KERNELS)
        self.ctx.check(load().genfire_recon_profile(self._h, iterations, ptr(ms, C.c_double), ptr(by, C.c_double)))
        self.done += iterations
        names = [load().genfire_profile_kernel_name(k).decode() for k in range(PROFILE_KERNELS)]
        return names, ms, by

    def tuning(self):
        """Autotuned FFT-pass variants (F2, F3, I2): 0 generic, 1 / 2 radix-8 register engine with 1 / 2
        columns per thread, 3 mixed radix, 4 radix-32 engine (512 or 1024 complex64 points)."""
        v = np.zeros(3, dtype=np.int32)
        self.ctx.check(load().genfire_recon_tuning(self._h, ptr(v, C.c_int32)))
        return [int(x) for x in v]

    def result_device(self, d_rec_ptr, d_errK_ptr=None):
        self.ctx.check(load().genfire_recon_result(self._h, C.c_void_p(d_rec_ptr),
                                                   C.c_void_p(d_errK_ptr) if d_errK_ptr else None,
                                                   None, None, None, 1))

    def close(self):
        if getattr(self, "_h", None):
            if self.ctx.handle:  # a closed context has already freed it
                load().genfire_recon_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ReconBatch:
    """A genfire_recon_batch: one graph launch iterates every member Recon concurrently."""

    def __init__(self, ctx, members):
        self.ctx = ctx
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m._h.value for m in self.members])
        h = C.c_void_p()
        ctx.check(load().genfire_recon_batch_create(ctx.handle, len(self.members), arr, C.byref(h)))
        self._h = h
        ctx._adopt(self)

    def iterate(self, count):
        self.ctx.check(load().genfire_recon_batch_iterate(self._h, count))
        for m in self.members:
            m.done += count

    def close(self):
        if getattr(self, "_h", None):
            if self.ctx.handle:  # a closed context has already freed it
                load().genfire_recon_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def grid_size(p, method=None):
    """(n1, n2) of measuredK for p's griddingMethod, or for `method` (1 FFT, 2 DFT) if given."""
    q = p
    if method is not None:
        q = Params()
        C.pointer(q)[0] = p
        q.griddingMethod = method
    n1 = C.c_int32()
    n2 = C.c_int32()
    st = load().genfire_grid_size(C.byref(q), C.byref(n1), C.byref(n2))
    if st != GENFIRE_OK:
        raise GenfireError(st, "GENFIRE: FFT gridding: Dim2 * oversamplingRatio (1 + (Dim2-1) * "
                               "oversamplingRatio for odd Dim2) must be an integer.")
    return n1.value, n2.value


def volumn_index(big, ori):
    b = np.asarray(big, dtype=np.int32)
    o = np.asarray(ori, dtype=np.int32)
    out = np.zeros(6, dtype=np.int32)
    st = load().genfire_volumn_index(ptr(b, C.c_int32), ptr(o, C.c_int32), ptr(out, C.c_int32))
    if st != GENFIRE_OK:
        raise GenfireError(st, (load().genfire_last_error(None) or b"").decode())
    return out.reshape(3, 2, order="F")
