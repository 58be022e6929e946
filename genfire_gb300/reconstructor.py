"""GENFIRE_Reconstructor, the host-side mirror of the reference class.

Same property names, defaults and method names as
@GENFIRE_Reconstructor/GENFIRE_Reconstructor.m; the hot-path methods
(fillInFourierGrid_DFT, CentroSymmetricity, reconstruct) call libgenfire.so
through its C ABI.  MATLAB's value semantics (``obj = obj.method()``) are kept
by returning ``self`` from every method, so a script written as

    G = GENFIRE_Reconstructor()
    G.filename_Projections = ...
    G = G.readFiles(); G = G.CheckPrepareData(); G = G.runGridding(); G = G.reconstruct()

reads as Genfire_test.m does.  Errors raise GenfireError with the reference's
'GENFIRE: ...' messages.
"""
import os

import numpy as np

from . import _lib
from ._lib import GenfireError, PREC_FP16_SCALED, PREC_FP64, PREC_MIXED

_PROPS = dict(
    # internal variables (GENFIRE_Reconstructor.m:6-28)
    InputProjections=None, InputAngles=None, measuredK=None, measuredK_mask=None, Support=None,
    initialObject=None, recIFFT=None, reconstruction=None, errK=None, errR=None, Dim1=None, Dim2=None,
    n1_oversampled=None, n2_oversampled=None, NumProjs=None, Rfree_complex=None,
    constraintEnforcementDelayIndicators=None, Rarr_record=None, Rarr2_record=None, simuProjs=None,
    # R factor monitoring (:30-32)
    monitor_R=0, monitorR_loopLength=10,
    # filenames (:34-39)
    filename_Projections="", filename_Angles="", filename_Support="", filename_InitialModel="",
    filename_Results="./results/GENFIRE_rec.mat",
    # reconstruction parameters (:41-47)
    numIterations=50, oversamplingRatio=3, interpolationCutoffDistance=.7, griddingMethod=1,
    allowMultipleGridMatches=1, calculate_Rfree=0,
    # read by reconstruct.m:46-60 but not declared by the reference class: the
    # number of resolution shells, the withheld fraction per shell and the seed
    numBinsRfree=10, percentValuesForRfree=0.05, RandomSeed=None,
    # axes vectors for phi, theta, psi (:49-52)
    vector1=(0, 0, 1), vector2=(0, 1, 0), vector3=(1, 0, 0),
    particleWindowSize=None,
    # constraints (:57-60)
    constraintEnforcementMode=1, constraintPositivity=1, constraintSupport=1,
    # DFT related (:62-65).  DFT_doGPU keeps the reference's default and is not
    # read: this implementation grids on the GPU whatever its value.
    DFT_CentroSymmetricity=1, DFT_doGPU=0, Vol_ind=None,
    # temp saves (:67-70)
    save_temp=0, save_loopLength=50, saveFilename="./results/temp_rec",
    # this build: arithmetic of the GPU path, 'fp64' (drop-in), 'mixed' (split-BF16 gridding,
    # complex64 iteration) or 'fp16_scaled' (split-FP16 gridding, complex64 iteration)
    precision="fp64", device=0,
)


def _load_array(fname):
    """importdata for the formats a Python caller has: .npy, .npz or MAT v5 (first variable)."""
    if fname.endswith(".npy"):
        return np.load(fname)
    if fname.endswith(".npz"):
        z = np.load(fname)
        return z[z.files[0]]
    import scipy.io
    d = scipy.io.loadmat(fname)
    keys = [k for k in d if not k.startswith("__")]
    return d[keys[0]]


def _exists(fname):
    return bool(fname) and os.path.isfile(fname)


class GENFIRE_Reconstructor:
    _ctx_cache = {}

    def __init__(self, **kw):
        for k, v in _PROPS.items():
            setattr(self, k, v)
        for k, v in kw.items():
            if k not in _PROPS:
                raise GenfireError(_lib.GENFIRE_ERR_ARG, "GENFIRE: Invalid option %s provided." % k)
            setattr(self, k, v)

    # ------------------------------------------------------------------ helpers
    def _ctx(self):
        c = GENFIRE_Reconstructor._ctx_cache.get(self.device)
        if c is None:
            c = _lib.Context(self.device)
            GENFIRE_Reconstructor._ctx_cache[self.device] = c
        return c

    def _prec(self):
        if self.precision in ("fp64", PREC_FP64):
            return PREC_FP64
        if self.precision in ("mixed", PREC_MIXED):
            return PREC_MIXED
        if self.precision in ("fp16_scaled", PREC_FP16_SCALED):
            return PREC_FP16_SCALED
        raise GenfireError(_lib.GENFIRE_ERR_ARG, "GENFIRE: precision must be 'fp64', 'mixed' or 'fp16_scaled'.")

    def params(self):
        """The genfire_params of the current properties."""
        p = _lib.default_params()
        p.Dim1 = int(self.Dim1)
        p.Dim2 = int(self.Dim2)
        p.NumProjs = int(self.NumProjs)
        p.DFT_CentroSymmetricity = int(self.DFT_CentroSymmetricity)
        p.oversamplingRatio = float(self.oversamplingRatio)
        p.interpolationCutoffDistance = float(self.interpolationCutoffDistance)
        for name in ("vector1", "vector2", "vector3"):
            getattr(p, name)[:] = [float(x) for x in np.asarray(getattr(self, name), dtype=float).reshape(3)]
        p.numIterations = int(self.numIterations)
        p.constraintEnforcementMode = int(self.constraintEnforcementMode)
        p.constraintPositivity = int(bool(self.constraintPositivity))
        p.constraintSupport = int(bool(self.constraintSupport))
        p.monitor_R = int(self.monitor_R)
        p.monitorR_loopLength = int(self.monitorR_loopLength)
        p.precision = self._prec()
        p.griddingMethod = int(self.griddingMethod)
        p.allowMultipleGridMatches = int(bool(self.allowMultipleGridMatches))
        return p

    # ------------------------------------------------------------------ GENFIRE_Reconstructor.m:82-112
    def readFiles(self):
        if _exists(self.filename_Projections):
            self.InputProjections = _load_array(self.filename_Projections)
        else:
            raise GenfireError(_lib.GENFIRE_ERR_ARG, "GENFIRE: Projections file does not exist!")
        if _exists(self.filename_Angles):
            self.InputAngles = _load_array(self.filename_Angles)
        else:
            raise GenfireError(_lib.GENFIRE_ERR_ARG, "GENFIRE: Angles file does not exist!")
        if self.filename_Support:
            if _exists(self.filename_Support):
                self.Support = _load_array(self.filename_Support) != 0
            else:
                print("GENFIRE: Support file does not exist!Making a support based on Projections.")
                s = self.InputProjections.shape
                self.Support = np.ones((s[0], s[1], s[0]), dtype=bool)
        if self.filename_InitialModel:
            if _exists(self.filename_InitialModel):
                self.initialObject = _load_array(self.filename_InitialModel)
            else:
                raise GenfireError(_lib.GENFIRE_ERR_ARG, "GENFIRE: Inital Model file does not exist!")
        return self

    # ------------------------------------------------------------------ :115-171
    def CheckPrepareData(self):
        P = np.asarray(self.InputProjections)
        if P.ndim == 2:
            P = P[:, :, None]
        self.InputProjections = P
        self.NumProjs = P.shape[2]
        self.Dim1 = P.shape[0]
        self.Dim2 = P.shape[1]
        self.particleWindowSize = [self.Dim1, self.Dim2]
        A = np.atleast_2d(np.asarray(self.InputAngles, dtype=np.float64))
        if A.shape[0] == 1 and self.NumProjs != 1:
            A = A.T
        if self.NumProjs != A.shape[0]:
            raise GenfireError(_lib.GENFIRE_ERR_ARG, "GENFIRE: Number of projections and Angles does not match!")
        if A.shape[1] > 3:
            raise GenfireError(_lib.GENFIRE_ERR_ARG, "GENFIRE: Input Angle 2nd dimenstions larger than three!")
        if A.shape[1] == 1:
            # a single angle per projection is theta; phi = psi = 0
            A = np.concatenate([np.zeros_like(A), A, np.zeros_like(A)], axis=1)
        self.InputAngles = A
        if self.initialObject is not None:
            if tuple(np.shape(self.initialObject)) != (self.Dim1, self.Dim2, self.Dim1):
                raise GenfireError(_lib.GENFIRE_ERR_ARG, "GENFIRE: Initial Model size does not match with projections!")
        if self.Support is None:
            self.Support = np.ones((self.Dim1, self.Dim2, self.Dim1), dtype=bool)
        if self.griddingMethod > 2:
            raise GenfireError(_lib.GENFIRE_ERR_ARG, "GENFIRE: Unrecognized gridding method.")
        mode = self.constraintEnforcementMode
        if mode == 1:
            d = np.concatenate([0.95 - 0.1 * np.arange(12), [-10, -10, -10], -0.15 + 0.1 * np.arange(12)])
        elif mode == 2:
            d = np.concatenate([0.95 - 0.1 * np.arange(12), [-10, -10]])
        elif mode == 3:
            d = np.array([-999.0] * 5)
        else:
            raise GenfireError(_lib.GENFIRE_ERR_ARG,
                               "GENFIRE: ERROR! constraintEnforcementMode value %d not understood" % mode)
        self.constraintEnforcementDelayIndicators = d
        self.n1_oversampled = int(_mround(self.Dim1 * self.oversamplingRatio))
        self.n2_oversampled = int(_mround(self.Dim2 * self.oversamplingRatio))
        return self

    # ------------------------------------------------------------------ :172-186
    def runGridding(self):
        print("GENFIRE: Assembling Fourier grid...\n")
        if self.griddingMethod == 1:
            self.fillInFourierGrid()
        if self.griddingMethod == 2:
            self.fillInFourierGrid_DFT()
        if self._prec() != PREC_FP64:
            self.measuredK = np.asfortranarray(self.measuredK, dtype=np.complex64)
        self.measuredK_mask = self.measuredK != 0
        self.Vol_ind = _lib.volumn_index(self.measuredK.shape, [self.Dim1, self.Dim2, self.Dim1])
        return self

    def fillInFourierGrid(self):
        """@GENFIRE_Reconstructor/fillInFourierGrid.m:27-168 (griddingMethod 1) on the GPU."""
        p = self.params()
        M, rec, n = self._ctx().grid_fft(p, self.InputProjections, self.InputAngles, want_rec=True)
        self.measuredK = M
        self.recIFFT = rec
        self.gridded_points = n
        print("GENFIRE: Fourier grid assembled.\n")
        return self

    def fillInFourierGrid_DFT(self):
        """@GENFIRE_Reconstructor/fillInFourierGrid_DFT.m:85-310 on the GPU."""
        p = self.params()
        M, rec, nk = self._ctx().grid_dft(p, self.InputProjections, self.InputAngles, want_rec=True)
        self.measuredK = M
        self.recIFFT = rec
        self.gridded_points = nk
        return self

    def CentroSymmetricity(self, FS, n1, n_k1, n2):
        """@GENFIRE_Reconstructor/CentroSymmetricity.m:2-72 on the GPU."""
        self.measuredK = self._ctx().centro_symmetricity(FS, n1, n_k1, n2)
        return self

    def reset_measuredK_mask(self):
        self.measuredK_mask = self.measuredK != 0
        return self

    # ------------------------------------------------------------------ reconstruct.m:28-194
    def reconstruct(self):
        p = self.params()
        # reconstruct.m works on size(measuredK): pick the grid convention that matches it
        shape = tuple(np.shape(self.measuredK))
        for method in (int(self.griddingMethod), 2, 1):
            try:
                n1, n2 = _lib.grid_size(p, method=method)
            except GenfireError:
                continue
            if shape == (n1, n2, n1):
                p.griddingMethod = method
                break
        else:
            raise GenfireError(_lib.GENFIRE_ERR_ARG, "GENFIRE: measuredK size does not match the projections.")
        shells = None
        mask = None
        if self.measuredK_mask is not None and not np.array_equal(self.measuredK_mask, self.measuredK != 0):
            mask = self.measuredK_mask
        if self.calculate_Rfree == 1:
            shells, mask = self._withhold_rfree(p, mask)
        print("GENFIRE: Reconstructing... \n")
        kw = dict(support=self.Support, initial=self.initialObject, mask=mask,
                  projections=self.InputProjections if p.monitor_R == 1 else None,
                  angles=self.InputAngles if p.monitor_R == 1 else None)
        save_every = int(self.save_loopLength) if int(self.save_temp) == 1 else 0
        if shells is None and save_every <= 0:
            rec, errK, errR, Rarr, Rarr2 = self._ctx().reconstruct(p, self.measuredK, **kw)
        else:
            r = self._ctx().recon(p, self.measuredK, **kw)
            try:
                if shells is not None:
                    r.set_rfree(shells)
                done = 0
                while done < p.numIterations:
                    step = p.numIterations - done
                    if save_every > 0:
                        step = min(step, save_every - done % save_every)
                    r.iterate(step)
                    done += step
                    if save_every > 0 and done % save_every == 0:
                        self._save_temp(r.result()[0], done)
                rec, errK, errR, Rarr, Rarr2 = r.result()
                if shells is not None:
                    self.Rfree_complex = r.rfree().astype(np.float32)
            finally:
                r.close()
        self.reconstruction = rec
        self.errK = errK
        if p.monitor_R == 1:
            self.errR = errR
            self.Rarr_record = Rarr
            self.Rarr2_record = Rarr2
        return self

    def _save_temp(self, rec, iteration):
        """reconstruct.m:155-158: the best object so far (cropped, after
        positivity and support) saved as temp_reconstruction to
        [saveFilename, num2str(iterationNum), '.mat']."""
        fn = "%s%d.mat" % (self.saveFilename, iteration)
        d = os.path.dirname(fn)
        if d:
            os.makedirs(d, exist_ok=True)
        import scipy.io
        scipy.io.savemat(fn, {"temp_reconstruction": rec})

    def _withhold_rfree(self, p, mask):
        """Rfree point selection (reconstruct.m:46-67): per shell, the candidates
        (measuredK ~= 0 in the shell, computed by the library), shuffled, the first
        floor(n * percentValuesForRfree) (at least one) withheld and cleared from
        the mask.  The shuffle is numpy's generator seeded with RandomSeed before
        every shell (the reference re-seeds MATLAB's rng the same way); MATLAB's
        randperm stream itself is not reproduced.  Returns (shells, mask)."""
        nb = int(self.numBinsRfree)
        cands = self._ctx().rfree_candidates(p, self.measuredK, nb)
        m = np.array(self.measuredK != 0 if mask is None else mask, dtype=bool, order="F", copy=True)
        flat = m.reshape(-1, order="F")
        shared = np.random.default_rng()
        shells = []
        for s, c in enumerate(cands):
            rng = np.random.default_rng(self.RandomSeed) if self.RandomSeed is not None else shared
            cut = int(np.floor(len(c) * float(self.percentValuesForRfree)))
            if cut == 0:
                cut = 1
            if len(c) < cut:
                raise GenfireError(_lib.GENFIRE_ERR_ARG,
                                   "GENFIRE: Rfree shell %d has no measured points to withhold." % (s + 1))
            sel = c[rng.permutation(len(c))][:cut]
            flat[sel] = False
            shells.append(sel)
        return shells, m

    # ------------------------------------------------------------------ :194-225
    def ClearCalcVariables(self):
        self.InputProjections = None
        self.InputAngles = None
        self.initialObject = None
        self.recIFFT = None
        return self

    def SaveResults(self):
        fn = self.filename_Results
        d = os.path.dirname(fn)
        if d:
            os.makedirs(d, exist_ok=True)
        out = {k: getattr(self, k) for k in ("reconstruction", "errK", "errR", "Rarr_record", "Rarr2_record")
               if getattr(self, k) is not None}
        if fn.endswith(".mat"):
            import scipy.io
            scipy.io.savemat(fn, out)
        else:
            np.savez(fn, **out)

    def set_parameters(self, *args):
        if len(args) % 2 != 0:
            raise GenfireError(_lib.GENFIRE_ERR_ARG,
                               "GENFIRE: Additional argument list not divisible by 2. Options should be 'key','value' pairs.")
        for i in range(0, len(args), 2):
            k, v = args[i], args[i + 1]
            if k in _PROPS:
                setattr(self, k, v)
            else:
                raise GenfireError(_lib.GENFIRE_ERR_ARG, "GENFIRE: Invalid option %s provided." % k)
        return self


def _mround(x):
    return float(np.sign(x) * np.floor(abs(x) + 0.5))
