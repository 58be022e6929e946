"""Generate the committed golden fixtures (run in the build container).

turb3_subset.npz
    Every 4th projection of the reference's own fixture
    data_turb3/pj_new_Turbu3_1015.mat (64 x 64, float64) with its angles
    (data_turb3/angles_usedin_refine_1015.mat), so tests can run on real data
    where the reference tree is absent.
turb3_oracle.npz
    Outputs of the CPU oracle on that subset (Genfire_test.m parameters with
    oversamplingRatio 2): per-projection K-point counts and SHA-256 digests of
    the selected index / D / u / v arrays, sampled measuredK values, a
    recIFFT slice, and 20 iterations of reconstruct (errK and a slice).

Usage:  python tests/golden/make_golden.py [path/to/reference]
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

TURB3_PARAMS = dict(oversamplingRatio=2.0, interpolationCutoffDistance=0.125, DFT_CentroSymmetricity=1,
                    vector1=(0, 0, 1), vector2=(0, 1, 0), vector3=(1, 0, 0), numIterations=20,
                    constraintEnforcementMode=3, constraintPositivity=1, constraintSupport=1)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def turb3_oracle(projs, angles):
    P = projs.shape[2]
    prm = O.make_params(projs.shape[0], projs.shape[1], P, **TURB3_PARAMS)
    n1 = O.oversampled(prm.Dim1, prm.oversamplingRatio)
    n2 = O.oversampled(prm.Dim2, prm.oversamplingRatio)
    digests = []
    for p in range(P):
        Rf, nrm = O.proj_geometry(prm, angles[p, 0], angles[p, 1], angles[p, 2])
        ind, dist, u, v, _ = O.select(n1, n2, 1, prm.interpolationCutoffDistance, Rf, nrm)
        digests.append([sha(ind.astype(np.int64)), sha(dist), sha(u), sha(v)])
    M, rec, nk = O.grid_dft(prm, projs, angles)
    rng = np.random.default_rng(7)
    nz = np.flatnonzero(M.reshape(-1, order="F"))
    sidx = np.sort(rng.choice(nz, size=min(2000, nz.size), replace=False))
    recon, errK, _, _, _ = O.reconstruct(prm, M)
    return dict(nk=nk, digests=np.array(digests), sample_idx=sidx, sample_val=M.reshape(-1, order="F")[sidx],
                M_abs_sum=np.abs(M).sum(), M_l2=np.linalg.norm(M), nnz=nz.size,
                rec_slice=rec[:, :, prm.Dim1 // 2].copy(), rec_l2=np.linalg.norm(rec),
                errK=errK, recon_slice=recon[:, :, prm.Dim1 // 2].copy(), recon_l2=np.linalg.norm(recon))


def main(ref=None):
    """ref: the reference tree (argument, or the GENFIRE_REFERENCE environment variable)."""
    import scipy.io
    ref = ref or os.environ.get("GENFIRE_REFERENCE")
    if not ref:
        raise SystemExit("usage: make_golden.py <reference tree>  (or set GENFIRE_REFERENCE)")
    pj = scipy.io.loadmat(os.path.join(ref, "data_turb3", "pj_new_Turbu3_1015.mat"))["pj_new_Turbu3_1015"]
    an = scipy.io.loadmat(os.path.join(ref, "data_turb3", "angles_usedin_refine_1015.mat"))["euler_angles"]
    projs = np.asfortranarray(pj[:, :, ::4], dtype=np.float64)
    angles = np.asfortranarray(an[::4], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "turb3_subset.npz"), projections=projs, angles=angles)
    out = turb3_oracle(projs, angles)
    np.savez_compressed(os.path.join(HERE, "turb3_oracle.npz"), **out)
    print("projections", projs.shape, "nk", out["nk"], "errK[-1]", out["errK"][-1])


if __name__ == "__main__":
    main(*sys.argv[1:])
