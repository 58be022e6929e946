"""A compact iteration case for profilers (ncu): by default the 256^3 object /
512^3 grid of the benchmark with a synthetic measured set (thin slabs around
30 random planes through the origin, about 2.3 M points), so a capture holds
~2.6 GB on the device and reaches the iteration kernels after a few launches.
Dim1 and Dim2 may be given (oversampling 2), e.g. 512 128 for a 1024 x 256 x
1024 grid whose dim-1 and dim-3 passes are 1024-point transforms.

    python -m genfire_gb300.profile_case [mixed|fp64] [iterations] [Dim1 Dim2]
"""
import os
import sys
import time

import numpy as np


def main(argv):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import __graft_entry__ as ge
    ge.build()
    import genfire_gb300 as G
    prec = G.PREC_MIXED if (len(argv) < 1 or argv[0] == "mixed") else G.PREC_FP64
    iters = int(argv[1]) if len(argv) > 1 else 3
    D1 = int(argv[2]) if len(argv) > 3 else 256
    D2 = int(argv[3]) if len(argv) > 3 else 256
    n1, n2 = 2 * D1, 2 * D2
    rng = np.random.default_rng(0)
    M = np.zeros((n1, n2, n1), dtype=np.complex64 if prec == G.PREC_MIXED else np.complex128, order="F")
    k1, k2 = np.arange(n1) - n1 // 2, np.arange(n2) - n2 // 2
    X, Y = np.meshgrid(k1, k2, indexing="ij")
    for _ in range(30):
        nrm = rng.standard_normal(3)
        nrm /= np.linalg.norm(nrm)
        base = X * nrm[0] + Y * nrm[1]
        if n1 == 512 and n2 == 512:
            # the default case, slice by slice (the set its profiles were taken on)
            for i3 in range(n1):
                m = np.abs(base + k1[i3] * nrm[2]) < 0.125
                if m.any():
                    M[:, :, i3][m] = (rng.standard_normal(m.sum()) + 1j * rng.standard_normal(m.sum())).astype(M.dtype)
            continue
        # other sizes: per (k1, k2) the few k3 within 0.125 of the plane
        if abs(nrm[2]) < 1e-3:
            continue
        c = np.rint(-base / nrm[2]).astype(np.int64)
        reach = int(np.ceil(0.125 / abs(nrm[2]))) + 1
        for d in range(-reach, reach + 1):
            k3 = c + d
            m = (np.abs(base + k3 * nrm[2]) < 0.125) & (k3 >= k1[0]) & (k3 <= k1[-1])
            if m.any():
                i1, i2 = np.nonzero(m)
                M[i1, i2, k3[m] + n1 // 2] = (rng.standard_normal(m.sum()) + 1j * rng.standard_normal(m.sum())).astype(M.dtype)
    p = G.default_params()
    p.Dim1, p.Dim2 = D1, D2
    p.NumProjs = 1
    p.oversamplingRatio = 2.0
    p.numIterations = iters
    p.constraintEnforcementMode = 3
    p.precision = prec
    ctx = G.Context(0)
    r = ctx.recon(p, M)
    t0 = time.time()
    r.iterate(iters)
    print("iterations", iters, "wall %.4f s" % (time.time() - t0), "measured points", np.count_nonzero(M),
          "pass variants (F2, F3, I2)", r.tuning())


if __name__ == "__main__":
    main(sys.argv[1:])
