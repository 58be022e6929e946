"""A compact iteration case for profilers (ncu): the 256^3 object / 512^3 grid
of the benchmark with a synthetic measured set (thin slabs around 30 random
planes through the origin, about 2.3 M points), so a capture holds ~2.6 GB on
the device and reaches the iteration kernels after a few launches.

    python -m genfire_gb300.profile_case [mixed|fp64] [iterations]
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
    n, D = 512, 256
    rng = np.random.default_rng(0)
    M = np.zeros((n, n, n), dtype=np.complex64 if prec == G.PREC_MIXED else np.complex128, order="F")
    k = np.arange(n) - n // 2
    X, Y = np.meshgrid(k, k, indexing="ij")
    for _ in range(30):
        nrm = rng.standard_normal(3)
        nrm /= np.linalg.norm(nrm)
        base = X * nrm[0] + Y * nrm[1]
        for i3 in range(n):
            m = np.abs(base + k[i3] * nrm[2]) < 0.125
            if m.any():
                M[:, :, i3][m] = (rng.standard_normal(m.sum()) + 1j * rng.standard_normal(m.sum())).astype(M.dtype)
    p = G.default_params()
    p.Dim1 = p.Dim2 = D
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
