"""A gridding case for profilers (ncu): fillInFourierGrid_DFT calls of the
benchmark's shape (90 random-Euler projections of 256 x 256, oversampling 2,
cutoff 0.125) on random projection data, in MIXED (split-BF16) or
FP16_SCALED (split-FP16) precision.

    python -m genfire_gb300.profile_grid_case [calls] [mixed|fp16]
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
    calls = int(argv[0]) if argv else 1
    prec = argv[1] if len(argv) > 1 else "mixed"
    rng = np.random.default_rng(0)
    D, P = 256, 90
    projs = np.asfortranarray(rng.random((D, D, P)))
    angles = np.asfortranarray(np.stack([rng.uniform(0, 360, P), rng.uniform(-72, 72, P), rng.uniform(0, 360, P)], 1))
    p = G.default_params()
    p.Dim1 = p.Dim2 = D
    p.NumProjs = P
    p.oversamplingRatio = 2.0
    p.interpolationCutoffDistance = 0.125
    p.vector3[0] = 0
    p.vector3[2] = 1
    p.precision = G.PREC_FP16_SCALED if prec == "fp16" else G.PREC_MIXED
    ctx = G.Context(0)
    for _ in range(calls):
        t0 = time.time()
        M, _, nk = ctx.grid_dft(p, projs, angles, want_rec=False)
        print("gridding call %.4f s, %d points" % (time.time() - t0, int(nk.sum())))


if __name__ == "__main__":
    main(sys.argv[1:])
