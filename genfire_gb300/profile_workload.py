"""Cases for profilers (ncu) on the benchmark's own seeded workload: the 256^3
object of 2000 Gaussian atoms, 90 random-Euler projections of 256 x 256
(genfire_gb300.synth "euler256"), oversampling 2, cutoff 0.125, mode 3,
positivity and the ellipsoid support.

    python -m genfire_gb300.profile_workload grid [calls] [mixed|fp16]
        fillInFourierGrid_DFT calls (selection, tensor-core DFT, zero fill, sums)
    python -m genfire_gb300.profile_workload iterate [iterations]
        the constraint table of the MIXED grid, then iterations (F1 F2 F3 I2 I1)
    python -m genfire_gb300.profile_workload project [calls]
        the MIXED R-factor of the ground-truth volume against the projections
        (k_project<float, trilinear> with the fused sums)
    python -m genfire_gb300.profile_workload fftgrid [calls]
        fillInFourierGrid (griddingMethod 1) calls, MIXED

The workload's projections are made by the FP64 projector (three launches of
k_project<double>) before the case runs.
"""
import os
import sys
import time

import numpy as np


def _setup():
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import __graft_entry__ as ge
    ge.build()
    import genfire_gb300 as G
    from genfire_gb300 import synth
    ctx = G.Context(0)

    def proj(vol, angles, vectors):
        return ctx.project(vol.astype(np.float64), angles, vectors=np.asarray(vectors, float).reshape(-1))
    w = synth.make_workload("euler256", proj)
    return G, ctx, w


def _params(G, w, precision, iters=1):
    p = G.default_params()
    D = w["D"]
    p.Dim1, p.Dim2, p.NumProjs = D, D, w["projections"].shape[2]
    p.oversamplingRatio = w["os"]
    p.interpolationCutoffDistance = 0.125
    for k, v in zip(("vector1", "vector2", "vector3"), w["vectors"]):
        getattr(p, k)[:] = [float(x) for x in v]
    p.numIterations = iters
    p.constraintEnforcementMode = 3
    p.constraintPositivity = 1
    p.constraintSupport = 1
    p.precision = precision
    return p


def main(argv):
    case = argv[0] if argv else "grid"
    G, ctx, w = _setup()
    projs, angles = w["projections"], w["angles_in"]
    if case == "grid":
        calls = int(argv[1]) if len(argv) > 1 else 2
        prec = G.PREC_FP16_SCALED if len(argv) > 2 and argv[2] == "fp16" else G.PREC_MIXED
        p = _params(G, w, prec)
        for _ in range(calls):
            t0 = time.time()
            _, _, nk = ctx.grid_dft(p, projs, angles, want_rec=False)
            print("gridding call %.4f s, %d points" % (time.time() - t0, int(nk.sum())))
    elif case == "iterate":
        iters = int(argv[1]) if len(argv) > 1 else 6
        M, _, _ = ctx.grid_dft(_params(G, w, G.PREC_MIXED), projs, angles, want_rec=False)
        p = _params(G, w, G.PREC_MIXED, iters)
        r = ctx.recon(p, M, support=w["support"])
        t0 = time.time()
        r.iterate(iters)
        print("iterations", iters, "wall %.4f s" % (time.time() - t0), "measured points", np.count_nonzero(M),
              "pass variants (F2, F3, I2)", r.tuning())
        r.close()
    elif case == "project":
        calls = int(argv[1]) if len(argv) > 1 else 2
        vol = w["vol"].astype(np.float32)
        for _ in range(calls):
            t0 = time.time()
            errR, _, _ = ctx.rfactor(vol, angles, projs, vectors=np.asarray(w["vectors"], float).reshape(-1),
                                     precision=G.PREC_MIXED)
            print("R-factor call %.4f s, errR %.6f" % (time.time() - t0, errR))
    elif case == "fftgrid":
        calls = int(argv[1]) if len(argv) > 1 else 2
        p = _params(G, w, G.PREC_MIXED)
        p.griddingMethod = 1
        p.allowMultipleGridMatches = 1
        for _ in range(calls):
            t0 = time.time()
            _, _, npairs = ctx.grid_fft(p, projs, angles, want_rec=False)
            print("FFT gridding call %.4f s, %d pairs" % (time.time() - t0, int(npairs)))
    else:
        raise SystemExit("unknown case %r (grid, iterate, project, fftgrid)" % case)


if __name__ == "__main__":
    main(sys.argv[1:])
