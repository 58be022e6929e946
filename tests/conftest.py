import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path through the C ABI)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def lib():
    from genfire_gb300 import build
    build.build()
    import genfire_gb300 as G
    G.load()
    return G


@pytest.fixture(scope="session")
def ctx(lib):
    c = lib.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    d = os.path.join(ROOT, "tests", "golden")
    return dict(subset=np.load(os.path.join(d, "turb3_subset.npz")),
                oracle=np.load(os.path.join(d, "turb3_oracle.npz")))


def params(G, D1, D2, P, **kw):
    """genfire_params with the class defaults, the sizes and overrides."""
    p = G.default_params()
    p.Dim1, p.Dim2, p.NumProjs = D1, D2, P
    for k, v in kw.items():
        if k in ("vector1", "vector2", "vector3"):
            getattr(p, k)[:] = [float(x) for x in v]
        elif k == "precision":
            p.precision = {"mixed": G.PREC_MIXED, "fp16": G.PREC_FP16_SCALED}.get(v, G.PREC_FP64)
        else:
            setattr(p, k, v)
    return p


def rel(a, b):
    import numpy as np
    nb = np.linalg.norm(np.asarray(b).ravel())
    return np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel()) / (nb if nb > 0 else 1.0)
