"""GENFIRE v2 reconstruction hot path on GB300 (sm_103a).

libgenfire.so (C ABI: include/genfire.h) holds the CUDA kernels; this package
binds it (``_lib``), mirrors the reference's GENFIRE_Reconstructor class
(``reconstructor``) and generates synthetic tilt series (``synth``).
"""
from ._lib import (Context, GenfireError, INTERP_CUBIC, INTERP_TRILINEAR, Params, PREC_FP16_SCALED,  # noqa: F401
                   PREC_FP64, PREC_MIXED, ReconBatch, default_params, grid_size, load, volumn_index)
from .reconstructor import GENFIRE_Reconstructor  # noqa: F401
