"""GB300 pair-counting engine for FCFC's hot path.

The compute path is libfcfcg.so (CUDA kernels for sm_103a behind a C ABI,
include/fcfcg.h); this package is its Python front end.
"""
from .capi import (BIN_ISO, BIN_SMU, BIN_SPI, GEOM_BOX, GEOM_SURVEY,  # noqa: F401
                   PREC_FP32_RECHECK, PREC_FP64, FCFCGError, load_library)
from .engine import PairCounter  # noqa: F401

__version__ = "0.1.0"
