"""GB300-native reconstruction hot path of FasterBackprojection.

The compute lives in libfbp.so (C ABI, include/fbp.h); this package is the
Python-side binding used by the tests and the benchmark, plus the synthetic
capture generator and the capture file formats.
"""
from ._lib import (  # noqa: F401
    FBP_BF16,
    FBP_BORDER_EDGE,
    FBP_BORDER_ZERO,
    FBP_CONFOCAL,
    FBP_EXHAUSTIVE,
    FBP_F16,
    FBP_F32,
    FBP_FILTER_LAPLACIAN,
    FBP_FILTER_LOG,
    FBP_FILTER_LOG_FFT,
    FBP_FILTER_NONE,
    FBP_LAYOUT_TIME_INNER,
    FBP_LAYOUT_TIME_MAJOR,
    FBP_LCT_GRID_DEPTH,
    FBP_LCT_GRID_REFERENCE,
    FBP_LCT_OUTPUT_CLAMPED_REAL,
    FBP_LCT_OUTPUT_MAGNITUDE,
    FBP_MIS_LEARNED,
    FBP_MIS_REFERENCE,
    FBP_MIS_REFERENCE_SCATTER,
    FBP_MIS_SPATIAL,
    FBP_MIS_UNIFORM,
    FBP_WEIGHTS_BATCHED,
    FBP_WEIGHTS_REFERENCE,
    FbpError,
    ReconInfo,
    ShapeParams,
)
from .api import Batch, Context, Mlp, make_info  # noqa: F401
