"""The reference's image code (FasterBackprojection/Image.h: flip, bilinear
resize) behind a host-only harness, oracle/_ref/libref_image.so, built by
`make -C oracle ref` from the reference's sources where they are present.
Test infrastructure: pins oracle/numpy_ref.transient_image."""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "_ref" / "libref_image.so"
_lib = None


def available() -> bool:
    return LIB.exists()


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(LIB))
        _lib.refimg_transient_save.restype = ctypes.c_int
        _lib.refimg_transient_save.argtypes = [ctypes.c_void_p] + [ctypes.c_uint32] * 6 + [ctypes.c_int,
                                                                                           ctypes.c_void_p]
    return _lib


def transient_image(slice_, width, height, size, stride=1, offset=0, normalize=False) -> np.ndarray:
    """The reference's TransientImage::save pixels, uint8 [h][w][4]."""
    s = np.array(slice_, dtype=np.float32)  # a copy: normalize writes into it
    ow, oh = size
    out = np.empty((oh, ow, 4), np.uint8)
    rc = _load().refimg_transient_save(s.ctypes.data, width, height, ow, oh, stride, offset, int(normalize),
                                       out.ctypes.data)
    if rc != 0:
        raise RuntimeError("refimg_transient_save failed")
    return out
