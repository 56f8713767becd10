"""ctypes binding of libfbp.so (the C ABI declared in include/fbp.h).

The library is loaded from the package's ``_lib/`` directory.  There is no
fallback: if the shared object is missing the import raises, so a caller
never silently runs anything but the CUDA path.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_uint32, c_uint64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libfbp.so"

# fbp_status
FBP_OK = 0
FBP_ERR_INVALID_ARG = 1
FBP_ERR_OOM = 2
FBP_ERR_CUDA = 3
FBP_ERR_TIMEOUT = 4
FBP_ERR_UNSUPPORTED = 5
FBP_ERR_DEVICE = 6
FBP_ERR_IO = 7
FBP_ERR_INTERNAL = 8
# fbp_dtype
FBP_F32, FBP_BF16, FBP_F16 = 0, 1, 2
# fbp_layout
FBP_LAYOUT_TIME_MAJOR, FBP_LAYOUT_TIME_INNER = 0, 1
# fbp_capture_system
FBP_CONFOCAL, FBP_EXHAUSTIVE = 0, 1
# fbp_filter
FBP_FILTER_NONE, FBP_FILTER_LAPLACIAN, FBP_FILTER_LOG, FBP_FILTER_LOG_FFT = 0, 1, 2, 3
# fbp_border
FBP_BORDER_ZERO, FBP_BORDER_EDGE = 0, 1
# fbp_weight_mode
FBP_WEIGHTS_BATCHED, FBP_WEIGHTS_REFERENCE = 0, 1

_F3 = c_float * 3
_U3 = c_uint32 * 3


class ReconInfo(ctypes.Structure):
    """fbp_recon_info: the reference's ReconstructionInfo layout (148 bytes)."""

    _fields_ = [
        ("sensor_position", _F3),
        ("capture_system", c_uint32),
        ("laser_position", _F3),
        ("time_offset", c_float),
        ("num_laser_targets", c_uint32),
        ("num_sensor_targets", c_uint32),
        ("num_time_bins", c_uint32),
        ("time_step", c_float),
        ("hidden_min", _F3),
        ("discard_first_last_bounces", c_uint32),
        ("hidden_max", _F3),
        ("hidden_size", _F3),
        ("voxel_size", _F3),
        ("wall_min", _F3),
        ("wall_size", _F3),
        ("wall_normal", _F3),
        ("voxel_res", _U3),
    ]


assert ctypes.sizeof(ReconInfo) == 148


class LctParams(ctypes.Structure):
    _fields_ = [
        ("width", c_float),
        ("bin_length", c_float),
        ("snr", c_float),
        ("diffuse", c_int),
        ("grid_mode", c_int),
        ("output", c_int),
    ]


FBP_LCT_GRID_REFERENCE, FBP_LCT_GRID_DEPTH = 0, 1
FBP_LCT_OUTPUT_CLAMPED_REAL, FBP_LCT_OUTPUT_MAGNITUDE = 0, 1


class MisParams(ctypes.Structure):
    _fields_ = [
        ("proposal", c_int),
        ("samples", c_uint32),
        ("seed", c_uint64),
        ("noise", c_void_p),
        ("noise_size", c_uint64),
        ("tile_cluster_cdf", c_void_p),
        ("cluster_side", c_uint32),
        ("scan_side", c_uint32),
        ("cv_side", c_uint32),
    ]


FBP_MIS_UNIFORM, FBP_MIS_SPATIAL, FBP_MIS_LEARNED, FBP_MIS_REFERENCE, FBP_MIS_REFERENCE_SCATTER = 0, 1, 2, 3, 4
FBP_MLP_FEATURES = 20


class ShapeParams(ctypes.Structure):
    _fields_ = [
        ("use_fourier_filter", c_int),
        ("postfilter", c_int),
        ("kernel_size", c_int),
        ("sigma", c_float),
        ("normalize", c_int),
    ]


class CaptureDesc(ctypes.Structure):
    """fbp_capture_desc: one capture of a batch."""

    _fields_ = [
        ("info", ReconInfo),
        ("cube", c_void_p),
        ("dtype", c_int),
        ("layout", c_int),
        ("laser_xyz", c_void_p),
        ("volume", c_void_p),
    ]


# (name, restype, argtypes) for every symbol include/fbp.h declares.
SIGNATURES = {
    "fbp_version": (c_char_p, []),
    "fbp_last_error": (c_char_p, []),
    "fbp_create": (c_int, [POINTER(c_void_p), c_int]),
    "fbp_destroy": (c_int, [c_void_p]),
    "fbp_check_device_status": (c_int, [c_void_p, c_void_p]),
    "fbp_kernel_launch_count": (c_uint64, [c_void_p]),
    "fbp_set_weight_mode": (c_int, [c_void_p, c_int]),
    "fbp_get_weight_mode": (c_int, [c_void_p, POINTER(c_int)]),
    "fbp_backproject_confocal": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_int, c_int, c_void_p, c_void_p,
                                         c_void_p]),
    "fbp_backproject_exhaustive": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_int, c_void_p, c_void_p,
                                           c_void_p, c_void_p]),
    "fbp_backproject_depths": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_int, c_int, c_void_p, c_void_p,
                                       c_void_p, c_uint32, c_void_p, c_void_p]),
    "fbp_debug_confocal_bins": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_void_p, c_uint64, c_void_p,
                                        c_void_p]),
    "fbp_debug_exhaustive_bins": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_void_p, c_void_p, c_uint64,
                                          c_void_p, c_void_p]),
    "fbp_debug_confocal_paths": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_void_p, c_uint64, c_void_p,
                                         c_void_p, c_void_p]),
    "fbp_linear_space": (c_int, [c_double, c_double, c_int, POINTER(c_double)]),
    "fbp_postfilter": (c_int, [c_void_p, c_int, c_int, c_float, c_void_p, c_void_p, c_uint32, c_uint32, c_uint32,
                               c_void_p]),
    "fbp_log_weights": (c_int, [c_int, c_float, POINTER(c_float)]),
    "fbp_normalize_minmax": (c_int, [c_void_p, c_void_p, c_uint64, c_void_p]),
    "fbp_normalize_minmax_noalloc": (c_int, [c_void_p, c_uint64, c_void_p]),
    "fbp_filter_h": (c_int, [c_void_p, c_void_p, c_uint64, c_uint32, c_float, c_float, c_float, c_int, c_void_p]),
    "fbp_mis_backproject": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_int, c_int, c_void_p,
                                    POINTER(MisParams), c_void_p, c_void_p]),
    "fbp_mis_reference_tables": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_int, c_int, c_void_p, c_void_p,
                                         c_void_p, c_void_p]),
    "fbp_mis_tile_grid": (c_int, [POINTER(ReconInfo), POINTER(c_uint32)]),
    "fbp_lct": (c_int, [c_void_p, c_void_p, c_int, c_uint32, c_uint32, POINTER(LctParams), c_void_p, c_void_p]),
    "fbp_backproject_confocal_scatter": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_int, c_int, c_void_p,
                                                 c_void_p, c_void_p]),
    "fbp_splat_backproject": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_int, c_int, c_void_p, c_uint32,
                                      c_uint32, c_uint32, c_void_p, c_void_p]),
    "fbp_transient_images": (c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, c_uint64, c_uint64, c_uint32,
                                     c_uint32, c_int, c_void_p, c_void_p]),
    "fbp_write_png": (c_int, [c_char_p, c_void_p, c_uint32, c_uint32]),
    "fbp_save_transient_images": (c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_uint32, c_uint64, c_uint64,
                                          c_uint32, c_uint32, c_int, c_char_p, c_void_p]),
    "fbp_plan_slabs": (c_int, [POINTER(ReconInfo), c_uint32, POINTER(c_uint32)]),
    "fbp_slab_bin_window": (c_int, [POINTER(ReconInfo), c_void_p, c_uint32, c_uint32, POINTER(c_uint32),
                                    POINTER(c_uint32)]),
    "fbp_backproject_confocal_slab": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_int, c_int, c_void_p,
                                              c_uint32, c_uint32, c_void_p, c_void_p]),
    "fbp_mlp_num_params": (c_uint32, []),
    "fbp_mlp_create": (c_int, [c_void_p, c_uint64, POINTER(c_void_p)]),
    "fbp_mlp_destroy": (c_int, [c_void_p]),
    "fbp_mlp_get_params": (c_int, [c_void_p, POINTER(c_float), c_uint32]),
    "fbp_mlp_set_params": (c_int, [c_void_p, POINTER(c_float), c_uint32]),
    "fbp_mlp_tile_count": (c_int, [POINTER(ReconInfo), POINTER(c_uint32)]),
    "fbp_mlp_features": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_int, c_int, c_void_p, c_uint32, c_uint32,
                                 c_void_p, c_uint32, c_void_p, c_void_p]),
    "fbp_mlp_labels": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_int, c_int, c_void_p, c_uint32, c_uint32,
                               c_void_p, c_uint32, c_void_p, c_void_p]),
    "fbp_mlp_forward": (c_int, [c_void_p, c_void_p, c_void_p, c_uint32, c_uint32, c_void_p, c_float, c_void_p,
                                c_void_p]),
    "fbp_mlp_gradients": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_uint32, c_void_p,
                                  c_void_p]),
    "fbp_mlp_train_step": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_uint32, c_float,
                                   c_void_p, c_void_p]),
    "fbp_batch_create": (c_int, [c_void_p, c_uint32, POINTER(CaptureDesc), POINTER(c_void_p)]),
    "fbp_batch_run": (c_int, [c_void_p, c_int, c_void_p]),
    "fbp_batch_autotune": (c_int, [c_void_p, c_void_p, POINTER(c_int)]),
    "fbp_batch_set_config": (c_int, [c_void_p, c_int, c_void_p]),
    "fbp_batch_destroy": (c_int, [c_void_p]),
    "fbp_reconstruct_shape_host": (c_int, [c_void_p, POINTER(ReconInfo), c_void_p, c_int, c_void_p, c_void_p,
                                           POINTER(ShapeParams), c_void_p, c_void_p]),
}

_lib = None


def load() -> ctypes.CDLL:
    """Load libfbp.so once and attach the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"libfbp.so not built ({LIB_PATH}); run __graft_entry__.build()")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class FbpError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"fbp status {status}: {msg}")
        self.status = status


def check(status: int) -> None:
    if status != FBP_OK:
        raise FbpError(status, load().fbp_last_error().decode())
