"""ctypes binding of oracle/_build/liboracle.so (FP64 C restatement).

TEST INFRASTRUCTURE ONLY — see oracle/__init__.py.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_float, c_int, c_int32, c_int64, c_uint32, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_F3 = c_float * 3
_U3 = c_uint32 * 3


class OracleInfo(ctypes.Structure):
    _fields_ = [
        ("sensor_position", _F3), ("capture_system", c_uint32), ("laser_position", _F3), ("time_offset", c_float),
        ("num_laser_targets", c_uint32), ("num_sensor_targets", c_uint32), ("num_time_bins", c_uint32),
        ("time_step", c_float), ("hidden_min", _F3), ("discard_first_last_bounces", c_uint32), ("hidden_max", _F3),
        ("hidden_size", _F3), ("voxel_size", _F3), ("wall_min", _F3), ("wall_size", _F3), ("wall_normal", _F3),
        ("voxel_res", _U3),
    ]


LAYOUT_TIME_MAJOR, LAYOUT_TIME_INNER = 0, 1
BINS_F64, BINS_GIVEN = 0, 1

_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise ImportError(f"{LIB} not built: run `make -C oracle`")
        _lib = ctypes.CDLL(str(LIB))
        assert _lib.oracle_info_size() == ctypes.sizeof(OracleInfo) == 148
    return _lib


def to_oracle_info(info) -> OracleInfo:
    """Copy any ctypes structure with the same 148-byte layout."""
    o = OracleInfo()
    ctypes.memmove(ctypes.byref(o), ctypes.byref(info), 148)
    return o


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _p(a):
    return a.ctypes.data_as(c_void_p)


def confocal_voxel(info, cube, laser_xyz, layout=LAYOUT_TIME_INNER, bins=None) -> np.ndarray:
    """FP64 volume [Vz][Vy][Vx] of backprojectConfocalVoxel."""
    lib = load()
    o = to_oracle_info(info)
    vx, vy, vz = o.voxel_res
    vol = np.empty((vz, vy, vx), dtype=np.float64)
    cube = _f32(cube)
    lx = _f32(laser_xyz)
    mode = BINS_F64 if bins is None else BINS_GIVEN
    b = None if bins is None else np.ascontiguousarray(bins, dtype=np.int32)
    rc = lib.oracle_confocal_voxel(ctypes.byref(o), _p(cube), c_int(layout), _p(lx), c_int(mode),
                                   None if b is None else _p(b), _p(vol))
    assert rc == 0
    return vol


def confocal_scatter_voxel(info, cube, laser_xyz, layout=LAYOUT_TIME_INNER) -> np.ndarray:
    """FP64 volume [Vz][Vy][Vx] of the ACCUMULATE_VOXEL_SCATTERING build."""
    lib = load()
    o = to_oracle_info(info)
    vx, vy, vz = o.voxel_res
    vol = np.empty((vz, vy, vx), dtype=np.float64)
    rc = lib.oracle_confocal_scatter_voxel(ctypes.byref(o), _p(_f32(cube)), c_int(layout), _p(_f32(laser_xyz)),
                                           _p(vol))
    assert rc == 0, rc
    return vol


def confocal_voxel_subset(info, cube, laser_xyz, idx, layout=LAYOUT_TIME_INNER, bins=None) -> np.ndarray:
    """FP64 values of the voxels idx; bins (len(idx) x L int32), when given,
    replace the FP64 bin computation."""
    lib = load()
    o = to_oracle_info(info)
    cube = _f32(cube)
    lx = _f32(laser_xyz)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.empty(idx.shape[0], dtype=np.float64)
    if bins is None:
        assert lib.oracle_confocal_voxel_subset(ctypes.byref(o), _p(cube), c_int(layout), _p(lx), _p(idx),
                                                c_int64(idx.shape[0]), _p(out)) == 0
    else:
        b = np.ascontiguousarray(bins, dtype=np.int32).reshape(idx.shape[0], o.num_laser_targets)
        assert lib.oracle_confocal_voxel_subset_bins(ctypes.byref(o), _p(cube), c_int(layout), _p(lx), _p(idx),
                                                     c_int64(idx.shape[0]), _p(b), _p(out)) == 0
    return out


def confocal_voxel_f32_subset(info, cube, laser_xyz, idx, layout=LAYOUT_TIME_INNER, threads=0) -> np.ndarray:
    """The FP32 restatement used as the timed CPU baseline."""
    lib = load()
    o = to_oracle_info(info)
    cube = _f32(cube)
    lx = _f32(laser_xyz)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.empty(idx.shape[0], dtype=np.float32)
    assert lib.oracle_confocal_voxel_f32_subset(ctypes.byref(o), _p(cube), c_int(layout), _p(lx), _p(idx),
                                                c_int64(idx.shape[0]), _p(out), c_int(threads)) == 0
    return out


def exhaustive_voxel(info, cube, laser_xyz, sensor_xyz, bins=None) -> np.ndarray:
    lib = load()
    o = to_oracle_info(info)
    vx, vy, vz = o.voxel_res
    vol = np.empty((vz, vy, vx), dtype=np.float64)
    cube = _f32(cube)
    mode = BINS_F64 if bins is None else BINS_GIVEN
    b = None if bins is None else np.ascontiguousarray(bins, dtype=np.int32)
    assert lib.oracle_exhaustive_voxel(ctypes.byref(o), _p(cube), _p(_f32(laser_xyz)), _p(_f32(sensor_xyz)),
                                       c_int(mode), None if b is None else _p(b), _p(vol)) == 0
    return vol


def exhaustive_voxel_subset(info, cube, laser_xyz, sensor_xyz, idx, bins=None) -> np.ndarray:
    """Voxels idx of the exhaustive volume; bins (optional) are the GPU's,
    bins[(i*L + l)*S + s] for voxel idx[i] (fbp_debug_exhaustive_bins' order)."""
    lib = load()
    o = to_oracle_info(info)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.empty(idx.shape[0], dtype=np.float64)
    b = None
    if bins is not None:
        b = np.ascontiguousarray(bins, dtype=np.int32)
        assert b.size == idx.shape[0] * o.num_laser_targets * o.num_sensor_targets
    assert lib.oracle_exhaustive_voxel_subset_bins(ctypes.byref(o), _p(_f32(cube)), _p(_f32(laser_xyz)),
                                                   _p(_f32(sensor_xyz)), _p(idx), c_int64(idx.shape[0]),
                                                   None if b is None else _p(b), _p(out)) == 0
    return out


def depth_confocal(info, cube, laser_xyz, depths, layout=LAYOUT_TIME_INNER) -> np.ndarray:
    lib = load()
    o = to_oracle_info(info)
    depths = np.ascontiguousarray(depths, dtype=np.float64)
    out = np.empty((o.num_laser_targets, depths.shape[0]), dtype=np.float64)
    assert lib.oracle_depth_confocal(ctypes.byref(o), _p(_f32(cube)), c_int(layout), _p(_f32(laser_xyz)),
                                     _p(depths), c_uint32(depths.shape[0]), _p(out)) == 0
    return out


def depth_exhaustive(info, cube, laser_xyz, sensor_xyz, depths) -> np.ndarray:
    lib = load()
    o = to_oracle_info(info)
    depths = np.ascontiguousarray(depths, dtype=np.float64)
    out = np.empty((o.num_laser_targets, depths.shape[0]), dtype=np.float64)
    assert lib.oracle_depth_exhaustive(ctypes.byref(o), _p(_f32(cube)), _p(_f32(laser_xyz)), _p(_f32(sensor_xyz)),
                                       _p(depths), c_uint32(depths.shape[0]), _p(out)) == 0
    return out


def log_weights(size: int, sigma: float) -> np.ndarray:
    w = np.empty(size ** 3, dtype=np.float32)
    assert load().oracle_log_weights(c_int(size), c_float(sigma), _p(w)) == 0
    return w


def log_filter(vol, w, size) -> np.ndarray:
    vol = _f32(vol)
    nz, ny, nx = vol.shape
    out = np.empty(vol.shape, dtype=np.float64)
    assert load().oracle_log_filter(_p(vol), _p(out), c_uint32(nx), c_uint32(ny), c_uint32(nz), _p(_f32(w)),
                                    c_int(size)) == 0
    return out


def laplacian_filter(vol, size) -> np.ndarray:
    vol = _f32(vol)
    nz, ny, nx = vol.shape
    out = np.empty(vol.shape, dtype=np.float64)
    assert load().oracle_laplacian_filter(_p(vol), _p(out), c_uint32(nx), c_uint32(ny), c_uint32(nz),
                                          c_int(size)) == 0
    return out


def normalize(v) -> np.ndarray:
    out = np.array(v, dtype=np.float64, copy=True)
    assert load().oracle_normalize(_p(out), c_int64(out.size)) == 0
    return out


def build_alias(cdf):
    cdf = _f32(cdf)
    n = cdf.shape[0]
    alias = np.zeros(n, dtype=np.uint32)
    prob = np.zeros(n, dtype=np.float32)
    rc = load().oracle_build_alias(_p(cdf), c_uint32(n), _p(alias), _p(prob))
    return rc, alias, prob
