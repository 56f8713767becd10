"""The reference's own CUDA kernels, compiled from its sources (oracle/_ref).

TEST INFRASTRUCTURE ONLY — see oracle/__init__.py.  Used by the GPU parity
tests as the bit-exact time-bin source and by bench.py to time the reference
kernels on the same GPU.  Needs oracle/_build/libref_loader.so (built by
`make -C oracle`, on any machine) and oracle/_ref/ref_kernels.cubin (built by
`make -C oracle ref` where the reference sources are present).
"""
from __future__ import annotations

import ctypes
from ctypes import c_char_p, c_float, c_int, c_size_t, c_uint, c_void_p
from pathlib import Path

HERE = Path(__file__).resolve().parent
LOADER = HERE / "_build" / "libref_loader.so"
CUBIN = HERE / "_ref" / "ref_kernels.cubin"
CUBIN_SCATTER = HERE / "_ref" / "ref_kernels_scatter.cubin"  # ACCUMULATE_VOXEL_SCATTERING build

_lib = None


def available() -> bool:
    return LOADER.exists() and CUBIN.exists()


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not available():
        raise ImportError("reference kernel harness not built (oracle/_build/libref_loader.so, oracle/_ref/ref_kernels.cubin)")
    lib = ctypes.CDLL(str(LOADER))
    lib.refk_last_error.restype = c_char_p
    for name in ["refk_load", "refk_set_state", "refk_set_mis_state", "refk_confocal_voxel", "refk_exhaustive_voxel",
                 "refk_depth_confocal", "refk_depth_exhaustive", "refk_confocal_voxel_mis", "refk_log_filter",
                 "refk_laplacian_filter", "refk_normalize"]:
        getattr(lib, name).restype = c_int
    lib.refk_load.argtypes = [c_char_p]
    lib.refk_load_variant.argtypes = [c_char_p]
    lib.refk_load_variant.restype = c_int
    lib.refk_select.argtypes = [c_int]
    lib.refk_select.restype = c_int
    lib.refk_set_state.argtypes = [c_void_p, c_size_t, c_void_p, c_void_p, c_void_p]
    lib.refk_set_mis_state.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p]
    lib.refk_confocal_voxel.argtypes = [c_void_p, c_uint, c_uint, c_uint, c_uint, c_void_p]
    lib.refk_exhaustive_voxel.argtypes = [c_void_p, c_uint, c_uint, c_uint, c_uint, c_uint, c_void_p]
    lib.refk_depth_confocal.argtypes = [c_void_p, c_void_p, c_uint, c_uint, c_void_p]
    lib.refk_depth_exhaustive.argtypes = [c_void_p, c_void_p, c_uint, c_uint, c_uint, c_void_p]
    lib.refk_confocal_voxel_mis.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_uint, c_uint, c_uint,
                                            c_uint, c_uint, c_void_p]
    lib.refk_log_filter.argtypes = [c_void_p, c_void_p, c_uint, c_uint, c_uint, c_void_p, c_int, c_void_p]
    lib.refk_laplacian_filter.argtypes = [c_void_p, c_void_p, c_uint, c_uint, c_uint, c_float, c_void_p]
    lib.refk_normalize.argtypes = [c_void_p, c_uint, c_void_p, c_void_p, c_void_p]
    if lib.refk_load(str(CUBIN).encode()) != 0:
        raise RuntimeError("refk_load: " + lib.refk_last_error().decode())
    _lib = lib
    return lib


def _chk(rc):
    if rc != 0:
        raise RuntimeError("reference harness: " + _lib.refk_last_error().decode())


def _ptr(t):
    return c_void_p(0 if t is None else t.data_ptr())


def _stream():
    import torch

    return c_void_p(torch.cuda.current_stream().cuda_stream)


def set_state(info, laser_xyz, sensor_xyz, cube):
    """cudaMemcpyToSymbol of rtRecInfo/laserTargets/sensorTargets/intensityCube (Laser.cu:52-55)."""
    lib = load()
    _chk(lib.refk_set_state(ctypes.byref(info), ctypes.sizeof(info), _ptr(laser_xyz), _ptr(sensor_xyz), _ptr(cube)))


def confocal_voxel(info, cube_time_major, laser_xyz):
    """backprojectConfocalVoxel into a zeroed volume; cube is cube[t*L + l] (float32)."""
    import torch

    lib = load()
    vx, vy, vz = info.voxel_res
    vol = torch.zeros((vz, vy, vx), dtype=torch.float32, device=cube_time_major.device)
    set_state(info, laser_xyz, laser_xyz, cube_time_major)
    _chk(lib.refk_confocal_voxel(_ptr(vol), vx, vy, vz, info.num_laser_targets, _stream()))
    return vol


def exhaustive_voxel(info, cube, laser_xyz, sensor_xyz):
    import torch

    lib = load()
    vx, vy, vz = info.voxel_res
    vol = torch.zeros((vz, vy, vx), dtype=torch.float32, device=cube.device)
    set_state(info, laser_xyz, sensor_xyz, cube)
    _chk(lib.refk_exhaustive_voxel(_ptr(vol), vx, vy, vz, info.num_laser_targets, info.num_sensor_targets, _stream()))
    return vol


def depth_confocal(info, cube_time_major, laser_xyz, depths):
    import torch

    lib = load()
    D = depths.numel()
    act = torch.zeros((info.num_laser_targets, D), dtype=torch.float32, device=cube_time_major.device)
    set_state(info, laser_xyz, laser_xyz, cube_time_major)
    _chk(lib.refk_depth_confocal(_ptr(act), _ptr(depths), D, info.num_laser_targets, _stream()))
    return act


def depth_exhaustive(info, cube, laser_xyz, sensor_xyz, depths):
    import torch

    lib = load()
    D = depths.numel()
    act = torch.zeros((info.num_laser_targets, D), dtype=torch.float32, device=cube.device)
    set_state(info, laser_xyz, sensor_xyz, cube)
    _chk(lib.refk_depth_exhaustive(_ptr(act), _ptr(depths), D, info.num_laser_targets, info.num_sensor_targets,
                                   _stream()))
    return act


def log_filter(vol, weights, ksize):
    import torch

    lib = load()
    nz, ny, nx = vol.shape
    out = torch.zeros_like(vol)
    _chk(lib.refk_log_filter(_ptr(vol), _ptr(out), nx, ny, nz, _ptr(weights), ksize, _stream()))
    return out


def laplacian_filter(vol, ksize):
    import torch

    lib = load()
    nz, ny, nx = vol.shape
    out = torch.zeros_like(vol)
    _chk(lib.refk_laplacian_filter(_ptr(vol), _ptr(out), nx, ny, nz, float(ksize), _stream()))
    return out


def normalize_(v):
    """normalizeReconstruction with min/max from torch (the reference uses CUB)."""
    import torch

    lib = load()
    mm = torch.stack([v.max(), v.min()]).contiguous()
    _chk(lib.refk_normalize(_ptr(v), v.numel(), _ptr(mm[0:1]), _ptr(mm[1:2]), _stream()))
    return v


def confocal_voxel_mis(info, cube_time_major, laser_xyz, spatial_sum, noise, alias, prob, num_samples):
    import torch

    lib = load()
    vx, vy, vz = info.voxel_res
    vol = torch.zeros((vz, vy, vx), dtype=torch.float32, device=cube_time_major.device)
    set_state(info, laser_xyz, laser_xyz, cube_time_major)
    _chk(lib.refk_set_mis_state(_ptr(noise), _ptr(spatial_sum), _ptr(alias), _ptr(prob)))
    _chk(lib.refk_confocal_voxel_mis(_ptr(spatial_sum), _ptr(vol), _ptr(noise), _ptr(alias), _ptr(prob), vx, vy, vz,
                                     num_samples, noise.numel(), _stream()))
    return vol


def scatter_available() -> bool:
    return available() and CUBIN_SCATTER.exists()


def confocal_voxel_scatter(info, cube_time_major, laser_xyz):
    """backprojectConfocalVoxel of the ACCUMULATE_VOXEL_SCATTERING build."""
    lib = load()
    _chk(lib.refk_load_variant(str(CUBIN_SCATTER).encode()))
    _chk(lib.refk_select(1))
    try:
        return confocal_voxel(info, cube_time_major, laser_xyz)
    finally:
        _chk(lib.refk_select(0))


def confocal_voxel_mis_scatter(info, cube_time_major, laser_xyz, spatial_sum, noise, alias, prob, num_samples):
    """backprojectConfocalVoxelMIS of the ACCUMULATE_VOXEL_SCATTERING build
    (transient_reconstruction.cuh:235-250; atomic adds per bin)."""
    lib = load()
    _chk(lib.refk_load_variant(str(CUBIN_SCATTER).encode()))
    _chk(lib.refk_select(1))
    try:
        return confocal_voxel_mis(info, cube_time_major, laser_xyz, spatial_sum, noise, alias, prob, num_samples)
    finally:
        _chk(lib.refk_select(0))
