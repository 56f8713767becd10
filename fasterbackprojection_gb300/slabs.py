"""Depth-slab partition of one confocal capture across ranks (host side of
fbp_plan_slabs / fbp_slab_bin_window / fbp_backproject_confocal_slab).

Each rank reconstructs a contiguous range of depth slices; voxels are
independent, so there is no collective on the data path.  A rank copies to
its GPU only the time bins its slab can reach; the slabs are gathered to
rank 0 afterwards (torch.distributed, any backend).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import ReconInfo, check, load


def plan(info: ReconInfo, nranks: int) -> list[tuple[int, int]]:
    b = (ctypes.c_uint32 * (nranks + 1))()
    check(load().fbp_plan_slabs(ctypes.byref(info), nranks, b))
    return [(int(b[r]), int(b[r + 1])) for r in range(nranks)]


def bin_window(info: ReconInfo, laser_xyz: np.ndarray, z_begin: int, z_end: int) -> tuple[int, int]:
    """Bins [lo, hi] the slab can reach (lo > hi: none)."""
    lx = np.ascontiguousarray(laser_xyz, dtype=np.float32)
    lo, hi = ctypes.c_uint32(), ctypes.c_uint32()
    check(load().fbp_slab_bin_window(ctypes.byref(info), ctypes.c_void_p(lx.ctypes.data), z_begin, z_end,
                                     ctypes.byref(lo), ctypes.byref(hi)))
    return int(lo.value), int(hi.value)


def windowed_cube(cube_host: np.ndarray, lo: int, hi: int) -> np.ndarray:
    """The capture [L][T] with only bins [lo, hi] kept (what a rank uploads)."""
    out = np.zeros_like(cube_host)
    if lo <= hi:
        out[:, lo:hi + 1] = cube_host[:, lo:hi + 1]
    return out


def reconstruct_rank(ctx, info: ReconInfo, cube_host, laser_xyz_host, rank: int, nranks: int, device):
    """This rank's slab on its GPU: uploads bins [lo, hi] of cube_host [L][T]
    (a pinned or pageable torch CPU tensor) into a zeroed device cube and
    runs the slab gather.  Returns (slab tensor, (z_begin, z_end), bytes copied)."""
    import torch

    z0, z1 = plan(info, nranks)[rank]
    vx, vy, _ = info.voxel_res
    if z0 >= z1:
        return torch.empty((0, vy, vx), dtype=torch.float32, device=device), (z0, z1), 0
    lo, hi = bin_window(info, laser_xyz_host.numpy() if hasattr(laser_xyz_host, "numpy") else laser_xyz_host, z0, z1)
    cube = torch.zeros(tuple(cube_host.shape), dtype=cube_host.dtype, device=device)
    copied = 0
    if lo <= hi:
        cube[:, lo:hi + 1].copy_(cube_host[:, lo:hi + 1], non_blocking=True)
        copied = cube_host.shape[0] * (hi - lo + 1) * cube_host.element_size()
    lx = torch.as_tensor(laser_xyz_host).to(device)
    slab = ctx.backproject_confocal_slab(info, cube, lx, z0, z1)
    return slab, (z0, z1), copied


def gather_to_rank0(slab, info: ReconInfo, nranks: int, rank: int):
    """Full [Vz][Vy][Vx] volume on rank 0 (None elsewhere) from every rank's
    slab (all ranks the same dtype), through torch.distributed point-to-point
    sends."""
    import torch
    import torch.distributed as dist

    bounds = plan(info, nranks)
    vx, vy, vz = info.voxel_res
    if rank != 0:
        if slab.numel():
            dist.send(slab.contiguous(), dst=0)
        return None
    full = torch.empty((vz, vy, vx), dtype=slab.dtype, device=slab.device)
    z0, z1 = bounds[0]
    full[z0:z1] = slab
    for r in range(1, nranks):
        a, b = bounds[r]
        if b > a:
            buf = torch.empty((b - a, vy, vx), dtype=slab.dtype, device=slab.device)
            dist.recv(buf, src=r)
            full[a:b] = buf
    return full
