"""Depth-slab partition across ranks, without a GPU: the planner covers the
volume once, the bin window is conservative, and a world_size-2 gloo run of
the FP64 oracle on windowed cubes gathers to the full oracle volume exactly."""
import os
import socket

import numpy as np
import pytest

from oracle import cpu


def _case(n=8, T=256, vres=(10, 12, 40), seed=5, discard=1):
    from fasterbackprojection_gb300 import make_info, scenes

    cap = scenes.confocal_points(n, T, 32e-12, n_points=30, seed=seed)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 1.6))
    info = make_info(num_laser_targets=n * n, num_time_bins=T, time_step=cap.time_step, voxel_res=vres,
                     hidden_min=hmin, voxel_size=vs, discard_first_last_bounces=discard,
                     laser_position=(0.05, -0.25, 0.1), sensor_position=(-0.1, -0.2, 0.05))
    return cap, info


@pytest.mark.parametrize("vz,nranks", [(40, 2), (40, 3), (16, 4), (257, 5), (7, 2)])
def test_plan_covers_the_volume_once(built, vz, nranks):
    from fasterbackprojection_gb300 import slabs

    _, info = _case(vres=(4, 4, vz))
    b = slabs.plan(info, nranks)
    assert b[0][0] == 0 and b[-1][1] == vz
    for (a0, a1), (c0, c1) in zip(b, b[1:]):
        assert a1 == c0
    for z0, z1 in b:
        assert z0 <= z1 and (z0 % 16 == 0 or z0 == vz)
    sizes = [z1 - z0 for z0, z1 in b]
    assert max(sizes) - min(sizes) <= 16


@pytest.mark.parametrize("discard", [1, 0])
def test_bin_window_contains_every_reachable_bin(built, discard):
    from fasterbackprojection_gb300 import slabs

    cap, info = _case(discard=discard)
    Vx, Vy, Vz = info.voxel_res
    L, T = info.num_laser_targets, info.num_time_bins
    lx = cap.laser_xyz.astype(np.float64)
    lp = np.array(info.laser_position[:], dtype=np.float64)
    sp = np.array(info.sensor_position[:], dtype=np.float64)
    for z0, z1 in slabs.plan(info, 3):
        lo, hi = slabs.bin_window(info, cap.laser_xyz, z0, z1)
        vz, vy, vx = np.meshgrid(np.arange(z0, z1), np.arange(Vy), np.arange(Vx), indexing="ij")
        p = np.stack([info.hidden_min[0] + (vx.ravel() + 0.5) * info.voxel_size[0],
                      info.hidden_min[1] + (vz.ravel() + 0.5) * info.voxel_size[1],
                      info.hidden_min[2] + (vy.ravel() + 0.5) * info.voxel_size[2]], 1)
        d = 2 * np.linalg.norm(p[:, None, :] - lx[None], axis=2) - info.time_offset
        if discard == 0:
            d = d + (np.linalg.norm(lx - lp, axis=1) + np.linalg.norm(lx - sp, axis=1))[None]
        b = np.floor(d / info.time_step)
        b = b[(b >= 0) & (b < T)]
        assert b.size == 0 or (lo <= b.min() and b.max() <= hi)
        assert hi - lo + 1 < T  # the window is a real saving for a slab


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    import torch
    import torch.distributed as dist

    from fasterbackprojection_gb300 import slabs

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cap, info = _case()
    Vx, Vy, Vz = info.voxel_res
    z0, z1 = slabs.plan(info, world)[rank]
    lo, hi = slabs.bin_window(info, cap.laser_xyz, z0, z1)
    cube = slabs.windowed_cube(cap.cube, lo, hi)  # what this rank would upload
    idx = np.arange(z0 * Vx * Vy, z1 * Vx * Vy, dtype=np.int64)
    slab = torch.from_numpy(cpu.confocal_voxel_subset(info, cube, cap.laser_xyz, idx).reshape(z1 - z0, Vy, Vx))
    full = slabs.gather_to_rank0(slab, info, world, rank)
    if rank == 0:
        np.save(out_path, full.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_the_full_volume(built, tmp_path):
    import torch.multiprocessing as mp

    out = str(tmp_path / "full.npy")
    mp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    cap, info = _case()
    want = cpu.confocal_voxel(info, cap.cube, cap.laser_xyz)
    np.testing.assert_array_equal(np.load(out), want)
