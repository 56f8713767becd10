"""Depth slabs on the GPU: each planned slab, computed from a cube holding only
its bin window, is bitwise the same rows of the full-volume gather."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nranks,discard", [(2, 1), (3, 1), (3, 0)])
def test_slabs_equal_rows_of_the_full_volume(ctx, cuda, nranks, discard):
    import torch

    from fasterbackprojection_gb300 import make_info, scenes, slabs

    cap = scenes.confocal_points(16, 512, 32e-12, n_points=40, seed=31)
    vres = (20, 24, 45)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 2.0))
    info = make_info(num_laser_targets=256, num_time_bins=512, time_step=cap.time_step, voxel_res=vres,
                     hidden_min=hmin, voxel_size=vs, discard_first_last_bounces=discard,
                     laser_position=(0.05, -0.25, 0.1), sensor_position=(-0.1, -0.2, 0.05))
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    full = ctx.backproject_confocal(info, torch.from_numpy(cap.cube).to(cuda), lx)
    saved = 0
    for r, (z0, z1) in enumerate(slabs.plan(info, nranks)):
        lo, hi = slabs.bin_window(info, cap.laser_xyz, z0, z1)
        saved += 512 - (hi - lo + 1)
        cube_r = torch.from_numpy(slabs.windowed_cube(cap.cube, lo, hi)).to(cuda)
        slab = ctx.backproject_confocal_slab(info, cube_r, lx, z0, z1)
        torch.cuda.synchronize()
        assert torch.equal(slab, full[z0:z1]), (r, z0, z1)
        # The same through the rank driver (host tensor, window upload).
        s2, (a, b), copied = slabs.reconstruct_rank(ctx, info, torch.from_numpy(cap.cube), cap.laser_xyz, r,
                                                    nranks, cuda)
        assert (a, b) == (z0, z1) and torch.equal(s2, full[z0:z1])
        assert copied == 256 * (hi - lo + 1) * 4
    ctx.check_device_status()
    assert saved > 0


def test_slab_rejects_bad_ranges(ctx, cuda):
    import torch

    from fasterbackprojection_gb300 import FbpError, make_info

    info = make_info(num_laser_targets=4, num_time_bins=16, time_step=0.01, voxel_res=(4, 4, 8),
                     hidden_min=(-1, -1, -1), voxel_size=(0.5, 0.1, 0.5))
    cube = torch.zeros((4, 16), device=cuda)
    lx = torch.zeros((4, 3), device=cuda)
    with pytest.raises(FbpError):
        ctx.backproject_confocal_slab(info, cube, lx, 4, 4)
    with pytest.raises(FbpError):
        ctx.backproject_confocal_slab(info, cube, lx, 0, 9)
