"""Scatter-form (rasterised ellipsoid) backprojection against its float32
NumPy restatement (oracle/numpy_ref.py): the same fragments land in the same
voxels (identical IEEE float32 index arithmetic), so the sets of touched
voxels are equal; the sums differ by FP32 atomic accumulation against the
oracle's FP64 sums (rel-L2 < 1e-5)."""
import numpy as np
import pytest

from oracle import numpy_ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _case(n=8, T=320, vres=(24, 20, 16), seed=41, t0=0.0):
    from fasterbackprojection_gb300 import make_info, scenes

    cap = scenes.confocal_points(n, T, 32e-12, n_points=30, seed=seed, noise=False)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 1.6))
    info = make_info(num_laser_targets=n * n, num_time_bins=T, time_step=cap.time_step, voxel_res=vres,
                     hidden_min=hmin, voxel_size=vs, time_offset=t0)
    return cap, info


@pytest.mark.parametrize("max_bins,grid,t0", [(0, (32, 32), 0.0), (120, (48, 40), 0.0), (0, (32, 32), 0.1)])
def test_splat_matches_oracle(ctx, cuda, max_bins, grid, t0):
    import torch

    cap, info = _case(t0=t0)
    got = ctx.splat_backproject(info, torch.from_numpy(cap.cube).to(cuda), torch.from_numpy(cap.laser_xyz).to(cuda),
                                max_bins=max_bins, grid=grid).cpu().numpy()
    ctx.check_device_status()
    want = numpy_ref.splat_backproject(info, cap.cube, cap.laser_xyz, max_bins=max_bins, grid=grid)
    assert want.sum() > 0
    np.testing.assert_array_equal(got > 0, want > 0)
    assert rel_l2(got, want) < 1e-5


def test_splat_of_an_empty_capture_is_zero(ctx, cuda):
    import torch

    cap, info = _case()
    vol = ctx.splat_backproject(info, torch.zeros((64, 320), device=cuda), torch.from_numpy(cap.laser_xyz).to(cuda))
    assert float(vol.abs().sum()) == 0.0


def test_splat_time_major_layout_and_bf16(ctx, cuda):
    import torch

    cap, info = _case()
    c = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    a = ctx.splat_backproject(info, c, lx, grid=(32, 32))
    b = ctx.splat_backproject(info, c.t().contiguous(), lx, grid=(32, 32), layout=0)
    assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < 1e-5
    h = ctx.splat_backproject(info, c.to(torch.bfloat16), lx, grid=(32, 32))
    want = numpy_ref.splat_backproject(info, c.to(torch.bfloat16).float().cpu().numpy(), cap.laser_xyz,
                                       grid=(32, 32))
    assert rel_l2(h.cpu().numpy(), want) < 1e-5
