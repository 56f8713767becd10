"""The host-buffer entry point (Laser::reconstructShape) against the composed
device calls and against the oracle pipeline."""
import numpy as np
import pytest

from oracle import cpu, numpy_ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _case(seed=3):
    from fasterbackprojection_gb300 import make_info, scenes

    cap = scenes.confocal_points(12, 512, 32e-12, n_points=40, seed=seed)
    vres = (24, 20, 28)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 2.4))
    info = make_info(num_laser_targets=144, num_time_bins=512, time_step=cap.time_step, voxel_res=vres,
                     hidden_min=hmin, voxel_size=vs)
    return cap, info


@pytest.mark.parametrize("use_filter,post", [(False, 0), (True, 2), (True, 1)])
def test_host_entry_matches_device_composition(ctx, cuda, use_filter, post):
    import torch

    cap, info = _case()
    host = ctx.reconstruct_shape_host(info, cap.cube, cap.laser_xyz, use_fourier_filter=use_filter, postfilter=post)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    if use_filter:
        ctx.filter_h_(cube, info.time_step)
    vol = ctx.backproject_confocal(info, cube, lx)
    if post:
        vol = ctx.postfilter(post, vol, 5, 1.0)
    ctx.normalize_(vol)
    np.testing.assert_array_equal(host, vol.cpu().numpy())


def test_host_entry_vs_oracle_pipeline(ctx, cuda):
    import torch

    cap, info = _case(seed=5)
    host = ctx.reconstruct_shape_host(info, cap.cube, cap.laser_xyz, use_fourier_filter=True, postfilter=2)
    filt = numpy_ref.filter_h(cap.cube, info.time_step).astype(np.float32)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    V = 24 * 20 * 28
    bins = ctx.debug_confocal_bins(info, lx, torch.arange(V, device=cuda)).cpu().numpy()
    vol = cpu.confocal_voxel(info, filt, cap.laser_xyz, bins=bins)
    vol = cpu.log_filter(vol.astype(np.float32), cpu.log_weights(5, 1.0), 5)
    vol = cpu.normalize(vol)
    assert rel_l2(host, vol) < 1e-4


def test_host_entry_bf16_capture(ctx, cuda):
    from fasterbackprojection_gb300 import scenes

    cap, info = _case(seed=7)
    bits = scenes.to_bits_bf16(cap.cube)
    out = ctx.reconstruct_shape_host(info, bits, cap.laser_xyz, use_fourier_filter=False)
    out32 = ctx.reconstruct_shape_host(info, scenes.from_bits_bf16(bits), cap.laser_xyz, use_fourier_filter=False)
    assert rel_l2(out, out32) < 1e-6
