"""Transient images on the GPU (fbp_transient_images) against the oracle's
TransientImage::save restatement (oracle/numpy_ref.py, itself pinned to the
reference's Image.h): bit-exact RGBA8 pixels for the depth planes of a real
depth-plane reconstruction and for contiguous slices, and the PNG files."""

import numpy as np
import pytest

from oracle import numpy_ref

pytestmark = pytest.mark.gpu


def _activation(ctx, cuda, n=16, D=24):
    """Normalised depth-plane activation [n*n][D], as Laser::reconstructDepthConfocal makes it."""
    import torch
    from fasterbackprojection_gb300 import make_info, scenes
    from fasterbackprojection_gb300.api import linear_space

    cap = scenes.confocal_points(n, 512, 32e-12, n_points=30, seed=43)
    info = make_info(num_laser_targets=n * n, num_time_bins=512, time_step=cap.time_step, voxel_res=(1, 1, 1),
                     hidden_min=(0, 0, 0), voxel_size=(1, 1, 1))
    depths = torch.from_numpy(linear_space(0.6, 1.0, D)).to(cuda)
    act = ctx.backproject_depths(info, torch.from_numpy(cap.cube).to(cuda), torch.from_numpy(cap.laser_xyz).to(cuda),
                                 depths)
    ctx.normalize_(act)
    return act


@pytest.mark.parametrize("size", [(256, 256), (64, 64), (16, 16), (37, 23)])
def test_depth_plane_images_match_oracle(ctx, cuda, size):
    act = _activation(ctx, cuda)
    imgs = ctx.depth_plane_images(act, 16, 16, size=size).cpu().numpy()
    ctx.check_device_status()
    a = act.cpu().numpy().ravel()
    D = act.shape[1]
    assert imgs.shape == (D, size[1], size[0], 4)
    for d in range(D):
        np.testing.assert_array_equal(imgs[d], numpy_ref.transient_image(a, 16, 16, size, stride=D, offset=d))
    assert imgs[..., 0].max() > 0


def test_contiguous_slices_with_normalisation_match_oracle(ctx, cuda):
    """NLosData::saveImages: one normalised image per contiguous slice."""
    import torch

    rng = np.random.default_rng(8)
    data = (rng.random((5, 12, 40), dtype=np.float32) * 3).astype(np.float32)
    data[2] = 0.0  # an all-zero plane: max 0, every pixel 0 / 0 -> 0
    data[3, 0, :] = -1.0
    imgs = ctx.transient_images(torch.from_numpy(data).to(cuda), 12, 40, 5, 1, 12 * 40, normalize=True).cpu().numpy()
    for p in range(5):
        np.testing.assert_array_equal(imgs[p], numpy_ref.transient_image(data[p].ravel(), 12, 40, (12, 40),
                                                                         normalize=True))
    assert imgs[2, ..., :3].max() == 0


def test_saved_png_files_hold_the_images(ctx, cuda, tmp_path):
    act = _activation(ctx, cuda, D=6)
    prefix = str(tmp_path) + "/"
    ctx.save_depth_planes(act, 16, 16, prefix, size=(64, 64))
    imgs = ctx.depth_plane_images(act, 16, 16, size=(64, 64)).cpu().numpy()
    from tests.test_images_cpu import _decode_png

    for d in range(6):
        data = (tmp_path / f"transient_{d}.png").read_bytes()
        np.testing.assert_array_equal(_decode_png(data), imgs[d])


def test_bad_arguments_are_rejected(ctx, cuda):
    import torch
    from fasterbackprojection_gb300 import FbpError

    act = torch.zeros((16, 4), device=cuda)
    with pytest.raises(FbpError):
        ctx.depth_plane_images(act, 4, 4, size=(1, 8))  # a resized image needs 2 x 2
    with pytest.raises(FbpError):
        ctx.transient_images(act, 0, 4, 4, 4, 1)
