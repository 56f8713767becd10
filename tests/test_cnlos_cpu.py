"""The host steps of python/lct.py's cnlos_reconstruction (fasterbackprojection_gb300.cnlos)
against literal restatements of the lct.py lines, and the arguments it hands to the GPU LCT."""
import numpy as np
import pytest


def _lct_py_steps(rect_data, bin_resolution, K, z_trim, z_offset):
    """lct.py:93-129 as written there (c = 3e8)."""
    c = 3e8
    M = rect_data.shape[2]
    range_max = M * c * bin_resolution
    for _ in range(K):
        M = M // 2
        bin_resolution = 2 * bin_resolution
        rect_data = rect_data[:, :, 0::2] + rect_data[:, :, 1::2]
        z_trim = round(z_trim / 2)
        z_offset = round(z_offset / 2)
    rect_data[:, :, :z_trim] = 0
    data = np.transpose(rect_data, (2, 1, 0))
    return data, bin_resolution, range_max, z_trim, z_offset


@pytest.mark.parametrize("K,z_trim,z_offset", [(0, 5, 3), (1, 600 // 16, 350 // 16), (2, 37, 175)])
def test_prepare_matches_lct_py(K, z_trim, z_offset):
    from fasterbackprojection_gb300 import cnlos

    rng = np.random.default_rng(K)
    rect = rng.poisson(1.5, (8, 8, 256)).astype(np.float64)
    keep = rect.copy()
    s = cnlos.Settings(K=K, z_trim=z_trim, z_offset=z_offset)
    p = cnlos.prepare(rect, s)
    data, br, rmax, zt, zo = _lct_py_steps(rect.copy(), 4e-12, K, z_trim, z_offset)
    np.testing.assert_array_equal(rect, keep)  # the caller's array is left alone
    np.testing.assert_array_equal(p.data, data.astype(np.float32))
    assert p.data.flags.c_contiguous and p.data.dtype == np.float32 and p.data.shape == (256 >> K, 8, 8)
    assert (p.bin_resolution, p.range_max, p.z_trim, p.z_offset) == (br, rmax, zt, zo)
    assert p.bin_length == pytest.approx(3e8 * 4e-12 * 2 ** K)


def test_round_half_to_even_like_lct_py():
    from fasterbackprojection_gb300 import cnlos

    # 350 -> 175 -> round(87.5) = 88 (Python rounds halves to even), 600 -> 300 -> 150.
    p = cnlos.prepare(np.zeros((4, 4, 64)), cnlos.Settings(K=2, z_trim=600, z_offset=350))
    assert (p.z_trim, p.z_offset) == (150, 88)
    with pytest.raises(ValueError):
        cnlos.prepare(np.zeros((4, 4, 6)), cnlos.Settings(K=2))  # 6 -> 3 bins cannot halve again
    with pytest.raises(ValueError):
        cnlos.prepare(np.zeros((4, 5, 8)))


def test_scene_table():
    from fasterbackprojection_gb300 import cnlos

    f, s = cnlos.scene_settings(7)
    assert f == "lct/data_s_u.mat" and s.z_offset == 800 and not s.isdiffuse and s.snr == 0.8
    f, s = cnlos.scene_settings(9)
    assert f == "lct/data_diffuse_s.mat" and s.z_offset == 100 and s.isdiffuse and s.snr == pytest.approx(0.08)
    assert [cnlos.scene_settings(k)[1].z_offset for k in range(1, 10)] == [350, 700, 350, 700, 300, 600, 800, 700, 100]
    with pytest.raises(ValueError):
        cnlos.scene_settings(10)


def test_load_capture_round_trip(tmp_path):
    scipy_io = pytest.importorskip("scipy.io")
    from fasterbackprojection_gb300 import cnlos

    rect = np.arange(4 * 4 * 16, dtype=np.float64).reshape(4, 4, 16)
    scipy_io.savemat(tmp_path / "a.mat", {"rect_data": rect, "width": np.array([[0.25]])})
    got, width = cnlos.load_capture(tmp_path / "a.mat")
    np.testing.assert_array_equal(got, rect)
    assert width == 0.25
    scipy_io.savemat(tmp_path / "b.mat", {"rect_data": rect})
    assert cnlos.load_capture(tmp_path / "b.mat")[1] == 0.4  # lct.py's stand-in width
    scipy_io.savemat(tmp_path / "c.mat", {"other": rect})
    with pytest.raises(ValueError):
        cnlos.load_capture(tmp_path / "c.mat")


def test_display_crop_axes_and_views():
    import torch

    from fasterbackprojection_gb300 import cnlos

    p = cnlos.prepare(np.zeros((4, 4, 128)), cnlos.Settings(K=1, z_trim=0, z_offset=6))
    width = 0.3
    vol = np.random.default_rng(0).random((64, 4, 4))
    ind = round(64 * 2 * width / (p.range_max / 2))  # lct.py:227
    assert p.z_offset == 3  # 6 capture bins, halved once
    want = vol[:, :, ::-1][3:3 + ind]  # lct.py:230, 236
    np.testing.assert_array_equal(cnlos.display_crop(vol, p, width), want)
    np.testing.assert_array_equal(cnlos.display_crop(torch.from_numpy(vol), p, width).numpy(), want)
    tz, ty, tx = cnlos.axes(64, 4, p, width)
    np.testing.assert_array_equal(tz, np.linspace(0, p.range_max / 2, 64)[3:3 + ind])
    np.testing.assert_array_equal(ty, np.linspace(-width, width, 4))
    v = cnlos.views(want)
    np.testing.assert_array_equal(v["front"], want.max(0))
    np.testing.assert_array_equal(v["top"], want.max(1))
    np.testing.assert_array_equal(v["side"], want.max(2).T)


def test_reconstruct_hands_the_prepared_capture_to_the_lct():
    import torch

    from fasterbackprojection_gb300 import (FBP_LAYOUT_TIME_MAJOR, FBP_LCT_GRID_DEPTH, FBP_LCT_OUTPUT_CLAMPED_REAL,
                                            FBP_LCT_OUTPUT_MAGNITUDE, cnlos)

    class RecordingContext:
        device = 0

        def lct(self, data, width, bin_length, snr, diffuse, grid_mode, layout, stream, output):
            self.args = dict(data=data.clone(), width=width, bin_length=bin_length, snr=snr, diffuse=diffuse,
                             grid_mode=grid_mode, layout=layout, output=output)
            return torch.arange(data.numel(), dtype=torch.float32).reshape(data.shape)

    rect = np.random.default_rng(2).poisson(1.0, (8, 8, 64)).astype(np.float64)
    ctx = RecordingContext()
    _, s = cnlos.scene_settings(9, cnlos.Settings(K=1, z_trim=4))
    vol = cnlos.reconstruct(ctx, rect, 0.4, s, device="cpu")
    p = cnlos.prepare(rect, s)
    a = ctx.args
    np.testing.assert_array_equal(a["data"].numpy(), p.data)
    assert a["layout"] == FBP_LAYOUT_TIME_MAJOR and a["diffuse"] and a["snr"] == pytest.approx(0.08)
    assert a["width"] == 0.4 and a["bin_length"] == pytest.approx(3e8 * 8e-12)
    full = torch.arange(p.data.size, dtype=torch.float32).reshape(p.data.shape).numpy()
    np.testing.assert_array_equal(vol.numpy(), cnlos.display_crop(full, p, 0.4))
    assert a["output"] == FBP_LCT_OUTPUT_CLAMPED_REAL
    # python/lct_2.py's variant: per-depth radiometry, magnitude output.
    cnlos.reconstruct(ctx, rect, 0.4, s, device="cpu", variant="lct_2")
    assert ctx.args["output"] == FBP_LCT_OUTPUT_MAGNITUDE and ctx.args["grid_mode"] == FBP_LCT_GRID_DEPTH
    with pytest.raises(ValueError):
        cnlos.reconstruct(ctx, rect, 0.4, s, device="cpu", variant="lct3")
