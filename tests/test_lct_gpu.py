"""GPU LCT and LoG-FFT against the reference's own lct.py outputs (golden
fixtures), the FP64 NumPy restatement, and the reference's cuFFT pipeline."""
from pathlib import Path

import numpy as np
import pytest

from oracle import numpy_ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "lct_golden.npz"


@pytest.mark.parametrize("name", ["lct_a", "lct_b"])
def test_lct_matches_reference_golden(ctx, cuda, name):
    import torch

    g = np.load(GOLDEN)
    width, bl, snr, diffuse = g[f"{name}_params"]
    data = torch.from_numpy(g[f"{name}_data"]).to(cuda)
    got = ctx.lct(data, float(width), float(bl), float(snr), bool(diffuse)).cpu().numpy()
    assert rel_l2(got, g[f"{name}_vol"]) < 1e-4


def test_lct_layouts_and_plan_cache(ctx, cuda):
    import torch
    from fasterbackprojection_gb300 import FBP_LAYOUT_TIME_INNER

    g = np.load(GOLDEN)
    data = torch.from_numpy(g["lct_a_data"]).to(cuda)  # [M][N][N]
    a = ctx.lct(data, 1.0, 0.03)
    b = ctx.lct(data.permute(1, 2, 0).contiguous(), 1.0, 0.03, layout=FBP_LAYOUT_TIME_INNER)
    c = ctx.lct(data, 1.0, 0.03)  # cached plan
    assert torch.equal(a, b) and torch.equal(a, c)
    d = ctx.lct(data, 1.0, 0.05)  # new plan
    assert not torch.equal(a, d)


@pytest.mark.parametrize("grid", ["reference", "depth"])
def test_lct_64x64x512_vs_fp64(ctx, cuda, grid):
    """64 x 64 scan, 512 bins of 32 ps (the LCT benchmark shape)."""
    import torch
    from fasterbackprojection_gb300 import FBP_LCT_GRID_DEPTH, FBP_LCT_GRID_REFERENCE, scenes

    cap = scenes.confocal_points(64, 512, 32e-12, n_points=200, seed=1)
    data = cap.cube.reshape(64, 64, 512).transpose(2, 0, 1).copy()  # [M][N][N]
    mode = FBP_LCT_GRID_REFERENCE if grid == "reference" else FBP_LCT_GRID_DEPTH
    got = ctx.lct(torch.from_numpy(data).to(cuda), 1.0, cap.time_step, 0.8, True, grid_mode=mode).cpu().numpy()
    want = numpy_ref.lct(data.astype(np.float64), 1.0, cap.time_step, 0.8, True, grid=grid)
    assert rel_l2(got, want) < 1e-4


@pytest.mark.parametrize("n,m", [(64, 512), (128, 32), (4, 8)])
def test_lct2_variant_vs_fp64(ctx, cuda, n, m):
    """python/lct_2.py's variant: per-depth radiometry and abs(vol) instead of
    max(real(vol), 0), through the three-pass (N <= 64), row/column (N > 64)
    and line-pipeline (N < 8) paths, against the FP64 restatement with the
    same two changes."""
    import torch
    from fasterbackprojection_gb300 import FBP_LCT_GRID_DEPTH, FBP_LCT_OUTPUT_MAGNITUDE, scenes

    cap = scenes.confocal_points(n, m, 32e-12 * (512 // m if m < 512 else 1), n_points=60, seed=n + m)
    data = cap.cube.reshape(n, n, m).transpose(2, 0, 1).copy()
    d = torch.from_numpy(data).to(cuda)
    got = ctx.lct(d, 1.0, cap.time_step, 0.8, True, grid_mode=FBP_LCT_GRID_DEPTH,
                  output=FBP_LCT_OUTPUT_MAGNITUDE).cpu().numpy()
    want = numpy_ref.lct(data.astype(np.float64), 1.0, cap.time_step, 0.8, True, grid="depth", output="magnitude")
    assert float(np.abs(want).max()) > 0
    assert rel_l2(got, want) < 1e-4
    # The magnitude bounds the clamped real part voxel by voxel.
    clamped = ctx.lct(d, 1.0, cap.time_step, 0.8, True, grid_mode=FBP_LCT_GRID_DEPTH).cpu().numpy()
    assert (got >= clamped - 1e-6 * float(np.abs(got).max())).all()


@pytest.mark.parametrize("n,m", [(4, 8), (128, 32), (256, 16), (8, 2048), (16, 1024), (64, 16)])
def test_lct_sizes_vs_fp64(ctx, cuda, n, m):
    """Scan grids and bin counts across the LCT paths (plane pass for
    8 <= N <= 64, row and column passes above, the line pipeline outside
    16 <= M <= 2048 or below N = 8) against the FP64 restatement."""
    import torch
    from fasterbackprojection_gb300 import scenes

    cap = scenes.confocal_points(n, m, 32e-12 * 512 / m, n_points=40, seed=n + m)
    data = cap.cube.reshape(n, n, m).transpose(2, 0, 1).copy()
    got = ctx.lct(torch.from_numpy(data).to(cuda), 1.0, cap.time_step, 0.8, True).cpu().numpy()
    want = numpy_ref.lct(data.astype(np.float64), 1.0, cap.time_step, 0.8, True)
    assert float(np.abs(want).max()) > 0
    assert rel_l2(got, want) < 1e-4


def test_lct_rejects_bad_sizes(ctx, cuda):
    import torch
    from fasterbackprojection_gb300 import FbpError

    with pytest.raises(FbpError):
        ctx.lct(torch.zeros((48, 16, 16), device=cuda), 1.0, 0.03)


def _log_response_np(n, sigma):
    f = np.arange(n, dtype=np.float32)
    f = np.where(f <= n // 2, f, f - n).astype(np.float32) / np.float32(n)
    fz, fy, fx = np.meshgrid(f, f, f, indexing="ij")
    k2 = fx * fx + fy * fy + fz * fz
    pi = np.float32(np.pi)
    return (-4 * pi * pi * k2 * np.exp(-2 * pi * pi * sigma * sigma * k2)).astype(np.float64)


@pytest.mark.parametrize("n", [32, 64])
def test_log_fft_filter(ctx, cuda, n):
    """LoGFFT::compute: unnormalised inverse of FFT(vol) * LoG response."""
    import torch
    from fasterbackprojection_gb300 import FBP_FILTER_LOG_FFT

    vol = np.random.default_rng(n).random((n, n, n)).astype(np.float32)
    got = ctx.postfilter(FBP_FILTER_LOG_FFT, torch.from_numpy(vol).to(cuda), 5, 1.0).cpu().numpy()
    want = np.real(np.fft.ifftn(np.fft.fftn(vol.astype(np.float64)) * _log_response_np(n, 1.0))) * n ** 3
    assert rel_l2(got, want) < 1e-5
    # The reference's own arithmetic path: R2C, half-grid response, C2R (cuFFT via torch).
    v = torch.from_numpy(vol).to(cuda)
    F = torch.fft.rfftn(v)
    K = torch.from_numpy(_log_response_np(n, 1.0)[:, :, : n // 2 + 1].astype(np.float32)).to(cuda)
    ref = torch.fft.irfftn(F * K, s=v.shape, norm="forward").cpu().numpy()
    assert rel_l2(got, ref) < 1e-5


def _log_response_xyz(nx, ny, nz, sigma):
    def freqs(n):
        f = np.arange(n, dtype=np.float32)
        return np.where(f <= n // 2, f, f - n).astype(np.float32) / np.float32(n)
    fz, fy, fx = np.meshgrid(freqs(nz), freqs(ny), freqs(nx), indexing="ij")
    k2 = fx * fx + fy * fy + fz * fz
    pi = np.float32(np.pi)
    return (-4 * pi * pi * k2 * np.exp(-2 * pi * pi * sigma * sigma * k2)).astype(np.float64)


@pytest.mark.parametrize("shape", [(64, 32, 128), (16, 16, 16), (32, 256, 64), (256, 32, 256), (32, 256, 256)])
def test_log_fft_filter_non_cubic(ctx, cuda, shape):
    """Non-cubic volumes (z, y, x): the half-spectrum path for axes in
    [32, 1024], the full complex passes below that; axes of 256 take the
    register (16 x 16) line transforms (x and z, x and y here)."""
    import torch
    from fasterbackprojection_gb300 import FBP_FILTER_LOG_FFT

    nz, ny, nx = shape
    vol = np.random.default_rng(nx * ny + nz).random(shape).astype(np.float32)
    got = ctx.postfilter(FBP_FILTER_LOG_FFT, torch.from_numpy(vol).to(cuda), 5, 1.5).cpu().numpy()
    want = np.real(np.fft.ifftn(np.fft.fftn(vol.astype(np.float64)) * _log_response_xyz(nx, ny, nz, 1.5)))
    want *= nx * ny * nz
    assert rel_l2(got, want) < 1e-5

