"""Randomised parity sweeps over the paths with the most forms: many random
geometries (ragged volumes of 5-70 voxels per axis, random wall, voxel and
bin sizes) against the reference's own kernels bit for bit, and LCT / LoG-FFT
sizes against the FP64 restatements."""
import numpy as np
import pytest

from oracle import numpy_ref
from tests.conftest import reference_weights, rel_l2
from tests.test_ref_parity_gpu import _rand_geometry

pytestmark = pytest.mark.gpu

T = 2048


@pytest.fixture(scope="module")
def harness(ctx):
    from oracle import harness as h

    if not h.available():
        pytest.skip("reference kernel harness not built (needs the reference sources when building)")
    h.load()
    return h


def _cube(cuda):
    import torch

    return torch.from_numpy((2.0 ** (np.arange(T) % 3)).astype(np.float32)).to(cuda)


def _lxyz(rng, cuda):
    import torch

    return torch.tensor([[rng.uniform(-1, 1), 0.0, rng.uniform(-1, 1)]], dtype=torch.float32, device=cuda)


@pytest.mark.parametrize("mode", ["plain", "bounces", "t0", "bounces_t0"])
def test_confocal_random_geometries_bitwise(ctx, harness, cuda, mode):
    """backprojectConfocalVoxel (transient_reconstruction.cuh:93-136), one scan
    point per geometry: every voxel of 60 random volumes bit for bit."""
    import torch

    discard, t0 = {"plain": (1, 0.0), "bounces": (0, 0.0), "t0": (1, 0.6), "bounces_t0": (0, 0.6)}[mode]
    rng = np.random.default_rng(5000 + len(mode))
    cube = _cube(cuda)
    bad = total = nonzero = 0
    with reference_weights(ctx):
        for _ in range(60):
            res = tuple(int(r) for r in rng.integers(5, 70, 3))
            info = _rand_geometry(rng, 48, T, discard, t0, res=res)
            lx = _lxyz(rng, cuda)
            ref = harness.confocal_voxel(info, cube, lx)
            got = ctx.backproject_confocal(info, cube.view(1, T), lx)
            torch.cuda.synchronize()
            bad += int((ref.view(torch.int32) != got.view(torch.int32)).sum())
            total += ref.numel()
            nonzero += int((ref != 0).sum())
    ctx.check_device_status()
    assert nonzero > total // 5, f"{nonzero} of {total} voxels non-zero"
    assert bad == 0, f"{bad} of {total} voxels differ from the reference kernel"


@pytest.mark.parametrize("mode", ["plain", "bounces", "t0", "fine", "mid", "long"])
def test_voxel_scattering_random_geometries_bitwise(ctx, harness, cuda, mode):
    """The ACCUMULATE_VOXEL_SCATTERING build (transient_reconstruction.cuh:
    112-126): walks shorter than a bin ("fine"), of 2-3 bins ("mid": every walk
    exactly the unrolled steps), 3.5-6 bins ("long": unconditional steps and
    the tail loop) and the random geometries' 3-30 bins."""
    import torch

    if not harness.scatter_available():
        pytest.skip("voxel-scattering build of the reference kernels not present")
    rng = np.random.default_rng(6000 + len(mode) * 7)
    cube = _cube(cuda)
    bad = total = nonzero = 0
    for _ in range(40):
        res = tuple(int(r) for r in rng.integers(5, 48, 3))
        info = _rand_geometry(rng, 32, T, 0 if mode == "bounces" else 1, 0.6 if mode == "t0" else 0.0, res=res)
        if mode in ("fine", "mid", "long"):
            lo, hi = {"fine": (0.2, 0.6), "mid": (1.2, 1.7), "long": (2.0, 3.5)}[mode]
            for k in range(3):
                info.voxel_size[k] = info.time_step * float(rng.uniform(lo, hi))
        lx = _lxyz(rng, cuda)
        ref = harness.confocal_voxel_scatter(info, cube, lx)
        got = ctx.backproject_confocal_scatter(info, cube.view(1, T), lx)
        torch.cuda.synchronize()
        bad += int((ref.view(torch.int32) != got.view(torch.int32)).sum())
        total += ref.numel()
        nonzero += int((ref != 0).sum())
    ctx.check_device_status()
    assert nonzero > total // 5, f"{nonzero} of {total} voxels non-zero"
    assert bad == 0, f"{bad} of {total} voxels differ from the reference scattering kernel"


@pytest.mark.parametrize("n,m", [(8, 16), (16, 64), (32, 128), (64, 32), (64, 256), (64, 1024), (128, 64),
                                 (128, 256), (16, 2048)])
@pytest.mark.parametrize("output", [0, 1])
def test_lct_sizes_and_outputs_vs_fp64(ctx, cuda, n, m, output):
    """python/lct.py (output 0, max(real, 0)) and lct_2.py's |vol| (output 1)
    across the plane-pass and row/column forms of the half z-spectrum."""
    import torch
    from fasterbackprojection_gb300 import scenes

    cap = scenes.confocal_points(n, m, 32e-12 * 512 / m, n_points=40, seed=7 * n + m)
    data = cap.cube.reshape(n, n, m).transpose(2, 0, 1).copy()
    got = ctx.lct(torch.from_numpy(data).to(cuda), 1.0, cap.time_step, 0.8, True, output=output).cpu().numpy()
    want = numpy_ref.lct(data.astype(np.float64), 1.0, cap.time_step, 0.8, True,
                         output="magnitude" if output else "clamped_real")
    assert float(np.abs(want).max()) > 0
    assert rel_l2(got, want) < 1e-5


def _log_response(nx, ny, nz, sigma):
    def freqs(n):
        a = np.arange(n, dtype=np.float32)
        return np.where(a <= n // 2, a, a - n).astype(np.float32) / np.float32(n)

    fz, fy, fx = np.meshgrid(freqs(nz), freqs(ny), freqs(nx), indexing="ij")
    k2 = fx * fx + fy * fy + fz * fz
    pi = np.float32(np.pi)
    return (-4 * pi * pi * k2 * np.exp(-2 * pi * pi * sigma * sigma * k2)).astype(np.float64)


@pytest.mark.parametrize("shape", [(256, 64, 32), (32, 256, 64), (64, 32, 256), (256, 256, 32), (128, 256, 256)])
def test_log_fft_256_axes_vs_fp64(ctx, cuda, shape):
    """LoGFFT::compute (PostprocessingFilters.cu:36-77) with 256-long axes (the
    register line transforms) in every position, against FP64 FFTs."""
    import torch
    from fasterbackprojection_gb300 import FBP_FILTER_LOG_FFT

    nz, ny, nx = shape
    vol = np.random.default_rng(nx + 3 * ny + 7 * nz).random(shape).astype(np.float32)
    got = ctx.postfilter(FBP_FILTER_LOG_FFT, torch.from_numpy(vol).to(cuda), 5, 1.3).cpu().numpy()
    want = np.real(np.fft.ifftn(np.fft.fftn(vol.astype(np.float64)) * _log_response(nx, ny, nz, 1.3)))
    want *= nx * ny * nz
    assert rel_l2(got, want) < 5e-6


def test_exhaustive_random_grids_vs_fp64(ctx, cuda):
    """backprojectExhaustiveVoxel (transient_reconstruction.cuh:138-166) over
    random laser / SPAD grids (4-36 lasers and SPADs: stages of up to 64 pairs
    with ragged last stages, laser blocks of 4 and single lasers), ragged
    volumes and random time offsets and bounce modes, against the FP64 oracle
    with the GPU's bins."""
    import torch
    from fasterbackprojection_gb300 import FBP_EXHAUSTIVE, make_info, scenes
    from oracle import cpu

    rng = np.random.default_rng(7100)
    worst, compared = 0.0, 0
    for trial in range(12):
        nl, ns = int(rng.integers(2, 7)), int(rng.integers(2, 7))
        Tb = int(rng.choice([256, 512, 1024]))  # 64 bins of 32 ps end before the scene's paths
        cap = scenes.exhaustive_points(nl, ns, Tb, 32e-12, n_points=20, seed=7100 + trial)
        L, S, Tb = cap.cube.shape
        vres = tuple(int(r) for r in rng.integers(6, 26, 3))
        hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, float(rng.uniform(1.2, 2.4))))
        info = make_info(num_laser_targets=L, num_sensor_targets=S, num_time_bins=Tb, time_step=cap.time_step,
                         voxel_res=vres, hidden_min=hmin, voxel_size=vs, capture_system=FBP_EXHAUSTIVE,
                         discard_first_last_bounces=int(rng.integers(0, 2)), laser_position=(0.0, -0.2, 0.1),
                         sensor_position=(0.1, -0.3, 0.0), time_offset=float(rng.choice([0.0, -0.05, 0.2])))
        cube = torch.from_numpy(cap.cube).to(cuda)
        lx = torch.from_numpy(cap.laser_xyz).to(cuda)
        sx = torch.from_numpy(cap.sensor_xyz).to(cuda)
        got = ctx.backproject_exhaustive(info, cube, lx, sx).cpu().numpy()
        V = vres[0] * vres[1] * vres[2]
        bins = ctx.debug_exhaustive_bins(info, lx, sx, torch.arange(V, device=cuda)).cpu().numpy()
        want = cpu.exhaustive_voxel(info, cap.cube, cap.laser_xyz, cap.sensor_xyz, bins=bins)
        if float(np.abs(want).max()) > 0:
            worst = max(worst, rel_l2(got, want))
            compared += 1
    ctx.check_device_status()
    assert compared >= 10, compared
    assert worst < 1e-6, worst
