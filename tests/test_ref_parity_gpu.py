"""Parity against the reference's own CUDA kernels, compiled from the reference
sources into oracle/_ref (the reference-kernel harness), on the same GPU.

* Time bins and weights: with one scan point every voxel receives exactly one
  term, so the reference's atomically accumulated volume equals I[bin] * w
  and must match the gather bit for bit with the reference's weights
  (FBP_WEIGHTS_REFERENCE); I[b] = 2^(b mod 3) makes a bin mismatch visible
  even where the weight matches.  With the default batched weights the bins
  are still the reference's (a wrong bin is off by a factor of 2) and each
  weight is within 6 ulp of the reference's reciprocal.
* Multi-scan volumes differ only by summation order (FP32 atomics in the
  reference vs blocked Kahan here): relative L2 <= 1e-5.
* LoG, Laplacian and normalisation keep the reference's per-output operation
  sequence: bitwise equal.
"""
import numpy as np
import pytest

from tests.conftest import reference_weights, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def harness(ctx):
    from oracle import harness as h

    if not h.available():
        pytest.skip("reference kernel harness not built (needs the reference sources when building)")
    h.load()
    return h


def _rand_geometry(rng, N, T, discard, t0_max, res=None):
    from fasterbackprojection_gb300 import make_info

    res = res or (N, N, N)
    step = float(rng.uniform(0.003, 0.012))
    hmin = (float(rng.uniform(-1, -0.5)), float(rng.uniform(-2.5, -1.5)), float(rng.uniform(-1, -0.5)))
    vs = tuple(float(rng.uniform(0.5, 2.0)) / r for r in res)
    lp = (float(rng.uniform(-1, 1)), float(rng.uniform(-1.3, -0.3)), float(rng.uniform(-1, 1)))
    sp = (float(rng.uniform(-1, 1)), float(rng.uniform(-1.3, -0.3)), float(rng.uniform(-1, 1)))
    return make_info(num_laser_targets=1, num_time_bins=T, time_step=step, voxel_res=res, hidden_min=hmin,
                     voxel_size=vs, time_offset=float(rng.uniform(0, t0_max)), discard_first_last_bounces=discard,
                     laser_position=lp, sensor_position=sp)


@pytest.mark.parametrize("mode", ["plain", "bounces", "t0", "bounces_t0"])
def test_confocal_single_scan_bitwise(ctx, harness, cuda, mode):
    import torch

    rng = np.random.default_rng({"plain": 1, "bounces": 2, "t0": 3, "bounces_t0": 4}[mode])
    T = 2048
    cube_np = (2.0 ** (np.arange(T) % 3)).astype(np.float32)
    cube = torch.from_numpy(cube_np).to(cuda)
    mismatch = 0
    total = 0
    for trial in range(12):
        info = _rand_geometry(rng, 48, T, 0 if "bounces" in mode else 1, 0.6 if "t0" in mode else 0.0,
                              res=(48, 40, 56))
        lxyz = torch.tensor([[rng.uniform(-1, 1), 0.0, rng.uniform(-1, 1)]], dtype=torch.float32, device=cuda)
        ref = harness.confocal_voxel(info, cube, lxyz)
        with reference_weights(ctx):
            got = ctx.backproject_confocal(info, cube.view(1, T), lxyz)
        torch.cuda.synchronize()
        mismatch += int((ref.view(torch.int32) != got.view(torch.int32)).sum())
        total += ref.numel()
    ctx.check_device_status()
    assert mismatch == 0, f"{mismatch} of {total} voxels differ from the reference kernel"


@pytest.mark.parametrize("mode", ["plain", "bounces", "t0", "bounces_t0"])
def test_confocal_single_scan_batched_weights_error_bound(ctx, harness, cuda, mode):
    """Default (batched, Montgomery) weights: the same voxels are non-zero and
    each differs from the reference kernel's I[bin] * rcp.approx(dist^2) by at
    most 6 ulp (the batched weight's ~3.5 ulp plus rcp.approx's own), far
    below the factor 2 a neighbouring bin would give."""
    import torch

    rng = np.random.default_rng({"plain": 31, "bounces": 32, "t0": 33, "bounces_t0": 34}[mode])
    T = 2048
    cube = torch.from_numpy((2.0 ** (np.arange(T) % 3)).astype(np.float32)).to(cuda)
    worst = 0.0
    for trial in range(12):
        info = _rand_geometry(rng, 48, T, 0 if "bounces" in mode else 1, 0.6 if "t0" in mode else 0.0,
                              res=(48, 40, 56))
        lxyz = torch.tensor([[rng.uniform(-1, 1), 0.0, rng.uniform(-1, 1)]], dtype=torch.float32, device=cuda)
        ref = harness.confocal_voxel(info, cube, lxyz).double()
        got = ctx.backproject_confocal(info, cube.view(1, T), lxyz).double()
        assert torch.equal(ref != 0, got != 0)
        nz = ref != 0
        if bool(nz.any()):
            worst = max(worst, float(((got[nz] - ref[nz]).abs() / ref[nz]).max()))
    ctx.check_device_status()
    assert worst <= 6 * 2.0 ** -23, worst


def test_confocal_matches_reference_kernel_multi_scan(ctx, harness, cuda):
    import torch
    from fasterbackprojection_gb300 import make_info, scenes

    cap = scenes.confocal_points(16, 512, 32e-12, n_points=40, seed=21)
    L, T = cap.cube.shape
    hmin, vs = scenes.volume_geometry((40, 36, 44), depth_range=(0.0, 2.4))
    for discard in (1, 0):
        info = make_info(num_laser_targets=L, num_time_bins=T, time_step=cap.time_step, voxel_res=(40, 36, 44),
                         hidden_min=hmin, voxel_size=vs, discard_first_last_bounces=discard,
                         laser_position=(0.0, -0.2, 0.1), sensor_position=(0.1, -0.2, 0.0))
        cube_ti = torch.from_numpy(cap.cube).to(cuda)
        cube_tm = cube_ti.t().contiguous()
        lxyz = torch.from_numpy(cap.laser_xyz).to(cuda)
        ref = harness.confocal_voxel(info, cube_tm, lxyz)
        got = ctx.backproject_confocal(info, cube_ti, lxyz)
        got_tm = ctx.backproject_confocal(info, cube_tm, lxyz, layout=0)
        assert torch.equal(got, got_tm)
        assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) < 1e-5


def test_exhaustive_single_pair_bitwise(ctx, harness, cuda):
    import torch
    from fasterbackprojection_gb300 import FBP_EXHAUSTIVE

    rng = np.random.default_rng(8)
    T = 2048
    cube = torch.from_numpy((2.0 ** (np.arange(T) % 3)).astype(np.float32)).to(cuda)
    bad = 0
    for trial in range(10):
        info = _rand_geometry(rng, 40, T, trial % 2, 0.3 * (trial % 3 == 2), res=(40, 32, 36))
        info.capture_system = FBP_EXHAUSTIVE
        info.num_sensor_targets = 1
        lxyz = torch.tensor([[rng.uniform(-1, 1), 0.0, rng.uniform(-1, 1)]], dtype=torch.float32, device=cuda)
        sxyz = torch.tensor([[rng.uniform(-1, 1), 0.0, rng.uniform(-1, 1)]], dtype=torch.float32, device=cuda)
        ref = harness.exhaustive_voxel(info, cube, lxyz, sxyz)
        with reference_weights(ctx):
            got = ctx.backproject_exhaustive(info, cube.view(1, 1, T), lxyz, sxyz)
        torch.cuda.synchronize()
        bad += int((ref.view(torch.int32) != got.view(torch.int32)).sum())
    assert bad == 0


def test_exhaustive_matches_reference_kernel_square_grid(ctx, harness, cuda):
    # The reference's pair split (l = ls / L, s = ls % L) is only correct when L == S.
    import torch
    from fasterbackprojection_gb300 import FBP_EXHAUSTIVE, make_info, scenes

    cap = scenes.exhaustive_points(4, 4, 512, 32e-12, n_points=30, seed=5)
    L, S, T = cap.cube.shape
    hmin, vs = scenes.volume_geometry((24, 20, 28), depth_range=(0.0, 2.0))
    info = make_info(num_laser_targets=L, num_sensor_targets=S, num_time_bins=T, time_step=cap.time_step,
                     voxel_res=(24, 20, 28), hidden_min=hmin, voxel_size=vs, capture_system=FBP_EXHAUSTIVE,
                     discard_first_last_bounces=0, laser_position=(0.0, -0.2, 0.1), sensor_position=(0.1, -0.3, 0.0))
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    sx = torch.from_numpy(cap.sensor_xyz).to(cuda)
    ref = harness.exhaustive_voxel(info, cube, lx, sx)
    got = ctx.backproject_exhaustive(info, cube, lx, sx)
    assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) < 1e-5


@pytest.mark.parametrize("system", ["confocal", "exhaustive"])
def test_depth_planes_match_reference_kernel(ctx, harness, cuda, system):
    import torch
    from fasterbackprojection_gb300 import FBP_EXHAUSTIVE, make_info, scenes
    from fasterbackprojection_gb300.api import linear_space

    depths = torch.from_numpy(linear_space(0.5, 0.9, 24)).to(cuda)
    if system == "confocal":
        cap = scenes.confocal_points(12, 512, 32e-12, n_points=30, seed=6)
        L, T = cap.cube.shape
        info = make_info(num_laser_targets=L, num_time_bins=T, time_step=cap.time_step, voxel_res=(1, 1, 1),
                         hidden_min=(0, 0, 0), voxel_size=(1, 1, 1), discard_first_last_bounces=0,
                         laser_position=(0.0, -0.2, 0.1), sensor_position=(0.1, -0.2, 0.0))
        cube = torch.from_numpy(cap.cube).to(cuda)
        lx = torch.from_numpy(cap.laser_xyz).to(cuda)
        ref = harness.depth_confocal(info, cube.t().contiguous(), lx, depths)
        got = ctx.backproject_depths(info, cube, lx, depths)
    else:
        cap = scenes.exhaustive_points(3, 3, 512, 32e-12, n_points=20, seed=7)
        L, S, T = cap.cube.shape
        info = make_info(num_laser_targets=L, num_sensor_targets=S, num_time_bins=T, time_step=cap.time_step,
                         voxel_res=(1, 1, 1), hidden_min=(0, 0, 0), voxel_size=(1, 1, 1),
                         capture_system=FBP_EXHAUSTIVE, discard_first_last_bounces=1)
        cube = torch.from_numpy(cap.cube).to(cuda)
        lx = torch.from_numpy(cap.laser_xyz).to(cuda)
        sx = torch.from_numpy(cap.sensor_xyz).to(cuda)
        ref = harness.depth_exhaustive(info, cube, lx, sx, depths)
        got = ctx.backproject_depths(info, cube, lx, depths, sensor_xyz=sx)
    assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("ksize", [3, 5, 7])
def test_log_filter_bitwise(ctx, harness, cuda, ksize):
    import torch
    from fasterbackprojection_gb300 import FBP_FILTER_LOG
    from fasterbackprojection_gb300.api import log_weights

    g = torch.Generator(device="cpu").manual_seed(ksize)
    vol = torch.rand((20, 27, 33), generator=g).to(cuda)
    w = torch.from_numpy(log_weights(ksize, 1.0)).to(cuda)
    ref = harness.log_filter(vol, w, ksize)
    got = ctx.postfilter(FBP_FILTER_LOG, vol, ksize, 1.0)
    assert torch.equal(ref, got)


@pytest.mark.parametrize("ksize", [3, 5])
def test_laplacian_filter_bitwise(ctx, harness, cuda, ksize):
    import torch
    from fasterbackprojection_gb300 import FBP_FILTER_LAPLACIAN

    g = torch.Generator(device="cpu").manual_seed(10 + ksize)
    vol = torch.rand((19, 22, 30), generator=g).to(cuda)
    ref = harness.laplacian_filter(vol, ksize)
    got = ctx.postfilter(FBP_FILTER_LAPLACIAN, vol, ksize)
    assert torch.equal(ref, got)


def test_normalize_bitwise(ctx, harness, cuda):
    import torch

    g = torch.Generator(device="cpu").manual_seed(3)
    v = (torch.rand(1_000_003, generator=g) * 7 - 2).to(cuda)
    ref = harness.normalize_(v.clone())
    got = ctx.normalize_(v.clone())
    assert torch.equal(ref, got)


@pytest.mark.parametrize("mode", ["plain", "bounces", "t0", "fine", "mid"])
def test_voxel_scattering_single_scan_bitwise(ctx, harness, cuda, mode):
    """The ACCUMULATE_VOXEL_SCATTERING build: with one scan point each voxel's
    bins are added by one reference thread in bin order, so the volume must
    match bit for bit (ext, step and every visited bin included).  "fine" and
    "mid" set the voxel diagonal to 0.35-1.0 and 2.1-2.9 time steps (two and
    three steps per pair); the random geometries of the other modes take
    3 to 30 steps."""
    import torch

    if not harness.scatter_available():
        pytest.skip("voxel-scattering build of the reference kernels not present")
    rng = np.random.default_rng({"plain": 11, "bounces": 12, "t0": 13, "fine": 14, "mid": 15}[mode])
    T = 2048
    cube = torch.from_numpy((2.0 ** (np.arange(T) % 3)).astype(np.float32)).to(cuda)
    mismatch = total = 0
    for trial in range(8):
        info = _rand_geometry(rng, 32, T, 0 if mode == "bounces" else 1, 0.6 if mode == "t0" else 0.0,
                              res=(32, 24, 40))
        if mode in ("fine", "mid"):
            lo, hi = (0.2, 0.6) if mode == "fine" else (1.2, 1.7)
            for k in range(3):
                info.voxel_size[k] = info.time_step * float(rng.uniform(lo, hi))
        lxyz = torch.tensor([[rng.uniform(-1, 1), 0.0, rng.uniform(-1, 1)]], dtype=torch.float32, device=cuda)
        ref = harness.confocal_voxel_scatter(info, cube, lxyz)
        got = ctx.backproject_confocal_scatter(info, cube.view(1, T), lxyz)
        torch.cuda.synchronize()
        mismatch += int((ref.view(torch.int32) != got.view(torch.int32)).sum())
        total += ref.numel()
    ctx.check_device_status()
    assert mismatch == 0, f"{mismatch} of {total} voxels differ from the reference kernel"


def test_voxel_scattering_multi_scan_matches_reference(ctx, harness, cuda):
    import torch
    from fasterbackprojection_gb300 import make_info, scenes

    if not harness.scatter_available():
        pytest.skip("voxel-scattering build of the reference kernels not present")
    cap = scenes.confocal_points(12, 512, 32e-12, n_points=30, seed=23)
    L, T = cap.cube.shape
    hmin, vs = scenes.volume_geometry((24, 20, 28), depth_range=(0.0, 2.4))
    info = make_info(num_laser_targets=L, num_time_bins=T, time_step=cap.time_step, voxel_res=(24, 20, 28),
                     hidden_min=hmin, voxel_size=vs)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lxyz = torch.from_numpy(cap.laser_xyz).to(cuda)
    ref = harness.confocal_voxel_scatter(info, cube.t().contiguous(), lxyz)
    got = ctx.backproject_confocal_scatter(info, cube, lxyz)
    plain = ctx.backproject_confocal(info, cube, lxyz)
    assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) < 1e-5
    assert float(got.sum()) > float(plain.sum())  # several bins per pair
