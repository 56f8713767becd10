"""Backprojection kernels against the FP64 CPU oracle.

Tolerances (relative L2 over the volume):
  * 1e-6 when the oracle is given the GPU's own time bins (isolates the
    accumulation: FP32 blocks + Kahan vs FP64), for FP32, BF16 and FP16
    storage (the oracle reads the decoded 16-bit values);
  * 1e-3 against fully independent FP64 bins, where rare pairs whose path
    lands within an FP32 rounding of a bin edge fall in the neighbouring bin
    (the count of such pairs is checked too).
"""
import numpy as np
import pytest

from oracle import cpu
from tests.conftest import reference_weights, rel_l2

pytestmark = pytest.mark.gpu


def _confocal_case(n=12, T=512, vres=(28, 24, 32), seed=11, discard=1, t0=0.0, depth=(0.0, 2.4)):
    from fasterbackprojection_gb300 import make_info, scenes

    cap = scenes.confocal_points(n, T, 32e-12, n_points=40, seed=seed)
    hmin, vs = scenes.volume_geometry(vres, depth_range=depth)
    info = make_info(num_laser_targets=n * n, num_time_bins=T, time_step=cap.time_step, voxel_res=vres,
                     hidden_min=hmin, voxel_size=vs, discard_first_last_bounces=discard, time_offset=t0,
                     laser_position=(0.05, -0.25, 0.1), sensor_position=(-0.1, -0.2, 0.05))
    return cap, info


def _gpu_bins(ctx, info, lxyz_t, cuda):
    import torch

    V = info.voxel_res[0] * info.voxel_res[1] * info.voxel_res[2]
    idx = torch.arange(V, dtype=torch.int64, device=cuda)
    return ctx.debug_confocal_bins(info, lxyz_t, idx).cpu().numpy()


@pytest.mark.parametrize("discard,t0", [(1, 0.0), (0, 0.0), (1, 0.3)])
def test_confocal_f32_vs_fp64_oracle(ctx, cuda, discard, t0):
    import torch

    cap, info = _confocal_case(discard=discard, t0=t0)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    got = ctx.backproject_confocal(info, cube, lx).cpu().numpy()
    ctx.check_device_status()
    bins = _gpu_bins(ctx, info, lx, cuda)
    want = cpu.confocal_voxel(info, cap.cube, cap.laser_xyz, bins=bins)
    assert rel_l2(got, want) < 1e-6
    # Fully independent FP64 bins.
    want64 = cpu.confocal_voxel(info, cap.cube, cap.laser_xyz)
    assert rel_l2(got, want64) < 1e-3


@pytest.mark.parametrize("discard,t0,dtype", [(1, 0.0, "f32"), (0, 0.0, "f32"), (1, 0.3, "f32"), (1, 0.0, "bf16")])
def test_confocal_batched_weights_match_reference_weights(ctx, cuda, discard, t0, dtype):
    """The default batched reciprocal against one reciprocal per pair on the
    same bins: 1e-6 relative L2 over the volume, 2e-6 relative per voxel."""
    import torch

    cap, info = _confocal_case(n=16, vres=(40, 36, 44), seed=29, discard=discard, t0=t0)
    cube = torch.from_numpy(cap.cube).to(cuda)
    if dtype == "bf16":
        cube = cube.to(torch.bfloat16)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    got = ctx.backproject_confocal(info, cube, lx).double()
    with reference_weights(ctx):
        want = ctx.backproject_confocal(info, cube, lx).double()
    ctx.check_device_status()
    assert float(want.abs().max()) > 0
    assert rel_l2(got.cpu().numpy(), want.cpu().numpy()) < 1e-6
    nz = want.abs() > 1e-3 * float(want.abs().max())
    assert float(((got - want).abs()[nz] / want.abs()[nz]).max()) < 2e-6


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
def test_confocal_benchmark_size_largest_voxels_vs_fp64(ctx, cuda, dtype):
    """The benchmark workload (256^2 scan x 1024 bins of 16 ps -> 256^3) on
    its 200 largest voxels and 200 random ones, against the FP64 oracle with
    the GPU's bins: 1e-6 relative L2.  The largest voxels sum ~65k terms of
    the largest weights; a lost compensation there shows as ~1e-5, which a
    random sample of a 16.7M-voxel volume rarely meets."""
    import torch
    from fasterbackprojection_gb300 import make_info, scenes

    cap = scenes.confocal_patches_torch(256, 1024, 16e-12, seed=2, device=cuda)
    hmin, vs = scenes.volume_geometry((256, 256, 256), depth_range=(0.0, 1.5))
    info = make_info(num_laser_targets=256 * 256, num_time_bins=1024, time_step=cap.time_step,
                     voxel_res=(256, 256, 256), hidden_min=hmin, voxel_size=vs)
    cube = cap.cube if dtype == "f32" else cap.cube.to(torch.bfloat16)
    vol = ctx.backproject_confocal(info, cube, cap.laser_xyz).view(-1)
    ctx.check_device_status()
    top = torch.topk(vol, 200).indices
    rnd = torch.from_numpy(np.random.default_rng(4).choice(vol.numel(), 200, replace=False)).to(cuda)
    idx = torch.sort(torch.unique(torch.cat([top, rnd]))).values
    bins = ctx.debug_confocal_bins(info, cap.laser_xyz, idx).cpu().numpy()
    host = cube.float().cpu().numpy()
    want = cpu.confocal_voxel_subset(info, host, cap.laser_xyz.cpu().numpy(), idx.cpu().numpy(), bins=bins)
    got = vol[idx].double().cpu().numpy()
    assert rel_l2(got, want) < 1e-6
    assert float(np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-30))) < 1e-5


@pytest.mark.parametrize("discard,t0,vres", [(1, 0.0, (28, 24, 32)), (0, 0.0, (20, 18, 44)), (1, 0.3, (24, 40, 16))])
def test_confocal_scatter_vs_fp64_oracle(ctx, cuda, discard, t0, vres):
    """The voxel-scattering gather (ACCUMULATE_VOXEL_SCATTERING,
    transient_reconstruction.cuh:112-126) against the FP64 oracle: the oracle's
    float32 replay of every walk from the GPU's FP32 paths (the GPU's bins,
    FP64 sums) within 1e-6; the independent FP64 walk (oracle/fbp_oracle.c)
    within 1e-2, where walk ends within an FP32 rounding of a bin edge differ."""
    import torch
    from oracle import numpy_ref

    cap, info = _confocal_case(vres=vres, seed=37, discard=discard, t0=t0)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    got = ctx.backproject_confocal_scatter(info, cube, lx).cpu().numpy().ravel()
    V = vres[0] * vres[1] * vres[2]
    paths, (rcp_dt, ext) = ctx.debug_confocal_paths(info, lx, torch.arange(V, device=cuda))
    ctx.check_device_status()
    want = numpy_ref.confocal_scatter_given_paths(cap.cube, paths.cpu().numpy(), rcp_dt, ext, info.time_step)
    assert float(np.abs(want).max()) > 0
    assert rel_l2(got, want) < 1e-6
    want64 = cpu.confocal_scatter_voxel(info, cap.cube, cap.laser_xyz).ravel()
    assert rel_l2(got, want64) < 1e-2


@pytest.mark.parametrize("dtype", ["bf16", "f16"])
def test_confocal_16bit_storage_vs_oracle(ctx, cuda, dtype):
    import torch

    cap, info = _confocal_case(seed=13)
    tdt = torch.bfloat16 if dtype == "bf16" else torch.float16
    cube16 = torch.from_numpy(cap.cube).to(cuda).to(tdt)
    decoded = cube16.float().cpu().numpy()
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    got = ctx.backproject_confocal(info, cube16, lx).cpu().numpy()
    bins = _gpu_bins(ctx, info, lx, cuda)
    want = cpu.confocal_voxel(info, decoded, cap.laser_xyz, bins=bins)
    assert rel_l2(got, want) < 1e-6


def test_confocal_bins_agree_with_fp64_except_at_edges(ctx, cuda):
    import torch

    cap, info = _confocal_case(seed=17)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    bins = _gpu_bins(ctx, info, lx, cuda)
    Vx, Vy, Vz = info.voxel_res
    v = np.arange(Vx * Vy * Vz)
    vz, r = np.divmod(v, Vx * Vy)
    vy, vx = np.divmod(r, Vx)
    p = np.stack([info.hidden_min[0] + (vx + 0.5) * info.voxel_size[0],
                  info.hidden_min[1] + (vz + 0.5) * info.voxel_size[1],
                  info.hidden_min[2] + (vy + 0.5) * info.voxel_size[2]], 1)
    d = 2 * np.linalg.norm(p[:, None, :] - cap.laser_xyz[None].astype(np.float64), axis=2)
    x = d / np.float64(np.float32(info.time_step))
    b64 = np.where((x > -1) & (x < info.num_time_bins), np.trunc(x), -1).astype(np.int64)
    diff = b64 != bins
    assert diff.mean() < 1e-4
    # Every disagreement sits within a few FP32 roundings of a bin edge.
    frac = np.abs(x[diff] - np.rint(x[diff]))
    assert np.all(frac < 1e-4)


def test_confocal_is_deterministic_and_layouts_agree(ctx, cuda):
    import torch

    cap, info = _confocal_case(seed=19)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    a = ctx.backproject_confocal(info, cube, lx)
    b = ctx.backproject_confocal(info, cube, lx)
    c = ctx.backproject_confocal(info, cube.t().contiguous(), lx, layout=0)
    assert torch.equal(a, b) and torch.equal(a, c)


@pytest.mark.parametrize("n,vres,T", [(5, (3, 5, 7), 96), (7, (9, 1, 33), 300), (11, (65, 17, 9), 700)])
def test_confocal_ragged_sizes(ctx, cuda, n, vres, T):
    """Scan counts not a multiple of the chunk, volumes not a multiple of the tile."""
    import torch

    cap, info = _confocal_case(n=n, T=T, vres=vres, seed=n)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    got = ctx.backproject_confocal(info, cube, lx).cpu().numpy()
    bins = _gpu_bins(ctx, info, lx, cuda)
    want = cpu.confocal_voxel(info, cap.cube, cap.laser_xyz, bins=bins)
    assert rel_l2(got, want) < 1e-6


def test_confocal_voxels_touching_the_wall(ctx, cuda):
    """Volumes reaching the wall exercise safeRCP's dist^2 <= EPS branch."""
    import torch

    cap, info = _confocal_case(seed=23, vres=(16, 16, 16), depth=(0.0, 0.2))
    info.hidden_min[1] = -0.1
    cube = torch.from_numpy(cap.cube).to(cuda)
    cube[:, :4] = 5.0  # make near-zero bins non-empty
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    got = ctx.backproject_confocal(info, cube, lx).cpu().numpy()
    bins = _gpu_bins(ctx, info, lx, cuda)
    want = cpu.confocal_voxel(info, cube.cpu().numpy(), cap.laser_xyz, bins=bins)
    assert rel_l2(got, want) < 1e-6


def test_confocal_empty_and_invalid_inputs(ctx, cuda):
    import torch
    from fasterbackprojection_gb300 import FbpError

    cap, info = _confocal_case()
    cube = torch.zeros_like(torch.from_numpy(cap.cube)).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    assert float(ctx.backproject_confocal(info, cube, lx).abs().max()) == 0.0
    info.num_time_bins = 0
    with pytest.raises(FbpError):
        ctx.backproject_confocal(info, cube, lx)
    cap, info = _confocal_case()
    info.time_step = -1.0
    with pytest.raises(FbpError):
        ctx.backproject_confocal(info, cube, lx)


@pytest.mark.parametrize("nl,ns,discard,t0,T", [(3, 4, 1, 0.0, 512), (4, 3, 0, 0.0, 512), (2, 5, 1, 0.0, 512),
                                                 (4, 4, 1, -0.05, 512), (4, 4, 0, 0.2, 512), (3, 4, 1, 0.0, 64),
                                                 (4, 4, 0, 0.0, 64)])
def test_exhaustive_vs_fp64_oracle(ctx, cuda, nl, ns, discard, t0, T):
    """Including L != S, where the reference's own pair split is out of range;
    laser blocks of 4 (L % 4 == 0) and single lasers; time offsets of zero
    (the subtraction skipped), negative and positive (conversion bins); and
    64 bins, where the tile's bin window is capped at the whole row."""
    import torch
    from fasterbackprojection_gb300 import FBP_EXHAUSTIVE, make_info, scenes

    cap = scenes.exhaustive_points(nl, ns, T, 32e-12, n_points=25, seed=nl * 10 + ns)
    L, S, T = cap.cube.shape
    vres = (20, 18, 22)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 2.0))
    info = make_info(num_laser_targets=L, num_sensor_targets=S, num_time_bins=T, time_step=cap.time_step,
                     voxel_res=vres, hidden_min=hmin, voxel_size=vs, capture_system=FBP_EXHAUSTIVE,
                     discard_first_last_bounces=discard, laser_position=(0.0, -0.2, 0.1),
                     sensor_position=(0.1, -0.3, 0.0), time_offset=t0)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    sx = torch.from_numpy(cap.sensor_xyz).to(cuda)
    got = ctx.backproject_exhaustive(info, cube, lx, sx).cpu().numpy()
    V = vres[0] * vres[1] * vres[2]
    bins = ctx.debug_exhaustive_bins(info, lx, sx, torch.arange(V, device=cuda)).cpu().numpy()
    want = cpu.exhaustive_voxel(info, cap.cube, cap.laser_xyz, cap.sensor_xyz, bins=bins)
    assert rel_l2(got, want) < 1e-6
    assert rel_l2(got, cpu.exhaustive_voxel(info, cap.cube, cap.laser_xyz, cap.sensor_xyz)) < 1e-3


@pytest.mark.parametrize("nl,ns", [(4, 4), (3, 5)])
def test_exhaustive_batched_weights_match_reference_weights(ctx, cuda, nl, ns):
    """Shared reciprocals (the default) against one reciprocal per triple."""
    import torch
    from fasterbackprojection_gb300 import FBP_EXHAUSTIVE, make_info, scenes

    cap = scenes.exhaustive_points(nl, ns, 512, 32e-12, n_points=25, seed=77 + nl)
    L, S, T = cap.cube.shape
    vres = (24, 20, 28)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 2.0))
    info = make_info(num_laser_targets=L, num_sensor_targets=S, num_time_bins=T, time_step=cap.time_step,
                     voxel_res=vres, hidden_min=hmin, voxel_size=vs, capture_system=FBP_EXHAUSTIVE)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    sx = torch.from_numpy(cap.sensor_xyz).to(cuda)
    got = ctx.backproject_exhaustive(info, cube, lx, sx).double()
    with reference_weights(ctx):
        want = ctx.backproject_exhaustive(info, cube, lx, sx).double()
    ctx.check_device_status()
    assert float(want.abs().max()) > 0
    assert rel_l2(got.cpu().numpy(), want.cpu().numpy()) < 1e-6


def test_exhaustive_benchmark_size_largest_voxels_vs_fp64(ctx, cuda):
    """The exhaustive benchmark workload (16^2 lasers x 32^2 SPADs x 1024 bins,
    FP16 -> 128^3) on its 100 largest voxels and 100 random ones, against the
    FP64 oracle with the GPU's bins: 1e-6 relative L2."""
    import torch
    from fasterbackprojection_gb300 import FBP_EXHAUSTIVE, make_info, scenes

    cap = scenes.exhaustive_points_torch(16, 32, 1024, 16e-12, n_points=500, seed=3, device=cuda)
    vres = (128, 128, 128)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 1.5))
    info = make_info(num_laser_targets=256, num_sensor_targets=1024, num_time_bins=1024, time_step=cap.time_step,
                     voxel_res=vres, hidden_min=hmin, voxel_size=vs, capture_system=FBP_EXHAUSTIVE)
    cube16 = cap.cube.to(torch.float16).contiguous()
    vol = ctx.backproject_exhaustive(info, cube16, cap.laser_xyz, cap.sensor_xyz).view(-1)
    ctx.check_device_status()
    top = torch.topk(vol, 100).indices
    rnd = torch.from_numpy(np.random.default_rng(6).choice(vol.numel(), 100, replace=False)).to(cuda)
    idx = torch.sort(torch.unique(torch.cat([top, rnd]))).values
    bins = ctx.debug_exhaustive_bins(info, cap.laser_xyz, cap.sensor_xyz, idx).cpu().numpy()
    want = cpu.exhaustive_voxel_subset(info, cube16.float().cpu().numpy().reshape(256 * 1024, 1024),
                                       cap.laser_xyz.cpu().numpy(), cap.sensor_xyz.cpu().numpy(), idx.cpu().numpy(),
                                       bins=bins.reshape(len(idx), -1))
    got = vol[idx].double().cpu().numpy()
    assert rel_l2(got, want) < 1e-6


def test_exhaustive_fp16_storage(ctx, cuda):
    import torch
    from fasterbackprojection_gb300 import FBP_EXHAUSTIVE, make_info, scenes

    cap = scenes.exhaustive_points(3, 4, 512, 32e-12, n_points=25, seed=31)
    L, S, T = cap.cube.shape
    vres = (16, 16, 16)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 2.0))
    info = make_info(num_laser_targets=L, num_sensor_targets=S, num_time_bins=T, time_step=cap.time_step,
                     voxel_res=vres, hidden_min=hmin, voxel_size=vs, capture_system=FBP_EXHAUSTIVE)
    cube = torch.from_numpy(cap.cube).to(cuda).half()
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    sx = torch.from_numpy(cap.sensor_xyz).to(cuda)
    got = ctx.backproject_exhaustive(info, cube, lx, sx).cpu().numpy()
    bins = ctx.debug_exhaustive_bins(info, lx, sx, torch.arange(16 ** 3, device=cuda)).cpu().numpy()
    want = cpu.exhaustive_voxel(info, cube.float().cpu().numpy(), cap.laser_xyz, cap.sensor_xyz, bins=bins)
    assert rel_l2(got, want) < 1e-6


def test_depth_planes_vs_oracle(ctx, cuda):
    import torch
    from fasterbackprojection_gb300 import make_info, scenes
    from fasterbackprojection_gb300.api import linear_space

    cap = scenes.confocal_points(10, 512, 32e-12, n_points=30, seed=41)
    L, T = cap.cube.shape
    info = make_info(num_laser_targets=L, num_time_bins=T, time_step=cap.time_step, voxel_res=(1, 1, 1),
                     hidden_min=(0, 0, 0), voxel_size=(1, 1, 1))
    depths = linear_space(0.6, 1.0, 50)
    got = ctx.backproject_depths(info, torch.from_numpy(cap.cube).to(cuda), torch.from_numpy(cap.laser_xyz).to(cuda),
                                 torch.from_numpy(depths).to(cuda)).cpu().numpy()
    want = cpu.depth_confocal(info, cap.cube, cap.laser_xyz, depths)
    assert rel_l2(got, want) < 1e-3
