"""Sampled (MIS) backprojection: the reference's one-sample MIS arithmetic
against its compiled kernel, and unbiasedness of the new estimators."""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _case(n=16, T=512, vres=(24, 20, 28), seed=11):
    from fasterbackprojection_gb300 import make_info, scenes

    cap = scenes.confocal_points(n, T, 32e-12, n_points=60, seed=seed)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 2.4))
    info = make_info(num_laser_targets=n * n, num_time_bins=T, time_step=cap.time_step, voxel_res=vres,
                     hidden_min=hmin, voxel_size=vs)
    return cap, info


def test_reference_mis_matches_reference_kernel_one_sample(ctx, cuda):
    """One sample per voxel (the reference kernel's += only races with more)."""
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_REFERENCE
    from oracle import harness

    if not harness.available():
        pytest.skip("reference kernel harness not built")
    harness.load()
    cap, info = _case()
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    cdf, alias, prob = ctx.mis_reference_tables(info, cube)
    assert cdf[0] == 0.0 and cdf[-1] == pytest.approx(1.0)
    V = 24 * 20 * 28
    noise = torch.rand(V, generator=torch.Generator().manual_seed(5)).to(cuda)
    got = ctx.mis_backproject(info, cube, lx, FBP_MIS_REFERENCE, 1, noise=noise)
    ref = harness.confocal_voxel_mis(info, cube.t().contiguous(), lx, torch.from_numpy(cdf).to(cuda), noise,
                                     torch.from_numpy(alias.astype(np.int32)).to(cuda),
                                     torch.from_numpy(prob).to(cuda), 1)
    assert torch.equal(got, ref)


def test_reference_mis_many_samples_is_deterministic(ctx, cuda):
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_REFERENCE

    cap, info = _case()
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    a = ctx.mis_backproject(info, cube, lx, FBP_MIS_REFERENCE, 0)  # 0 = L/4 samples, default noise
    b = ctx.mis_backproject(info, cube, lx, FBP_MIS_REFERENCE, 0)
    assert torch.equal(a, b) and float(a.abs().max()) > 0


@pytest.mark.parametrize("samples", [1, 7, 64, 300])
def test_reference_mis_many_samples_match_oracle(ctx, cuda, samples):
    """The sum over samples of the reference's one-sample terms (its own
    kernel races on `+=` beyond one sample), against the FP64 restatement with
    the GPU's time bins: chunks of 256 samples, a ragged last chunk, and fewer
    samples than a warp."""
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_REFERENCE
    from oracle import numpy_ref

    cap, info = _case()
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    cdf, alias, prob = ctx.mis_reference_tables(info, cube)
    V = 24 * 20 * 28
    noise = torch.rand(V + 17, generator=torch.Generator().manual_seed(6)).to(cuda)
    got = ctx.mis_backproject(info, cube, lx, FBP_MIS_REFERENCE, samples, noise=noise).cpu().numpy()
    bins = ctx.debug_confocal_bins(info, lx, torch.arange(V, device=cuda)).cpu().numpy()
    want = numpy_ref.mis_reference(info, cap.cube, cap.laser_xyz, cdf, alias, prob, noise.cpu().numpy(), samples,
                                   bins=bins)
    assert float(np.abs(want).max()) > 0
    assert rel_l2(got, want) < 1e-6


def _scatter_case(seed=11):
    # 2.4 m deep volume in 28 slices: a voxel diagonal of ~12 cm, walks of
    # 10-13 bins of 9.6 mm.
    return _case(seed=seed)


def test_reference_mis_scatter_matches_reference_build_one_sample(ctx, cuda):
    """The voxel-scattering build of the reference's MIS kernel: with one
    sample per voxel each voxel's atomic adds come from one thread in bin
    order, so its volume is deterministic and must match bit for bit."""
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_REFERENCE_SCATTER
    from oracle import harness

    if not harness.scatter_available():
        pytest.skip("reference scatter build not present")
    harness.load()
    cap, info = _scatter_case()
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    cdf, alias, prob = ctx.mis_reference_tables(info, cube)
    V = 24 * 20 * 28
    noise = torch.rand(V, generator=torch.Generator().manual_seed(7)).to(cuda)
    got = ctx.mis_backproject(info, cube, lx, FBP_MIS_REFERENCE_SCATTER, 1, noise=noise)
    ref = harness.confocal_voxel_mis_scatter(info, cube.t().contiguous(), lx, torch.from_numpy(cdf).to(cuda), noise,
                                             torch.from_numpy(alias.astype(np.int32)).to(cuda),
                                             torch.from_numpy(prob).to(cuda), 1)
    ctx.check_device_status()
    assert float(ref.abs().max()) > 0
    assert torch.equal(got, ref)


@pytest.mark.parametrize("samples", [16, 64])
def test_reference_mis_scatter_many_samples_match_reference_build(ctx, cuda, samples):
    """Many samples: the reference adds with atomics (any order), so the
    volumes agree to 1e-5 relative L2."""
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_REFERENCE_SCATTER
    from oracle import harness

    if not harness.scatter_available():
        pytest.skip("reference scatter build not present")
    harness.load()
    cap, info = _scatter_case(seed=12)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    cdf, alias, prob = ctx.mis_reference_tables(info, cube)
    V = 24 * 20 * 28
    noise = torch.rand(V + 5, generator=torch.Generator().manual_seed(8)).to(cuda)
    got = ctx.mis_backproject(info, cube, lx, FBP_MIS_REFERENCE_SCATTER, samples, noise=noise)
    ref = harness.confocal_voxel_mis_scatter(info, cube.t().contiguous(), lx, torch.from_numpy(cdf).to(cuda), noise,
                                             torch.from_numpy(alias.astype(np.int32)).to(cuda),
                                             torch.from_numpy(prob).to(cuda), samples)
    ctx.check_device_status()
    assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) < 1e-5


@pytest.mark.parametrize("samples", [1, 37, 300])
def test_reference_mis_scatter_match_oracle(ctx, cuda, samples):
    """Against numpy_ref.mis_reference(scatter=True): its float32 replay of
    the walk from the GPU's FP32 paths (the same bins, FP64 sums) within 1e-6,
    and its independent FP64 walk within 1e-2 (walks whose ends land within an
    FP32 rounding of a bin edge differ by a bin)."""
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_REFERENCE_SCATTER
    from oracle import numpy_ref

    cap, info = _scatter_case(seed=13)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    cdf, alias, prob = ctx.mis_reference_tables(info, cube)
    V = 24 * 20 * 28
    noise = torch.rand(V + 3, generator=torch.Generator().manual_seed(9)).to(cuda)
    got = ctx.mis_backproject(info, cube, lx, FBP_MIS_REFERENCE_SCATTER, samples, noise=noise).cpu().numpy()
    paths, consts = ctx.debug_confocal_paths(info, lx, torch.arange(V, device=cuda))
    ctx.check_device_status()
    nz = noise.cpu().numpy()
    want = numpy_ref.mis_reference(info, cap.cube, cap.laser_xyz, cdf, alias, prob, nz, samples, scatter=True,
                                   paths=paths.cpu().numpy(), consts=consts)
    assert float(np.abs(want).max()) > 0
    assert rel_l2(got, want) < 1e-6
    want64 = numpy_ref.mis_reference(info, cap.cube, cap.laser_xyz, cdf, alias, prob, nz, samples, scatter=True)
    assert rel_l2(got, want64) < 1e-2


@pytest.mark.parametrize("proposal", ["uniform", "spatial", "clusters", "clusters_cv"])
def test_unbiased_estimators_converge_to_full_backprojection(ctx, cuda, proposal):
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_LEARNED, FBP_MIS_SPATIAL, FBP_MIS_UNIFORM
    from fasterbackprojection_gb300.api import mis_tile_grid

    cap, info = _case(seed=13)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    full = ctx.backproject_confocal(info, cube, lx).double()
    kw = {}
    mode = {"uniform": FBP_MIS_UNIFORM, "spatial": FBP_MIS_SPATIAL, "clusters": FBP_MIS_LEARNED,
            "clusters_cv": FBP_MIS_LEARNED}[proposal]
    if proposal.startswith("clusters"):
        tiles = mis_tile_grid(info)
        G = 16  # 4 x 4 clusters of 4 x 4 scan points
        rng = np.random.default_rng(0)
        w = rng.uniform(0.2, 1.0, (int(np.prod(tiles)), G))
        cdf = np.cumsum(w / w.sum(1, keepdims=True), axis=1).astype(np.float32)
        cdf[:, -1] = 1.0
        kw = dict(tile_cluster_cdf=torch.from_numpy(cdf).to(cuda), cluster_side=4, scan_side=16,
                  cv_side=2 if proposal == "clusters_cv" else 0)
    K = 4 if proposal.startswith("clusters") else 64  # clusters of 16 scan points each
    runs = 200
    acc = torch.zeros_like(full)
    single = None
    for r in range(runs):
        est = ctx.mis_backproject(info, cube, lx, mode, K, seed=1000 + r, **kw).double()
        if single is None:
            single = rel_l2(est.cpu().numpy(), full.cpu().numpy())
        acc += est
    mean_err = rel_l2((acc / runs).cpu().numpy(), full.cpu().numpy())
    # Averaging R independent unbiased estimates shrinks the error ~ 1/sqrt(R).
    assert mean_err < 2.5 * single / np.sqrt(runs), (single, mean_err)


def test_more_samples_lower_error(ctx, cuda):
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_SPATIAL

    cap, info = _case(seed=17)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    full = ctx.backproject_confocal(info, cube, lx).cpu().numpy()
    errs = [rel_l2(ctx.mis_backproject(info, cube, lx, FBP_MIS_SPATIAL, K, seed=3).cpu().numpy(), full)
            for K in (16, 64, 256)]
    assert errs[0] > errs[1] > errs[2]


def test_control_variate_with_every_cluster_is_the_full_backprojection(ctx, cuda):
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_LEARNED

    cap, info = _case(seed=19)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    full = ctx.backproject_confocal(info, cube, lx).cpu().numpy()
    # K = G = 16 uniform: every cluster once, the control variate cancels.
    got = ctx.mis_backproject(info, cube, lx, FBP_MIS_LEARNED, 16, seed=3, cluster_side=4, scan_side=16, cv_side=2)
    ctx.check_device_status()
    assert rel_l2(got.cpu().numpy(), full) < 1e-5


def test_ragged_edge_clusters_with_every_cluster_are_the_full_backprojection(ctx, cuda):
    """A 20 x 20 scan in 8 x 8 clusters: the last row and column of clusters
    reach past the grid; their missing points are read as zeros.  With
    K = G = 9 uniform draws every cluster is gathered once with weight 1."""
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_LEARNED

    cap, info = _case(n=20, seed=27)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    full = ctx.backproject_confocal(info, cube, lx).cpu().numpy()
    got = ctx.mis_backproject(info, cube, lx, FBP_MIS_LEARNED, 9, seed=5, cluster_side=8, scan_side=20)
    ctx.check_device_status()
    got = got.cpu().numpy()
    assert np.isfinite(got).all()
    assert rel_l2(got, full) < 1e-5


def test_control_variate_lowers_the_error(ctx, cuda):
    """Dense scan (64^2 points, 3.1 cm pitch): the 2 x 2-point block sums
    track the real contributions, so the residual estimator beats plain
    cluster sampling at the same 8 of 64 clusters per tile."""
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_LEARNED, make_info, scenes

    n = 64
    cap = scenes.confocal_points(n, 512, 32e-12, n_points=60, seed=23)
    hmin, vs = scenes.volume_geometry((32, 32, 32), depth_range=(0.0, 1.5))
    info = make_info(num_laser_targets=n * n, num_time_bins=512, time_step=cap.time_step, voxel_res=(32, 32, 32),
                     hidden_min=hmin, voxel_size=vs)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    full = ctx.backproject_confocal(info, cube, lx).cpu().numpy()
    plain, cv = [], []
    for seed in range(6):
        plain.append(rel_l2(ctx.mis_backproject(info, cube, lx, FBP_MIS_LEARNED, 8, seed=seed, cluster_side=8,
                                                scan_side=n).cpu().numpy(), full))
        cv.append(rel_l2(ctx.mis_backproject(info, cube, lx, FBP_MIS_LEARNED, 8, seed=seed, cluster_side=8,
                                             scan_side=n, cv_side=2).cpu().numpy(), full))
    ctx.check_device_status()
    assert np.mean(cv) < 0.7 * np.mean(plain), (np.mean(cv), np.mean(plain))
