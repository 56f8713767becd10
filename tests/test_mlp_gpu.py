"""Learned MIS proposal: the tensor-core MLP kernels (forward, gradients,
Adam), its features and targets, and the cluster-sampled estimator, against
the CPU oracle (oracle/mlp_ref.py).

Tolerances: the GPU rounds every tensor-core operand to BF16 and accumulates
in FP32; the oracle rounds at the same points and accumulates in FP64, so the
two differ where an FP32 and an FP64 value round to neighbouring BF16 values
(one BF16 ulp, 2^-8 relative, in a few activations).  Logits: rel-L2 <= 4e-3;
gradients: rel-L2 <= 2e-2 per parameter block; loss: 1e-3 relative.
"""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _random_params(seed=0):
    from oracle import mlp_ref

    rng = np.random.default_rng(seed)
    p = np.zeros(mlp_ref.NPARAM, np.float32)
    p[mlp_ref.OW1:mlp_ref.OB1] = (rng.uniform(-0.4, 0.4, (64, 32)) * (np.arange(32) < 19)).ravel()
    p[mlp_ref.OB1:mlp_ref.OW2] = rng.uniform(-0.1, 0.1, 64)
    p[mlp_ref.OW2:mlp_ref.OB2] = rng.uniform(-0.2, 0.2, 64 * 64)
    p[mlp_ref.OB2:mlp_ref.OW3] = rng.uniform(-0.1, 0.1, 64)
    p[mlp_ref.OW3:mlp_ref.OB3] = rng.uniform(-0.2, 0.2, 64 * 64)
    p[mlp_ref.OB3:mlp_ref.OW4] = rng.uniform(-0.1, 0.1, 64)
    p[mlp_ref.OW4:mlp_ref.OB4] = rng.uniform(-0.3, 0.3, 64)
    p[mlp_ref.OB4] = 0.05
    return p


def _random_rows(B, G, seed=1):
    rng = np.random.default_rng(seed)
    f = np.zeros((B, G, 20), np.float32)
    f[..., 0:3] = rng.uniform(-0.8, 0.8, (B, G, 3))
    f[..., 3:19] = rng.exponential(0.7, (B, G, 16))
    q = rng.exponential(1.0, (B, G)) ** 3
    q /= q.sum(axis=1, keepdims=True)
    return f, q.astype(np.float32)


@pytest.mark.parametrize("G", [256, 200, 64])
def test_forward_matches_oracle(ctx, cuda, G):
    import torch

    from fasterbackprojection_gb300 import Mlp
    from oracle import mlp_ref

    m = Mlp(ctx, seed=3)
    p = _random_params(4)
    m.set_params(p)
    f, _ = _random_rows(3, G)
    ft = torch.from_numpy(f).to(cuda)
    logits, cdf = m.forward(ft, logits=True, defensive=0.1, cdf=True)
    torch.cuda.synchronize()
    ctx.check_device_status()
    want, _ = mlp_ref.forward(p, f.astype(np.float64))
    got = logits.cpu().numpy()
    assert rel_l2(got, want) < 4e-3, rel_l2(got, want)
    # CDF of 0.9 softmax + 0.1 uniform.
    e = np.exp(want - want.max(axis=1, keepdims=True))
    pw = 0.9 * e / e.sum(axis=1, keepdims=True) + 0.1 / G
    c = cdf.cpu().numpy()
    assert np.all(np.diff(c, axis=1) > 0) and np.all(c[:, -1] == 1.0)
    np.testing.assert_allclose(c, np.cumsum(pw, axis=1), atol=2e-3)
    m.close()


def test_gradients_match_oracle_and_are_deterministic(ctx, cuda):
    import torch

    from fasterbackprojection_gb300 import Mlp
    from oracle import mlp_ref

    m = Mlp(ctx, seed=5)
    p = _random_params(6)
    m.set_params(p)
    G = 200
    f, q = _random_rows(6, G, seed=7)
    ft = torch.from_numpy(f).to(cuda)
    qt = torch.from_numpy(q).to(cuda)
    idx = torch.tensor([4, 0, 5, 2], dtype=torch.int32, device=cuda)
    g1 = m.gradients(ft, qt, idx)
    g2 = m.gradients(ft, qt, idx)
    torch.cuda.synchronize()
    ctx.check_device_status()
    assert torch.equal(g1, g2)
    got = g1.cpu().numpy()
    sel = [4, 0, 5, 2]
    loss, want = mlp_ref.loss_and_grad(p, f[sel].astype(np.float64), q[sel].astype(np.float64))
    assert got[-1] == pytest.approx(loss, rel=1e-3)
    blocks = {"W1": (mlp_ref.OW1, mlp_ref.OB1), "b1": (mlp_ref.OB1, mlp_ref.OW2), "W2": (mlp_ref.OW2, mlp_ref.OB2),
              "b2": (mlp_ref.OB2, mlp_ref.OW3), "W3": (mlp_ref.OW3, mlp_ref.OB3), "b3": (mlp_ref.OB3, mlp_ref.OW4),
              "w4": (mlp_ref.OW4, mlp_ref.OB4)}
    for name, (a, b) in blocks.items():
        assert rel_l2(got[a:b], want[a:b]) < 2e-2, (name, rel_l2(got[a:b], want[a:b]))
    # d loss / d b4 = sum(softmax - q) = 0 up to rounding.
    assert abs(got[mlp_ref.OB4]) < 1e-5 and abs(want[mlp_ref.OB4]) < 1e-8
    m.close()


def test_adam_step_moves_against_the_gradient(ctx, cuda):
    import torch

    from fasterbackprojection_gb300 import Mlp

    m = Mlp(ctx, seed=8)
    p0 = m.get_params()
    f, q = _random_rows(4, 64, seed=9)
    ft = torch.from_numpy(f).to(cuda)
    qt = torch.from_numpy(q).to(cuda)
    idx = torch.arange(4, dtype=torch.int32, device=cuda)
    g = m.gradients(ft, qt, idx).cpu().numpy()[:-1]
    loss = torch.zeros(1, device=cuda)
    m.train_step(ft, qt, idx, 1e-3, loss=loss)
    p1 = m.get_params()
    step = p1 - p0
    # First Adam step: -lr * sign(g) wherever the gradient is not tiny.
    big = np.abs(g) > 1e-4
    np.testing.assert_allclose(step[big], -1e-3 * np.sign(g[big]), rtol=1e-3, atol=1e-7)
    assert float(loss) > 0
    m.close()


def _point_capture(n, T, seed, vres=(64, 48, 40)):
    from fasterbackprojection_gb300 import make_info, scenes

    cap = scenes.confocal_points(n, T, 32e-12, n_points=60, seed=seed)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 1.5))
    info = make_info(num_laser_targets=n * n, num_time_bins=T, time_step=cap.time_step, voxel_res=vres,
                     hidden_min=hmin, voxel_size=vs)
    return cap, info


def test_features_match_oracle(ctx, cuda):
    import torch

    from oracle import mlp_ref

    cap, info = _point_capture(16, 512, 21)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    assert ctx.mlp_tile_count(info) == 72
    tiles = np.array([0, 5, 17, 40, 71], np.int32)
    got = ctx.mlp_features(info, cube, lx, 4, 16, tiles=torch.from_numpy(tiles).to(cuda)).cpu().numpy()
    want = mlp_ref.features(info, cap.cube, cap.laser_xyz, 16, 4, tiles)
    assert got.shape == want.shape == (5, 16, 20)
    np.testing.assert_allclose(got[..., :3], want[..., :3], atol=1e-6)
    # Pooled bins: rows whose window position rounds differently may shift.
    close = np.all(np.abs(got[..., 3:] - want[..., 3:]) < 1e-4, axis=-1)
    assert close.mean() > 0.97, close.mean()
    # All tiles at once equals the listed ones.
    every = ctx.mlp_features(info, cube, lx, 4, 16).cpu().numpy()
    np.testing.assert_array_equal(every[tiles], got)


def test_labels_match_oracle(ctx, cuda):
    import torch

    from oracle import mlp_ref

    cap, info = _point_capture(16, 512, 22)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    tiles = np.array([3, 30, 71], np.int32)
    got = ctx.mlp_labels(info, cube, lx, 4, 16, torch.from_numpy(tiles).to(cuda)).cpu().numpy()
    want = mlp_ref.labels(info, cap.cube, cap.laser_xyz, 16, 4, tiles)
    np.testing.assert_allclose(got.sum(axis=1), 1.0, rtol=1e-5)
    for i in range(len(tiles)):
        assert rel_l2(got[i], want[i]) < 1e-3, (i, rel_l2(got[i], want[i]))


def test_cluster_sampling_with_every_cluster_is_the_full_backprojection(ctx, cuda):
    import torch

    from fasterbackprojection_gb300 import FBP_MIS_LEARNED

    cap, info = _point_capture(16, 512, 23)
    cube = torch.from_numpy(cap.cube).to(cuda)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    full = ctx.backproject_confocal(info, cube, lx).cpu().numpy()
    # Uniform over 16 clusters with K = 16: every cluster exactly once, weight 1.
    got = ctx.mis_backproject(info, cube, lx, FBP_MIS_LEARNED, 16, seed=5, cluster_side=4, scan_side=16)
    assert rel_l2(got.cpu().numpy(), full) < 1e-5


def test_trained_proposal_beats_uniform_clusters(ctx, cuda):
    """Training on point scenes lowers the loss, and on held-out scenes the
    learned proposal's MIS error at 8 of 64 clusters per tile is below the
    uniform-cluster estimator's (the method without the network)."""
    import torch

    from fasterbackprojection_gb300 import FBP_MIS_LEARNED, Mlp

    n, cs, T = 32, 4, 512
    feats, labels = [], []
    rng = np.random.default_rng(0)
    for s in range(24):
        cap, info = _point_capture(n, T, 100 + s)
        cube = torch.from_numpy(cap.cube).to(cuda)
        lx = torch.from_numpy(cap.laser_xyz).to(cuda)
        nt = ctx.mlp_tile_count(info)
        tiles = torch.from_numpy(rng.choice(nt, 24, replace=False).astype(np.int32)).to(cuda)
        feats.append(ctx.mlp_features(info, cube, lx, cs, n, tiles=tiles))
        labels.append(ctx.mlp_labels(info, cube, lx, cs, n, tiles))
    F = torch.cat(feats)
    Q = torch.cat(labels)
    m = Mlp(ctx, seed=1)
    all_idx = torch.arange(F.shape[0], dtype=torch.int32, device=cuda)
    loss0 = float(m.gradients(F, Q, all_idx)[-1])
    g = torch.Generator(device="cpu").manual_seed(0)
    for it in range(400):
        idx = torch.randperm(F.shape[0], generator=g)[:64].to(torch.int32).to(cuda)
        m.train_step(F, Q, idx, 2e-3)
    loss1 = float(m.gradients(F, Q, all_idx)[-1])
    assert loss1 < 0.9 * loss0, (loss0, loss1)

    errs_l, errs_u = [], []
    for s in range(3):
        cap, info = _point_capture(n, T, 900 + s)
        cube = torch.from_numpy(cap.cube).to(cuda)
        lx = torch.from_numpy(cap.laser_xyz).to(cuda)
        full = ctx.backproject_confocal(info, cube, lx).cpu().numpy()
        f = ctx.mlp_features(info, cube, lx, cs, n)
        _, cdf = m.forward(f, logits=False, defensive=0.1, cdf=True)
        for seed in range(4):
            el = ctx.mis_backproject(info, cube, lx, FBP_MIS_LEARNED, 8, seed=seed, tile_cluster_cdf=cdf,
                                     cluster_side=cs, scan_side=n).cpu().numpy()
            eu = ctx.mis_backproject(info, cube, lx, FBP_MIS_LEARNED, 8, seed=seed, cluster_side=cs,
                                     scan_side=n).cpu().numpy()
            errs_l.append(rel_l2(el, full))
            errs_u.append(rel_l2(eu, full))
    ctx.check_device_status()
    assert np.mean(errs_l) < 0.8 * np.mean(errs_u), (np.mean(errs_l), np.mean(errs_u))
    m.close()
