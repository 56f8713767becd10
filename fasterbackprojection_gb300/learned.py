"""Training and use of the learned MIS proposal (host side of fbp_mlp_*).

The network scores (voxel tile, scan cluster) pairs; FBP_MIS_LEARNED then
draws whole clusters per tile from the resulting distribution.  Training data
are full-backprojection targets of seeded point scenes (64 x 64 scan points,
512 bins of 32 ps, 200 points at depth U[0.4, 1.2] m, Poisson noise at 1e4
photons per scan point) over the evaluation volume's tile geometry; clusters
have the same physical size at every scan resolution (12.5 cm squares: 4 x 4
points at 64^2, 16 x 16 at 256^2), so G = 256 clusters in both.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from . import _lib
from .api import Context, Mlp, make_info
from . import scenes


@dataclass
class TrainingSet:
    features: object  # [samples][G][FBP_MLP_FEATURES] float32 (device)
    labels: object    # [samples][G] float32 (device)
    scenes: int
    seconds: float


def point_scene_info(n: int, T: int, time_step: float, vres, depth_range=(0.0, 1.5)):
    hmin, vs = scenes.volume_geometry(vres, depth_range=depth_range)
    return make_info(num_laser_targets=n * n, num_time_bins=T, time_step=time_step, voxel_res=vres,
                     hidden_min=hmin, voxel_size=vs)


def build_training_set(ctx: Context, seeds, vres=(256, 256, 256), n: int = 64, T: int = 512, dt_s: float = 32e-12,
                       cluster_side: int = 4, tiles_per_scene: int = 64, device="cuda") -> TrainingSet:
    """Features and targets of `tiles_per_scene` random tiles of each scene."""
    import torch

    t0 = time.perf_counter()
    feats, labels = [], []
    for s in seeds:
        cap = scenes.confocal_points_torch(n, T, dt_s, seed=int(s), device=device)
        info = point_scene_info(n, T, cap.time_step, vres)
        nt = ctx.mlp_tile_count(info)
        rng = np.random.default_rng(int(s))
        tiles = torch.from_numpy(rng.choice(nt, min(tiles_per_scene, nt), replace=False).astype(np.int32)).to(device)
        feats.append(ctx.mlp_features(info, cap.cube, cap.laser_xyz, cluster_side, n, tiles=tiles))
        labels.append(ctx.mlp_labels(info, cap.cube, cap.laser_xyz, cluster_side, n, tiles))
    F = torch.cat(feats)
    Q = torch.cat(labels)
    torch.cuda.synchronize()
    ctx.check_device_status()
    return TrainingSet(F, Q, len(seeds), time.perf_counter() - t0)


def train(ctx: Context, mlp: Mlp, data: TrainingSet, epochs: int = 3, batch: int = 256, lr: float = 2e-3,
          seed: int = 0):
    """Adam over shuffled minibatches of tiles; returns (losses per epoch,
    seconds).  The losses are the full-set cross-entropy after each epoch."""
    import torch

    dev = data.features.device
    n = data.features.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    all_idx = torch.arange(n, dtype=torch.int32, device=dev)
    losses = [float(mlp.gradients(data.features, data.labels, all_idx)[-1])]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(epochs):
        perm = torch.randperm(n, generator=g).to(torch.int32).to(dev)
        for i in range(0, n - batch + 1, batch):
            mlp.train_step(data.features, data.labels, perm[i:i + batch], lr)
        torch.cuda.synchronize()
        losses.append(float(mlp.gradients(data.features, data.labels, all_idx)[-1]))
    ctx.check_device_status()
    return losses, time.perf_counter() - t0


def proposal(ctx: Context, mlp: Mlp, info, cube, laser_xyz, cluster_side: int, scan_side: int,
             defensive: float = 0.1, layout=_lib.FBP_LAYOUT_TIME_INNER, stream=None):
    """Per-tile inclusive CDF over clusters for a capture."""
    f = ctx.mlp_features(info, cube, laser_xyz, cluster_side, scan_side, layout=layout, stream=stream)
    _, cdf = mlp.forward(f, logits=False, defensive=defensive, cdf=True, stream=stream)
    return cdf


def main(argv=None) -> int:
    """Train the proposal on point scenes and evaluate it on a seeded
    256^2 x 1024 patch capture (BF16):
    python -m fasterbackprojection_gb300.learned --scenes 2000 --out w.npy"""
    import argparse
    import json

    import torch

    from . import FBP_MIS_LEARNED

    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--samples", type=int, default=8, help="clusters per voxel tile")
    ap.add_argument("--scan", type=int, default=256)
    ap.add_argument("--out", default=None, help="save the trained parameters (.npy)")
    a = ap.parse_args(argv)
    dev = torch.device("cuda", 0)
    ctx = Context(0)
    vres = (a.scan, a.scan, a.scan)
    data = build_training_set(ctx, range(10000, 10000 + a.scenes), vres=vres, device=dev)
    mlp = Mlp(ctx, seed=7)
    losses, train_s = train(ctx, mlp, data, epochs=a.epochs)
    if a.out:
        np.save(a.out, mlp.get_params())
    cap = scenes.confocal_patches_torch(a.scan, 1024, 16e-12, seed=2, device=dev)
    info = point_scene_info(a.scan, 1024, cap.time_step, vres)
    cube = cap.cube.to(torch.bfloat16)
    full = ctx.backproject_confocal(info, cube, cap.laser_xyz).double()
    cs = a.scan // 16
    cdf = proposal(ctx, mlp, info, cube, cap.laser_xyz, cs, a.scan)
    est = ctx.mis_backproject(info, cube, cap.laser_xyz, FBP_MIS_LEARNED, a.samples, seed=0, tile_cluster_cdf=cdf,
                              cluster_side=cs, scan_side=a.scan, cv_side=max(1, cs // 4)).double()
    ctx.check_device_status()
    err = float(torch.linalg.vector_norm(est - full) / torch.linalg.vector_norm(full))
    print(json.dumps({"scenes": a.scenes, "losses": losses, "train_s": train_s, "data_s": data.seconds,
                      "samples": a.samples, "rel_l2_vs_full": err}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
