"""Batched confocal reconstruction (fbp_batch_*) against the single-capture
gather and the FP64 oracle.

  * tile shape 0 is the single-capture gather's tile, so every volume of a
    batch equals fbp_backproject_confocal's bit for bit;
  * the other tile shapes regroup the scan points into different stages, so
    they agree to 1e-6 relative L2 (FP32 stage sums + Kahan fold);
  * a graph replay re-reads the cubes (changing a cube in place changes the
    replayed result) and equals a plain run bit for bit.
"""
import numpy as np
import pytest

from oracle import cpu
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

# (scan side, T, voxel_res, discard, t0, layout)
CASES = [
    (12, 512, (28, 24, 32), 1, 0.0, 1),
    (8, 256, (16, 16, 16), 0, 0.0, 1),
    (16, 384, (20, 36, 12), 1, 0.3, 0),
    (10, 640, (40, 8, 24), 1, 0.0, 0),
    (6, 128, (9, 7, 5), 0, 0.0, 1),
]


def _captures(cuda, dtype=None, cases=CASES, seed0=30):
    import torch

    from fasterbackprojection_gb300 import make_info, scenes

    out = []
    for i, (n, T, vres, discard, t0, layout) in enumerate(cases):
        cap = scenes.confocal_points(n, T, 32e-12, n_points=30, seed=seed0 + i)
        hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 2.2))
        info = make_info(num_laser_targets=n * n, num_time_bins=T, time_step=cap.time_step, voxel_res=vres,
                         hidden_min=hmin, voxel_size=vs, discard_first_last_bounces=discard, time_offset=t0,
                         laser_position=(0.05, -0.25, 0.1), sensor_position=(-0.1, -0.2, 0.05))
        cube = torch.from_numpy(cap.cube).to(cuda)  # [L][T]
        if layout == 0:
            cube = cube.t().contiguous()  # [T][L]
        if dtype is not None:
            cube = cube.to(dtype)
        lx = torch.from_numpy(cap.laser_xyz).to(cuda)
        vol = torch.full((vres[2], vres[1], vres[0]), float("nan"), device=cuda)
        out.append(dict(info=info, cube=cube, lx=lx, vol=vol, layout=layout, host=cap))
    return out


def _batch(ctx, caps):
    from fasterbackprojection_gb300 import Batch

    return Batch(ctx, [(c["info"], c["cube"], c["lx"], c["vol"], c["layout"]) for c in caps])


@pytest.mark.parametrize("dtype", [None, "bf16"])
def test_batch_tile0_equals_single_capture_gather(ctx, cuda, dtype):
    import torch

    tdt = {None: None, "bf16": torch.bfloat16}[dtype]
    caps = _captures(cuda, tdt)
    b = _batch(ctx, caps)
    b.run()
    torch.cuda.synchronize()
    ctx.check_device_status()
    for c in caps:
        single = ctx.backproject_confocal(c["info"], c["cube"], c["lx"], layout=c["layout"])
        torch.cuda.synchronize()
        assert torch.equal(c["vol"], single)
    b.close()


def test_batch_tile_shapes_agree_with_oracle(ctx, cuda):
    import torch

    caps = _captures(cuda)
    b = _batch(ctx, caps)
    ref = []
    for c in caps:
        bins = None
        info = c["info"]
        V = info.voxel_res[0] * info.voxel_res[1] * info.voxel_res[2]
        idx = torch.arange(V, dtype=torch.int64, device=cuda)
        bins = ctx.debug_confocal_bins(info, c["lx"], idx).cpu().numpy()
        ref.append(cpu.confocal_voxel(info, c["host"].cube, c["host"].laser_xyz, bins=bins))
    for cfg in range(4):
        b.set_config(cfg)
        b.run()
        torch.cuda.synchronize()
        ctx.check_device_status()
        for c, want in zip(caps, ref):
            assert rel_l2(c["vol"].cpu().numpy(), want) < 1e-6, cfg
    b.close()


def test_batch_graph_replay_rereads_inputs(ctx, cuda):
    import torch

    caps = _captures(cuda)
    b = _batch(ctx, caps)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b.run(use_graph=False, stream=s)
        s.synchronize()
        plain = [c["vol"].clone() for c in caps]
        for c in caps:
            c["vol"].fill_(float("nan"))
        b.run(use_graph=True, stream=s)  # captures, then replays
        s.synchronize()
        for c, p in zip(caps, plain):
            assert torch.equal(c["vol"], p)
        # Scale every cube in place by 2: the replay must see it.
        for c in caps:
            c["cube"].mul_(2.0)
        before = ctx.launches
        b.run(use_graph=True, stream=s)
        s.synchronize()
        assert ctx.launches > before
        for c, p in zip(caps, plain):
            torch.testing.assert_close(c["vol"], 2.0 * p, rtol=1e-6, atol=1e-6 * float(p.abs().max()))
    ctx.check_device_status()
    b.close()


def test_batch_autotune_picks_a_valid_shape(ctx, cuda):
    import torch

    caps = _captures(cuda)
    b = _batch(ctx, caps)
    chosen = b.autotune()
    assert chosen in (0, 1, 2, 3)
    b.run()
    torch.cuda.synchronize()
    for c in caps:
        single = ctx.backproject_confocal(c["info"], c["cube"], c["lx"], layout=c["layout"])
        assert rel_l2(c["vol"].cpu().numpy(), single.cpu().numpy()) < 1e-6
    b.close()


def test_batch_many_uneven_captures(ctx, cuda):
    """40 captures of 4..20 scan side and 64..1024 bins, volumes 3..40."""
    import torch

    rng = np.random.default_rng(3)
    cases = []
    for _ in range(40):
        n = int(rng.integers(4, 21))
        T = int(rng.choice([64, 200, 512, 1024]))
        vres = tuple(int(v) for v in rng.integers(3, 41, size=3))
        cases.append((n, T, vres, int(rng.integers(0, 2)), 0.0, int(rng.integers(0, 2))))
    caps = _captures(cuda, cases=cases, seed0=200)
    b = _batch(ctx, caps)
    b.run()
    torch.cuda.synchronize()
    ctx.check_device_status()
    for c in caps:
        single = ctx.backproject_confocal(c["info"], c["cube"], c["lx"], layout=c["layout"])
        assert torch.equal(c["vol"], single)
    b.close()


def test_batch_rejects_bad_descriptors(ctx, cuda):
    import torch

    from fasterbackprojection_gb300 import Batch, FbpError

    caps = _captures(cuda, cases=CASES[:2])
    caps[1]["cube"] = caps[1]["cube"].to(torch.float16)
    with pytest.raises(FbpError):
        Batch(ctx, [(c["info"], c["cube"], c["lx"], c["vol"], c["layout"]) for c in caps])
    with pytest.raises(FbpError):
        Batch(ctx, [])
