"""The single-capture pipeline (confocal backprojection, LoG, min-max
normalisation) records into a CUDA graph after one warm-up call: no host
synchronisation or allocation inside the calls, and a replay re-reads the
inputs."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
def test_confocal_pipeline_replays_from_a_cuda_graph(ctx, cuda, dtype):
    import torch
    from fasterbackprojection_gb300 import FBP_FILTER_LOG, make_info, scenes

    cap = scenes.confocal_points(16, 512, 32e-12, n_points=40, seed=21)
    vres = (24, 20, 28)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 2.0))
    info = make_info(num_laser_targets=256, num_time_bins=512, time_step=cap.time_step, voxel_res=vres,
                     hidden_min=hmin, voxel_size=vs)
    cube = torch.from_numpy(cap.cube).to(cuda)
    if dtype == "bf16":
        cube = cube.to(torch.bfloat16)
    lx = torch.from_numpy(cap.laser_xyz).to(cuda)
    vol = torch.empty((28, 20, 24), device=cuda)
    out = torch.empty_like(vol)

    def step():
        ctx.backproject_confocal(info, cube, lx, out=vol)
        ctx.postfilter(FBP_FILTER_LOG, vol, 5, 1.0, out=out)
        ctx.normalize_(out)

    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        step()  # warm-up: workspaces and tables are allocated here
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    vol_eager, out_eager = vol.clone(), out.clone()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        step()
    cube.mul_(2)  # exact in both dtypes: every stage scales by exactly 2 or is scale-free
    g.replay()
    torch.cuda.synchronize()
    ctx.check_device_status()
    assert torch.equal(vol, 2 * vol_eager)
    assert torch.equal(out, out_eager)
