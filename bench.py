#!/usr/bin/env python3
"""Throughput of the confocal reconstruction hot path on GB300.

Workload (one step): confocal full backprojection of a 256 x 256 scan x 1024
bin capture (16 ps bins, FP32 storage) into a 256^3 FP32 volume over
2 x 2 x 1.5 m, then the 5^3 LoG filter (sigma 1 voxel) and min-max
normalisation.  Seeded synthetic scene (8 planar patches, r^-4 falloff,
Poisson noise at 1e4 photons per scan point), generated on the device.
Metric: backprojected voxel-samples/s = (voxels x scan points) per step / time.

  value  device-resident inputs, CUDA-event timed over --steps steps
  e2e    the same step through fbp_reconstruct_shape_host from pinned HOST
         buffers (H2D of the cube, D2H of the volume inside the timed region)

--impl reference times the reference algorithm's CPU form (there is no CPU
backprojection in the reference: the oracle's FP32 restatement of its kernel,
all host cores) on a bounded sample of the same workload.
Multi-GPU (torchrun): each rank reconstructs its own capture (weak scaling, no
collective on the data path); value = all ranks' samples / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_SCAN, N_BINS, DT, VRES = 256, 1024, 16e-12, (256, 256, 256)
METRIC = "Backprojected voxel-samples/s"
UNIT = "voxel-samples/s"
WORKLOAD = "confocal_bp+log_256x256x1024_to_256^3"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", choices=["full", "medium", "small"], default="full",
                    help="full: 256^2 scan -> 256^3 (the benchmark); medium: 128^2 -> 128^3 and small: 64^2 -> 64^3 "
                         "(profiling and plumbing checks)")
    ap.add_argument("--no-extras", action="store_true", help="skip bf16 / reference-CUDA / CPU / batched legs")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-capture batched leg")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-MIS leg")
    ap.add_argument("--no-configs", action="store_true", help="skip the LCT / exhaustive / filter legs")
    ap.add_argument("--mode", choices=["weak", "slabs"], default="weak",
                    help="multi-GPU: weak = one capture per rank; slabs = the same capture split into depth slabs "
                         "(strong scaling; each rank uploads only its slab's bin window in the e2e leg)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg")
    ap.add_argument("--only", choices=["exhaustive", "filters", "lct", "scatter_forms", "batched", "reference_kernels",
                                       "learned"],
                    help="run one extra leg alone on the benchmark capture and print its JSON (profiling runs)")
    a = ap.parse_args()
    a.small = a.size != "full"
    return a


SIZES = {"full": (N_SCAN, VRES), "medium": (128, (128, 128, 128)), "small": (64, (64, 64, 64))}


# ------------------------------------------------------------------ clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ distributed

def dist_setup(backend: str):
    import torch.distributed as dist

    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend)
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, ws: int, device=None) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


# ------------------------------------------------------------------- peaks

def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """dram read+write bytes per launch of the gather kernel from the committed
    ncu summary (profiles/), scaled to the full workload there."""
    p = ROOT / "profiles" / "confocal_gather_256x256x1024_to_256cube.md"
    if not p.exists():
        return None
    m = re.search(r"traffic_per_launch_bytes:\s*([0-9.eE+]+)", p.read_text())
    return float(m.group(1)) if m else None


# Multi-function unit (XU) of an sm_100-class SM: 16 results per clock (4 per
# SM sub-partition).  The confocal pair loop issues one sqrt.approx per pair
# (the reference's bin, irreducible for bit-exact bins) and, with the batched
# weights, one rcp.approx per two pairs.
XU_PER_CLK_SM = 16
MUFU_PER_PAIR = 1.5
MUFU_PER_PAIR_FLOOR = 1.0


def gather_roofline(samples, bp_ms, clocks, hbm_peak, hbm_kind):
    """Roofline of the dominant kernel (the confocal gather).  It is bound by
    the XU (MUFU) pipe and instruction issue, not by HBM: the bound is stated
    in voxel-samples per clock per SM against the XU ceiling of its own
    arithmetic, at the SM clock sampled during the timed region.  The
    bytes-per-sample accounting (4 B, the cube element the reference gathers
    per pair) is kept as a separate, labelled figure."""
    rate = samples / (bp_ms / 1e3)
    sms = 152
    try:
        import torch

        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    except Exception:
        pass
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    per_clk_sm = rate / (sms * mhz * 1e6)
    peak = XU_PER_CLK_SM / MUFU_PER_PAIR
    floor = XU_PER_CLK_SM / MUFU_PER_PAIR_FLOOR
    hbm_achieved = samples * 4 / (bp_ms / 1e3) / 1e9
    return {
        "bound": "mufu", "achieved": per_clk_sm, "peak": peak, "unit": "voxel-samples/clk/SM",
        "frac": per_clk_sm / peak, "traffic": profiled_traffic(),
        "peak_basis": f"{XU_PER_CLK_SM} XU results/clk/SM / {MUFU_PER_PAIR} MUFU ops per pair (sqrt.approx + "
                      f"rcp.approx per two pairs) at the sampled {mhz:.0f} MHz x {sms} SMs = "
                      f"{peak * sms * mhz * 1e6:.3e} voxel-samples/s",
        "frac_of_bitwise_bin_floor": per_clk_sm / floor,
        "bitwise_bin_floor_note": f"{floor:.0f} voxel-samples/clk/SM: one sqrt.approx per pair, the least any "
                                  "kernel with the reference's bins needs",
        "hbm_accounting": {"achieved_gbs": hbm_achieved, "peak_gbs": hbm_peak, "frac": hbm_achieved / hbm_peak,
                           "peak_source": hbm_kind,
                           "note": "4 B per voxel-sample (the element the reference gathers per pair) / gather "
                                   "launch time; windows are served from shared memory, so this exceeds HBM and "
                                   "is not the limiter"},
        "traffic_note": "dram read + write bytes per gather launch from the committed ncu summary (profiles/)",
    }


# --------------------------------------------------------------- workloads

def make_workload(device, seed: int, size: str):
    from fasterbackprojection_gb300 import make_info, scenes

    n, vres = SIZES[size]
    cap = scenes.confocal_patches_torch(n, N_BINS, DT, seed=seed, device=device)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 1.5))
    info = make_info(num_laser_targets=n * n, num_time_bins=N_BINS, time_step=cap.time_step, voxel_res=vres,
                     hidden_min=hmin, voxel_size=vs)
    return cap, info


def cpu_sample_rate(info, cube_np, lx_np, target_s=10.0, threads=0):
    """The oracle's FP32 restatement of the reference kernel on the host cores,
    over a voxel sample sized to about target_s seconds.  Returns
    (samples/s, description, seconds)."""
    import numpy as np
    from oracle import cpu

    V = info.voxel_res[0] * info.voxel_res[1] * info.voxel_res[2]
    rng = np.random.default_rng(0)
    n = 64
    while True:
        idx = np.sort(rng.choice(V, size=min(n, V), replace=False)).astype(np.int64)
        t0 = time.perf_counter()
        cpu.confocal_voxel_f32_subset(info, cube_np, lx_np, idx, threads=threads)
        dt = time.perf_counter() - t0
        if dt > 0.7 * target_s or n >= V:
            break
        n = int(min(V, n * max(1.5, min(16.0, target_s / max(dt, 1e-3)))))
    pairs = idx.shape[0] * info.num_laser_targets
    return pairs / dt, f"{idx.shape[0]} random voxels x {info.num_laser_targets} scan points", dt


# ------------------------------------------------------------- our arm

def run_ours(args):
    import numpy as np
    import torch

    from fasterbackprojection_gb300 import FBP_FILTER_LOG, Context

    ws, rank, local = dist_setup("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.mode == "slabs":
        return run_slabs(args, ws, rank, local, dev)
    cap, info = make_workload(dev, 2 + rank, args.size)
    L = info.num_laser_targets
    V = info.voxel_res[0] * info.voxel_res[1] * info.voxel_res[2]
    samples = V * L
    ctx = Context(local)
    cube = cap.cube.contiguous()
    lx = cap.laser_xyz.contiguous()
    vx, vy, vz = info.voxel_res
    vol = torch.empty((vz, vy, vx), device=dev)
    vol2 = torch.empty_like(vol)
    stream = torch.cuda.current_stream()

    def step(c):
        ctx.backproject_confocal(info, c, lx, out=vol)
        ctx.postfilter(FBP_FILTER_LOG, vol, 5, 1.0, out=vol2)
        ctx.normalize_(vol2)

    for _ in range(args.warmup):
        step(cube)
    torch.cuda.synchronize()
    ctx.check_device_status()

    # Timed region: K full steps, plus per-launch events around the gather.
    bp_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = ctx.launches
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for k in range(args.steps):
            bp_ev[k][0].record(stream)
            ctx.backproject_confocal(info, cube, lx, out=vol)
            bp_ev[k][1].record(stream)
            ctx.postfilter(FBP_FILTER_LOG, vol, 5, 1.0, out=vol2)
            ctx.normalize_(vol2)
        t_end.record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    launches = ctx.launches - launches0
    ms_total = t_start.elapsed_time(t_end)
    ms_total = max_over_ranks(ms_total, ws, dev)
    ms_step = ms_total / args.steps
    bp_ms = statistics.mean(a.elapsed_time(b) for a, b in bp_ev)
    value = ws * samples * args.steps / (ms_total / 1e3)
    ctx.check_device_status()

    # End to end through the C ABI from pinned host buffers.
    e2e = None
    if not args.no_e2e:
        host_cube = torch.empty(cube.shape, dtype=cube.dtype, pin_memory=True)
        host_cube.copy_(cube)
        host_lx = torch.empty(lx.shape, dtype=lx.dtype, pin_memory=True)
        host_lx.copy_(lx)
        host_vol = torch.empty(vol.shape, dtype=torch.float32, pin_memory=True)
        hc, hl, hv = host_cube.numpy(), host_lx.numpy(), host_vol.numpy()

        def e2e_step():
            ctx.reconstruct_shape_host(info, hc, hl, use_fourier_filter=False, postfilter=FBP_FILTER_LOG,
                                       kernel_size=5, sigma=1.0, normalize=True, out=hv)

        for _ in range(max(1, args.warmup)):
            e2e_step()
        # The capture's H2D copy alone, for the spread of the host-memory DMA.
        h2d_ms = []
        for _ in range(args.steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            cube.copy_(host_cube, non_blocking=True)
            b.record(stream)
            torch.cuda.synchronize()
            h2d_ms.append(round(a.elapsed_time(b), 3))
        barrier(ws)
        call_ms = []
        with ClockSampler(local) as clk_e2e:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                t1 = time.perf_counter()
                e2e_step()
                call_ms.append(round((time.perf_counter() - t1) * 1e3, 2))
            e2e_s = max_over_ranks(time.perf_counter() - t0, ws, dev)
        e2e = {"value": ws * samples * args.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(hc.nbytes + hl.nbytes),
               "d2h_bytes_per_step": int(hv.nbytes), "ms_per_step": e2e_s * 1e3 / args.steps,
               # same kernels, same inputs as the device-resident step
               "matches_device_path": bool(torch.equal(host_vol.to(dev), vol2)),
               "ms_per_call": call_ms, "h2d_alone_ms": h2d_ms, "clocks": clk_e2e.summary()}

    extras = {}
    # The extra legs and the CPU baseline run with one GPU only: at N > 1 the
    # line is the scaling measurement alone, so the other GPUs are not held.
    if not args.no_extras and rank == 0 and ws == 1:
        # BF16 storage of the same capture.
        cube16 = cube.to(torch.bfloat16)
        for _ in range(2):
            ctx.backproject_confocal(info, cube16, lx, out=vol)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            ctx.backproject_confocal(info, cube16, lx, out=vol)
        e1.record(stream)
        torch.cuda.synchronize()
        bf_ms = e0.elapsed_time(e1) / args.steps
        extras["bf16_storage"] = {"bp_ms": round(bf_ms, 3), "value": samples / (bf_ms / 1e3),
                                  "achieved_gbs_2B_per_sample": samples * 2 / (bf_ms / 1e3) / 1e9}
        del cube16
        extras["reference_cuda"] = reference_cuda_rate(info, cube, lx, dev)
        ctx.backproject_confocal(info, cube, lx, out=vol)
        extras["error_vs_fp64"] = fp64_error(ctx, info, cube, lx, vol)
        if not args.no_batch:
            extras["batched"] = batched_leg(ctx, dev, 2)
        if not args.no_learned:
            extras["learned_mis"] = learned_mis_leg(ctx, dev, info, cube, lx)
        if not args.no_configs:
            extras["reference_kernels"] = reference_kernels_leg(ctx, dev, info, cube, lx, vol)
            extras["scatter_forms"] = scatter_forms_leg(ctx, dev, info, cube, lx)
            pk = measured_peaks()[0]
            extras["filters"] = filters_leg(ctx, dev, vol, cube, info.time_step, pk)
            extras["lct"] = lct_leg(ctx, dev, pk)
            extras["exhaustive"] = exhaustive_leg(ctx, dev)

    peak, peak_kind = measured_peaks()
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded 8-patch scene, Poisson noise), generated on device",
        "config": {"workload": WORKLOAD if not args.small else f"{args.size}_{int(round(L ** 0.5))}^2x1024_to_{vx}^3",
                   "scan": [int(round(L ** 0.5))] * 2, "bins": N_BINS, "bin_ps": 16,
                   "volume": list(info.voxel_res), "storage": "f32", "postfilter": "LoG k=5 sigma=1",
                   "l2": "inputs larger than L2 (cube 256 MiB)", "per_gpu": "one capture per rank"},
        "e2e": e2e,
        "roofline": gather_roofline(samples, bp_ms, clocks, peak, peak_kind),
        "bp_ms_per_launch": bp_ms,
        "gpu_launches": launches,
    }
    if not args.no_extras and rank == 0 and ws == 1:
        line["cpu_baseline"] = cpu_baseline(info, cube, lx)
        line.update(extras)
    line["clocks"] = clocks
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def run_slabs(args, ws, rank, local, dev):
    """Strong scaling: every rank reconstructs its depth slab of the same
    capture (backprojection only; the LoG would need halos across slabs).
    value = all ranks' voxel-samples / max-over-ranks time.  e2e: each rank
    copies only its slab's bin window from pinned host memory and reads its
    slab back."""
    import torch

    from fasterbackprojection_gb300 import Context, slabs

    cap, info = make_workload(dev, 2, args.size)
    ctx = Context(local)
    L = info.num_laser_targets
    vx, vy, vz = info.voxel_res
    z0, z1 = slabs.plan(info, ws)[rank]
    cube, lx = cap.cube.contiguous(), cap.laser_xyz.contiguous()
    slab = torch.empty((max(z1 - z0, 0), vy, vx), device=dev)

    def step():
        if z1 > z0:
            ctx.backproject_confocal_slab(info, cube, lx, z0, z1, out=slab)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(ws)
    stream = torch.cuda.current_stream()
    launches0 = ctx.launches
    with ClockSampler(local) as clk:
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.steps):
            step()
        b.record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    launches = ctx.launches - launches0
    ms = max_over_ranks(a.elapsed_time(b), ws, dev) / args.steps
    total = vx * vy * vz * L
    e2e = None
    if not args.no_e2e:
        host_cube = torch.empty(cube.shape, dtype=cube.dtype, pin_memory=True)
        host_cube.copy_(cube)
        host_lx = lx.cpu().numpy()
        host_slab = torch.empty(tuple(slab.shape), dtype=torch.float32, pin_memory=True)
        h2d = 0
        for _ in range(max(1, args.warmup)):
            s, _, h2d = slabs.reconstruct_rank(ctx, info, host_cube, host_lx, rank, ws, dev)
            host_slab.copy_(s)
        torch.cuda.synchronize()
        barrier(ws)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s, _, h2d = slabs.reconstruct_rank(ctx, info, host_cube, host_lx, rank, ws, dev)
            host_slab.copy_(s)
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(time.perf_counter() - t0, ws, dev)
        e2e = {"value": total * args.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(host_slab.numel() * 4), "note": "rank 0's bytes"}
    line = {
        "metric": METRIC, "value": total / (ms / 1e3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded 8-patch scene), generated on device",
        "config": {"workload": "confocal_bp_slabs_" + WORKLOAD, "volume": list(info.voxel_res),
                   "slabs": slabs.plan(info, ws), "postfilter": "none (slab mode)",
                   "l2": "inputs larger than L2 (cube 256 MiB)"},
        "e2e": e2e, "gpu_launches": launches, "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def reference_cuda_rate(info, cube, lx, dev):
    """The reference's own backprojectConfocalVoxel (compiled from its sources,
    oracle/_ref) on the same GPU, over the first depth slices of the volume."""
    import ctypes

    import torch

    try:
        from oracle import harness
    except Exception as e:  # pragma: no cover
        return {"unavailable": f"harness import failed: {e}"}
    if not harness.available():
        return {"unavailable": "reference kernels not built (needs the reference sources at build time)"}
    sub = type(info)()
    ctypes.memmove(ctypes.byref(sub), ctypes.byref(info), ctypes.sizeof(info))
    nz = 8
    sub.voxel_res[2] = nz
    cube_tm = cube.t().contiguous()
    harness.confocal_voxel(sub, cube_tm, lx)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    reps = 2
    for _ in range(reps):
        harness.confocal_voxel(sub, cube_tm, lx)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    samples = sub.voxel_res[0] * sub.voxel_res[1] * nz * sub.num_laser_targets
    del cube_tm
    return {"kernel": "backprojectConfocalVoxel (reference, sm_103a, fast math)", "value": samples / (ms / 1e3),
            "unit": UNIT, "sample": f"{nz} of {info.voxel_res[2]} depth slices", "ms": ms}


def reference_kernels_leg(ctx, dev, info, cube, lx, vol):
    """Our kernels next to the reference's own kernels (compiled from its
    sources, oracle/_ref) on the same GPU and data: LoG (k=5), Laplacian (k=5)
    and min-max normalisation on the 256^3 volume, the one-sample-per-voxel
    MIS kernel, depth-plane backprojection (64^2 x 512, 200 planes) and the
    exhaustive kernel on an L == S capture (16^2 x 16^2, the only shape it
    indexes correctly).  Each entry: ours_ms, reference_ms, speedup, and
    whether the outputs are bitwise equal (where the arithmetic is the
    reference's)."""
    import numpy as np
    import torch

    from fasterbackprojection_gb300 import (FBP_EXHAUSTIVE, FBP_FILTER_LAPLACIAN, FBP_FILTER_LOG, FBP_MIS_REFERENCE,
                                            make_info, scenes)
    from fasterbackprojection_gb300.api import linear_space, log_weights

    try:
        from oracle import harness
    except Exception as e:  # pragma: no cover
        return {"unavailable": f"harness import failed: {e}"}
    if not harness.available():
        return {"unavailable": "reference kernels not built (needs the reference sources at build time)"}
    harness.load()
    out = {}

    def both(name, ours, ref, reps=3, compare=True):
        o, o_ms = timed_ms(ours, reps)
        r, r_ms = timed_ms(ref, reps)
        e = {"ours_ms": o_ms, "reference_ms": r_ms, "speedup": r_ms / o_ms}
        if compare:
            e["bitwise_equal"] = bool(torch.equal(o, r))
            e["rel_l2"] = float(torch.linalg.vector_norm((o - r).double()) /
                                max(float(torch.linalg.vector_norm(r.double())), 1e-30))
        out[name] = e

    w5 = torch.from_numpy(log_weights(5, 1.0)).to(dev)
    both("log_k5_256^3", lambda: ctx.postfilter(FBP_FILTER_LOG, vol, 5, 1.0), lambda: harness.log_filter(vol, w5, 5))
    both("laplacian_k5_256^3", lambda: ctx.postfilter(FBP_FILTER_LAPLACIAN, vol, 5),
         lambda: harness.laplacian_filter(vol, 5))
    a, b = vol.clone(), vol.clone()
    both("normalize_256^3", lambda: ctx.normalize_(a.copy_(vol)), lambda: harness.normalize_(b.copy_(vol)))
    # MIS (the reference's one-sample balance-heuristic kernel): 64 samples per
    # voxel over the whole 256^3 volume.  Ours includes the per-call proposal
    # tables (scan totals on the GPU, Vose alias on the host, as the
    # reference's host code builds them); the reference column is its kernel
    # alone.  With more than one sample the reference's += races, so only
    # the one-sample case is compared bitwise (tests).
    V = info.voxel_res[0] * info.voxel_res[1] * info.voxel_res[2]
    noise = torch.rand(V, generator=torch.Generator().manual_seed(5)).to(dev)
    cdf, alias, prob = ctx.mis_reference_tables(info, cube)
    cdf_t, alias_t, prob_t = (torch.from_numpy(cdf).to(dev), torch.from_numpy(alias.astype(np.int32)).to(dev),
                              torch.from_numpy(prob).to(dev))
    cube_tm = cube.t().contiguous()
    both("mis_reference_64_samples_256^2x1024_to_256^3",
         lambda: ctx.mis_backproject(info, cube, lx, FBP_MIS_REFERENCE, 64, noise=noise),
         lambda: harness.confocal_voxel_mis(info, cube_tm, lx, cdf_t, noise, alias_t, prob_t, 64), reps=2,
         compare=False)
    del cube_tm
    # Depth planes (confocal, 64^2 x 512, 200 planes around 0.8 m).
    cap = scenes.confocal_points(64, 512, 32e-12, n_points=200, seed=1)
    dinfo = make_info(num_laser_targets=4096, num_time_bins=512, time_step=cap.time_step, voxel_res=(1, 1, 1),
                      hidden_min=(0, 0, 0), voxel_size=(1, 1, 1))
    dc = torch.from_numpy(cap.cube).to(dev)
    dlx = torch.from_numpy(cap.laser_xyz).to(dev)
    depths = torch.from_numpy(linear_space(0.7, 0.9, 200)).to(dev)
    dtm = dc.t().contiguous()
    both("depth_planes_64^2x512_200", lambda: ctx.backproject_depths(dinfo, dc, dlx, depths),
         lambda: harness.depth_confocal(dinfo, dtm, dlx, depths))
    # Exhaustive on L == S = 16^2, 8 of 128 depth slices.
    ecap = scenes.exhaustive_points(16, 16, 1024, 16e-12, n_points=100, seed=3)
    hmin, vs = scenes.volume_geometry((128, 128, 128), depth_range=(0.0, 1.5))
    einfo = make_info(num_laser_targets=256, num_sensor_targets=256, num_time_bins=1024, time_step=ecap.time_step,
                      voxel_res=(128, 128, 8), hidden_min=hmin, voxel_size=vs, capture_system=FBP_EXHAUSTIVE)
    ec = torch.from_numpy(ecap.cube).to(dev)
    elx, esx = torch.from_numpy(ecap.laser_xyz).to(dev), torch.from_numpy(ecap.sensor_xyz).to(dev)
    both("exhaustive_16^2x16^2x1024_8_slices", lambda: ctx.backproject_exhaustive(einfo, ec, elx, esx),
         lambda: harness.exhaustive_voxel(einfo, ec, elx, esx))
    ctx.check_device_status()
    return out


def scatter_forms_leg(ctx, dev, info, cube, lx):
    """The scatter-form rows next to the headline workload: the voxel-scattering
    gather (the reference's ACCUMULATE_VOXEL_SCATTERING build) over the full
    256^3 volume and against the reference's own kernel of that build on the
    first 8 depth slices; the rasterised ellipsoid splat (700 bins, 256 x 256
    pixel grid, the reference's GL defaults); the depth-plane images of a
    64^2-scan, 200-plane reconstruction enlarged to 256 x 256."""
    import ctypes

    import torch

    from fasterbackprojection_gb300 import make_info, scenes
    from fasterbackprojection_gb300.api import linear_space

    out = {}
    V = info.voxel_res[0] * info.voxel_res[1] * info.voxel_res[2]
    pairs = V * info.num_laser_targets
    n = int(round(info.num_laser_targets ** 0.5))
    vdiag = sum(float(v) ** 2 for v in info.voxel_size) ** 0.5
    bin_m = info.time_step
    shape = f"{n}^2 x {info.num_time_bins} FP32 -> {info.voxel_res[0]}^3"
    vol = torch.empty(V, dtype=torch.float32, device=dev)
    _, ms = timed_ms(lambda: ctx.backproject_confocal_scatter(info, cube, lx, out=vol), reps=2)
    e = {"workload": f"{shape}, voxel extent (diagonal) {vdiag * 1e3:.1f} mm, bins of {bin_m * 1e3:.1f} mm "
                     f"(about {vdiag / bin_m:.1f} bins per walk)",
         "ms": ms, "value": pairs / (ms / 1e3), "unit": UNIT}
    try:
        from oracle import harness

        if harness.scatter_available():
            harness.load()
            sub = type(info)()
            ctypes.memmove(ctypes.byref(sub), ctypes.byref(info), ctypes.sizeof(info))
            sub.voxel_res[2] = 8
            cube_tm = cube.t().contiguous()
            o, o_ms = timed_ms(lambda: ctx.backproject_confocal_scatter(sub, cube, lx), reps=2)
            r, r_ms = timed_ms(lambda: harness.confocal_voxel_scatter(sub, cube_tm, lx), reps=2)
            del cube_tm
            e["reference_8_slices"] = {"ours_ms": o_ms, "reference_ms": r_ms, "speedup": r_ms / o_ms,
                                       "rel_l2": float(torch.linalg.vector_norm((o - r).double()) /
                                                       max(float(torch.linalg.vector_norm(r.double())), 1e-30))}
        else:
            e["reference_8_slices"] = {"unavailable": "reference scatter build not present"}
    except Exception as ex:  # pragma: no cover
        e["reference_8_slices"] = {"unavailable": f"harness: {ex}"}
    out["voxel_scattering"] = e
    # The reference-mode MIS kernel of the same build (transient_reconstruction.cuh:
    # 235-250): 64 samples per voxel, each walking its voxel's bin range.
    from fasterbackprojection_gb300 import FBP_MIS_REFERENCE_SCATTER

    noise = torch.rand(V, generator=torch.Generator().manual_seed(5)).to(dev)
    mvol = torch.empty(V, dtype=torch.float32, device=dev)
    _, m_ms = timed_ms(lambda: ctx.mis_backproject(info, cube, lx, FBP_MIS_REFERENCE_SCATTER, 64, noise=noise,
                                                   out=mvol), reps=2)
    m = {"workload": f"64 samples per voxel, {shape}, walks of about {vdiag / bin_m:.1f} bins", "ms": m_ms,
         "samples_per_s": V * 64 / (m_ms / 1e3)}
    try:
        from oracle import harness

        if harness.scatter_available():
            harness.load()
            cdf, alias, prob = ctx.mis_reference_tables(info, cube)
            cube_tm = cube.t().contiguous()
            args = (torch.from_numpy(cdf).to(dev), noise, torch.from_numpy(alias.astype("int32")).to(dev),
                    torch.from_numpy(prob).to(dev))
            r, r_ms = timed_ms(lambda: harness.confocal_voxel_mis_scatter(info, cube_tm, lx, args[0], args[1], args[2],
                                                                          args[3], 64), reps=2)
            del cube_tm
            m.update({"reference_ms": r_ms, "speedup": r_ms / m_ms,
                      "rel_l2_vs_reference": float(torch.linalg.vector_norm((mvol.view_as(r) - r).double()) /
                                                   max(float(torch.linalg.vector_norm(r.double())), 1e-30))})
        else:
            m["reference"] = {"unavailable": "reference scatter build not present"}
    except Exception as ex:  # pragma: no cover
        m["reference"] = {"unavailable": f"harness: {ex}"}
    out["mis_voxel_scattering"] = m
    del mvol, noise
    svol = torch.empty(V, dtype=torch.float32, device=dev)
    _, ms = timed_ms(lambda: ctx.splat_backproject(info, cube, lx, max_bins=700, grid=(256, 256), out=svol), reps=2)
    nz = int((cube[:, :700] > 1.1920929e-7).sum())
    out["splat"] = {"workload": f"{shape}, bins < 700, 256 x 256 pixel grid", "ms": ms,
                    "instances": nz, "instances_per_s": nz / (ms / 1e3),
                    "gl_timing": "unavailable on this box (no graphics stack)"}
    del svol
    cap = scenes.confocal_points(64, 512, 32e-12, n_points=200, seed=1)
    dinfo = make_info(num_laser_targets=4096, num_time_bins=512, time_step=cap.time_step, voxel_res=(1, 1, 1),
                      hidden_min=(0, 0, 0), voxel_size=(1, 1, 1))
    depths = torch.from_numpy(linear_space(0.7, 0.9, 200)).to(dev)
    act = ctx.backproject_depths(dinfo, torch.from_numpy(cap.cube).to(dev), torch.from_numpy(cap.laser_xyz).to(dev),
                                 depths)
    ctx.normalize_(act)
    imgs = torch.empty((200, 256, 256, 4), dtype=torch.uint8, device=dev)
    _, ms = timed_ms(lambda: ctx.depth_plane_images(act, 64, 64, size=(256, 256), out=imgs), reps=5)
    out["depth_plane_images"] = {"workload": "200 planes of 64^2 -> 256^2 RGBA8 (bilinear)", "ms": ms,
                                 "bytes_written": imgs.numel(), "achieved_gbs": imgs.numel() / (ms / 1e3) / 1e9}
    ctx.check_device_status()
    return out


def fp64_error(ctx, info, cube, lx, vol, nvox=512, seed=5):
    """rel-L2 of a gathered volume against the FP64 oracle over a random voxel
    sample: with the oracle's own FP64 bins, and with the GPU's bins (which
    isolates the accumulation).  cube is the device cube the gather read."""
    import numpy as np
    import torch
    from oracle import cpu

    V = info.voxel_res[0] * info.voxel_res[1] * info.voxel_res[2]
    rng = np.random.default_rng(seed)
    rnd = rng.choice(V, size=min(nvox, V), replace=False)
    # plus the 128 largest voxels: the longest sums of the largest weights
    top = torch.topk(vol.reshape(-1), min(128, V)).indices.cpu().numpy()
    idx = np.unique(np.concatenate([rnd, top])).astype(np.int64)
    idx_t = torch.from_numpy(idx).to(lx.device)
    bins = ctx.debug_confocal_bins(info, lx, idx_t).cpu().numpy()
    host = cube.float().cpu().numpy()
    lxn = lx.cpu().numpy()
    got = vol.reshape(-1)[idx_t].double().cpu().numpy()
    want64 = cpu.confocal_voxel_subset(info, host, lxn, idx)
    want_same = cpu.confocal_voxel_subset(info, host, lxn, idx, bins=bins)

    def rel(a, b):
        nb = float(np.linalg.norm(b))
        return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))

    is_top = np.isin(idx, top)
    return {"rel_l2_vs_fp64": rel(got, want64), "rel_l2_vs_fp64_same_bins": rel(got, want_same),
            "rel_l2_vs_fp64_same_bins_largest_128": rel(got[is_top], want_same[is_top]),
            "voxels": int(idx.shape[0]), "sample": f"{nvox} random voxels and the 128 largest"}


def batched_leg(ctx, dev, steps):
    """64 confocal captures of uneven sizes (scan N in {32,64,128,256}^2, bins
    in {256..2048} over the same 16.4 ns window, volume N^3, BF16 storage)
    reconstructed by one persistent launch replayed from a CUDA graph, tile
    shape chosen by the autotuner.  Per-capture error vs FP64 on 128 voxels."""
    import numpy as np
    import torch

    from fasterbackprojection_gb300 import FBP_LAYOUT_TIME_INNER, Batch, make_info, scenes
    from oracle import cpu

    caps, errs_in = [], []
    for c in scenes.batched_configs(seed0=100, count=64):
        n, T, vres = c["n"], c["T"], c["vres"]
        cap = scenes.confocal_patches_torch(n, T, DT * N_BINS / T, seed=c["seed"], device=dev)
        hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 1.5))
        info = make_info(num_laser_targets=n * n, num_time_bins=T, time_step=cap.time_step, voxel_res=vres,
                         hidden_min=hmin, voxel_size=vs)
        cube16 = cap.cube.to(torch.bfloat16).contiguous()
        lx = cap.laser_xyz.contiguous()
        V = vres[0] * vres[1] * vres[2]
        idx = np.sort(np.random.default_rng(c["seed"]).choice(V, size=min(128, V), replace=False)).astype(np.int64)
        idx_t = torch.from_numpy(idx).to(dev)
        bins = ctx.debug_confocal_bins(info, lx, idx_t).cpu().numpy()
        lxn = lx.cpu().numpy()
        dec = cube16.float().cpu().numpy()
        want64 = cpu.confocal_voxel_subset(info, dec, lxn, idx)
        want_same = cpu.confocal_voxel_subset(info, dec, lxn, idx, bins=bins)
        want_f32 = cpu.confocal_voxel_subset(info, cap.cube.cpu().numpy(), lxn, idx)
        del cap, dec
        vol = torch.empty((vres[2], vres[1], vres[0]), device=dev)
        caps.append((info, cube16, lx, vol, FBP_LAYOUT_TIME_INNER))
        errs_in.append((idx_t, want64, want_same, want_f32))
    samples = sum(c[0].num_laser_targets * c[0].voxel_res[0] * c[0].voxel_res[1] * c[0].voxel_res[2] for c in caps)
    b = Batch(ctx, caps)
    s = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(s):
        chosen = b.autotune(stream=s)
        b.run(use_graph=True, stream=s)  # capture + first replay (warm-up)
        s.synchronize()
        ctx.check_device_status(stream=s)
        launches0 = ctx.launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(steps):
            b.run(use_graph=True, stream=s)
        e1.record(s)
        s.synchronize()
        ms = e0.elapsed_time(e1) / steps
        launches = (ctx.launches - launches0) // steps
        # The same captures one after another through the single-capture call.
        q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        tmp = [torch.empty_like(c[3]) for c in caps]
        q0.record(s)
        for c, t in zip(caps, tmp):
            ctx.backproject_confocal(c[0], c[1], c[2], out=t, stream=s)
        q1.record(s)
        s.synchronize()
        seq_ms = q0.elapsed_time(q1)
    same_as_single = all(torch.equal(c[3], t) for c, t in zip(caps, tmp)) if chosen == 0 else None
    del tmp

    def rel(a, b_):
        nb = float(np.linalg.norm(b_))
        return float(np.linalg.norm(a - b_) / (nb if nb > 0 else 1.0))

    per = []
    for c, (idx_t, w64, wsame, wf32) in zip(caps, errs_in):
        got = c[3].reshape(-1)[idx_t].double().cpu().numpy()
        per.append((rel(got, w64), rel(got, wsame), rel(got, wf32)))
    b.close()
    sizes = [f"{int(round(c[0].num_laser_targets ** 0.5))}^2x{c[0].num_time_bins}" for c in caps]
    return {
        "workload": "64 confocal captures, scan {32,64,128,256}^2, bins {256,512,1024,2048}, volume N^3, bf16",
        "captures": len(caps), "samples_per_step": samples, "ms_per_step": ms, "value": samples / (ms / 1e3),
        "unit": UNIT, "steps": steps, "graph": True, "autotuned_tile": chosen, "gpu_launches_per_step": launches,
        "sequential_single_capture_ms": seq_ms, "tile0_equals_single_capture": same_as_single,
        "max_rel_l2_vs_fp64": max(p[0] for p in per), "max_rel_l2_vs_fp64_same_bins": max(p[1] for p in per),
        "max_rel_l2_vs_fp32_cube": max(p[2] for p in per),
        "per_capture": [{"capture": z, "rel_l2_vs_fp64": round(p[0], 9), "rel_l2_vs_fp32_cube": round(p[2], 6)}
                        for z, p in zip(sizes, per)],
        "error_sample": "128 random voxels per capture; FP64 oracle on the decoded BF16 cube (vs_fp64) and on "
                        "the FP32 cube before rounding (vs_fp32_cube, includes the storage rounding)",
    }


def timed_ms(fn, reps=5, stream=None):
    """Mean CUDA-event time of fn() over reps calls after one warm-up call."""
    import torch

    stream = stream or torch.cuda.current_stream()
    fn()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        out = fn()
    b.record(stream)
    torch.cuda.synchronize()
    return out, a.elapsed_time(b) / reps


def lct_moved_bytes(N, M):
    """Bytes the fused LCT passes read and write once each: capture in and
    volume out (4 B), the z spectra of planes kz <= M (complex64; written by
    the z pass, read and written by the plane pass, read by the inverse z
    pass) and their Wiener planes; N > 64 adds the row-transformed planes
    (N x 2N, written, read and written by the column pass, read back)."""
    P = M + 1
    b = 8 * M * N * N + 4 * 8 * P * N * N + 8 * P * (2 * N) ** 2
    if N > 64:
        b += 4 * 8 * P * N * (2 * N)
    return b


def lct_leg(ctx, dev, peak):
    """LCT of the 64^2 x 512 x 32 ps point capture (200 points) into 64x64x512,
    against the oracle's FP64 restatement of python/lct.py, which is also
    timed on the host cores (the reference's lct.py cannot run here: it
    needs the Stanford .mat captures; its steps are restated)."""
    import numpy as np
    import torch

    from fasterbackprojection_gb300 import scenes
    from oracle import numpy_ref

    N, M = 64, 512
    cap = scenes.confocal_points(N, M, 32e-12, n_points=200, seed=1)
    data = cap.cube.reshape(N, N, M).transpose(2, 0, 1).copy()  # [M][N][N]
    d = torch.from_numpy(data).to(dev)
    t0 = time.perf_counter()
    first = ctx.lct(d, 1.0, cap.time_step, 0.8, True)
    torch.cuda.synchronize()
    first_s = time.perf_counter() - t0
    vol, ms = timed_ms(lambda: ctx.lct(d, 1.0, cap.time_step, 0.8, True), reps=20)
    bytes_run = 4 * M * N * N * 2 + 2 * 2 * 8 * (2 * M) * (2 * N) ** 2
    # CPU: the FP64 NumPy restatement, timed step by step on all host cores.
    t0 = time.perf_counter()
    psf = numpy_ref.define_psf(N, M, 1.0 / (M * cap.time_step))
    t_psf = time.perf_counter() - t0
    t0 = time.perf_counter()
    mtx, mtxi = numpy_ref.resampling_operator(M)
    t_res = time.perf_counter() - t0
    t0 = time.perf_counter()
    want = numpy_ref.lct(data.astype(np.float64), 1.0, cap.time_step, 0.8, True, psf=psf, mtx=mtx, mtxi=mtxi)
    t_steps = time.perf_counter() - t0
    got = vol.cpu().numpy()
    # The row/column-pass form (N >= 128): timed only, its parity is tested.
    N2, M2 = 128, 1024
    cap2 = scenes.confocal_points(N2, M2, 16e-12, n_points=200, seed=2)
    d2 = torch.from_numpy(cap2.cube.reshape(N2, N2, M2).transpose(2, 0, 1).copy()).to(dev)
    _, ms2 = timed_ms(lambda: ctx.lct(d2, 1.0, cap2.time_step, 0.8, True))
    bytes2 = 4 * M2 * N2 * N2 * 2 + 2 * 2 * 8 * (2 * M2) * (2 * N2) ** 2
    moved2 = lct_moved_bytes(N2, M2)
    del d2
    return {
        "workload": "LCT, 64^2 scan x 512 bins of 32 ps, 200 points -> 64x64x512 (diffuse, snr 0.8)",
        "rows_cols_form": {"workload": "LCT, 128^2 scan x 1024 bins of 16 ps, 200 points -> 128x128x1024",
                           "gpu_ms": ms2, "bytes_per_run": bytes2, "achieved_gbs": bytes2 / (ms2 / 1e3) / 1e9,
                           "frac": bytes2 / (ms2 / 1e3) / 1e9 / peak, "moved_bytes_per_run": moved2,
                           "moved_frac": moved2 / (ms2 / 1e3) / 1e9 / peak},
        "gpu_ms": ms, "gpu_first_call_s": first_s,
        "roofline": {"bound": "hbm", "bytes_per_run": bytes_run, "achieved_gbs": bytes_run / (ms / 1e3) / 1e9,
                     "peak_gbs": peak, "frac": bytes_run / (ms / 1e3) / 1e9 / peak,
                     "bytes_note": "4 B per capture and volume element plus one read and write of the padded "
                                   "complex64 volume per forward and inverse 3-D transform",
                     "moved_bytes_per_run": lct_moved_bytes(N, M),
                     "moved_frac": lct_moved_bytes(N, M) / (ms / 1e3) / 1e9 / peak,
                     "moved_note": "the passes' own buffers, each read or written once: the spectra of planes "
                                   "kz <= M only (Hermitian z-lines), the Wiener planes kz <= M"},
        "rel_l2_vs_fp64": float(np.linalg.norm(got - want) / np.linalg.norm(want)),
        "cpu": {"kind": "port", "cores": os.cpu_count(), "define_psf_s": t_psf, "resampling_operator_s": t_res,
                "steps_1_4_s": t_steps, "total_s": t_psf + t_res + t_steps,
                "sample": "full run of the FP64 NumPy restatement of python/lct.py (numpy FFT, sparse operator)"},
        "speedup_vs_cpu_steps": t_steps / (ms / 1e3),
    }


def exhaustive_leg(ctx, dev):
    """Exhaustive backprojection: 16^2 lasers x 32^2 SPADs, 1024 bins of
    16 ps, FP16, 500 points -> 128^3; error vs FP64 on 128 voxels."""
    import numpy as np
    import torch

    from fasterbackprojection_gb300 import FBP_EXHAUSTIVE, make_info, scenes
    from oracle import cpu

    cap = scenes.exhaustive_points_torch(16, 32, 1024, 16e-12, n_points=500, seed=3, device=dev)
    vres = (128, 128, 128)
    hmin, vs = scenes.volume_geometry(vres, depth_range=(0.0, 1.5))
    L, S = 256, 1024
    info = make_info(num_laser_targets=L, num_sensor_targets=S, num_time_bins=1024, time_step=cap.time_step,
                     voxel_res=vres, hidden_min=hmin, voxel_size=vs, capture_system=FBP_EXHAUSTIVE)
    cube16 = cap.cube.to(torch.float16).contiguous()
    del cap.cube
    vol, ms = timed_ms(lambda: ctx.backproject_exhaustive(info, cube16, cap.laser_xyz, cap.sensor_xyz), reps=3)
    triples = 128 ** 3 * L * S
    rnd = np.random.default_rng(3).choice(128 ** 3, 128, replace=False)
    top = torch.topk(vol.reshape(-1), 64).indices.cpu().numpy()  # the longest sums of the largest weights
    idx = np.unique(np.concatenate([rnd, top])).astype(np.int64)
    cube_np = cube16.float().cpu().numpy().reshape(L * S, 1024)
    lx_np, sx_np = cap.laser_xyz.cpu().numpy(), cap.sensor_xyz.cpu().numpy()
    want = cpu.exhaustive_voxel_subset(info, cube_np, lx_np, sx_np, idx)
    # The same voxels with the GPU's own bins: isolates the accumulation (FP32
    # blocks + Kahan, the weights) from bins that flip at FP32 bin edges.
    gbins = ctx.debug_exhaustive_bins(info, cap.laser_xyz, cap.sensor_xyz, torch.from_numpy(idx).to(dev))
    gbins = gbins.cpu().numpy().reshape(len(idx), L * S)
    want_same = cpu.exhaustive_voxel_subset(info, cube_np, lx_np, sx_np, idx, bins=gbins)
    got = vol.reshape(-1)[torch.from_numpy(idx).to(dev)].double().cpu().numpy()
    # FP64 bins of the same triples: how many differ from the GPU's, and how
    # much of the independent-bins error those flips alone account for.
    vxs, vys, vzs = idx % 128, (idx // 128) % 128, idx // (128 * 128)
    vsz = np.array(info.voxel_size, dtype=np.float64)
    pts = np.array(info.hidden_min, dtype=np.float64) + np.stack([vxs, vzs, vys], 1) * vsz + 0.5 * vsz
    rl = np.linalg.norm(lx_np.astype(np.float64)[None, :, None, :] - pts[:, None, None, :], axis=3)
    rs = np.linalg.norm(sx_np.astype(np.float64)[None, None, :, :] - pts[:, None, None, :], axis=3)
    b64 = np.floor((rl + rs) / float(info.time_step)).reshape(len(idx), L * S)
    b64 = np.where((b64 >= 0) & (b64 < 1024), b64, -1).astype(np.int64)
    nz = cube_np[np.arange(L * S)[None, :], np.clip(gbins, 0, 1023)] > 1e-5
    flipped = (b64 != gbins)
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    return {
        "workload": "exhaustive 16^2 x 32^2 x 1024 (16 ps) FP16 -> 128^3, 500 points",
        "ms": ms, "value": triples / (ms / 1e3), "unit": "voxel-samples/s (voxel, laser, SPAD)",
        "achieved_gbs_2B_per_sample": triples * 2 / (ms / 1e3) / 1e9,
        "rel_l2_vs_fp64": rel(got, want), "error_voxels": int(len(idx)),
        "error_sample": "128 random voxels and the 64 largest",
        "rel_l2_vs_fp64_same_bins": rel(got, want_same),
        "rel_l2_vs_fp64_same_bins_largest_64": rel(got[np.isin(idx, top)], want_same[np.isin(idx, top)]),
        "bin_flips": {"triples": int(flipped.size), "flipped": int(flipped.sum()),
                      "flipped_on_nonzero_samples": int((flipped & nz).sum()),
                      "rel_l2_fp64_gpu_bins_vs_fp64_bins": rel(want_same, want),
                      "note": "flips are triples whose path lies within an FP32 rounding of a bin edge; "
                              "the FP64-vs-FP64 difference with the two bin sets is the whole "
                              "independent-bins error"},
        "reference_cuda": {"unavailable": "the reference kernel splits the pair index by L (l = ls/L, "
                                          "s = ls%L) and reads laserTargets out of bounds when L != S"},
    }


def filters_leg(ctx, dev, vol, cube, time_step, peak):
    """LoG (k=5, sigma 1), min-max normalisation and filter_H on the
    benchmark volume / capture: HBM rooflines (LoG 8 B per voxel, normalise
    12 B per voxel, filter_H 8 B per bin)."""
    import torch

    from fasterbackprojection_gb300 import FBP_FILTER_LOG

    V = vol.numel()
    out = torch.empty_like(vol)
    _, log_ms = timed_ms(lambda: ctx.postfilter(FBP_FILTER_LOG, vol, 5, 1.0, out=out), reps=20)
    tmp = out.clone()
    _, norm_ms = timed_ms(lambda: ctx.normalize_(tmp), reps=20)
    # The allocation-free entry point on the same volume (same result bits).
    import ctypes

    from fasterbackprojection_gb300 import _lib

    lib = _lib.load()
    tmp2 = out.clone()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _, na_ms = timed_ms(lambda: lib.fbp_normalize_minmax_noalloc(ctypes.c_void_p(tmp2.data_ptr()), V, sp), reps=20)
    res = {"log": {"ms": log_ms, "bytes": 8 * V, "achieved_gbs": 8 * V / (log_ms / 1e3) / 1e9,
                   "frac": 8 * V / (log_ms / 1e3) / 1e9 / peak},
           "normalize": {"ms": norm_ms, "bytes": 12 * V, "achieved_gbs": 12 * V / (norm_ms / 1e3) / 1e9,
                         "frac": 12 * V / (norm_ms / 1e3) / 1e9 / peak,
                         "noalloc_ms": na_ms, "noalloc_bitwise_equal": bool(torch.equal(tmp, tmp2))}}
    c = cube.clone()
    nb = c.numel()
    _, fh_ms = timed_ms(lambda: ctx.filter_h_(c, time_step), reps=20)
    res["filter_h"] = {"ms": fh_ms, "bytes": 8 * nb, "achieved_gbs": 8 * nb / (fh_ms / 1e3) / 1e9,
                       "frac": 8 * nb / (fh_ms / 1e3) / 1e9 / peak,
                       "workload": "256^2 series x 1024 bins, wavelength 10 bins (taps over 1106 padded bins)"}
    # The reference's filter_H arithmetic path (Laser.cu:174-234) on the same
    # GPU: zero-padded series, batched C2C FFT (cuFFT through torch), the
    # product with the filter's spectrum, unnormalised inverse, real part.
    try:
        import numpy as np

        from oracle import numpy_ref

        T = cube.shape[-1]
        Ls = nb // T
        sigma, _t6, npad = numpy_ref.filter_h_params(T, time_step, 10 * time_step)
        K = numpy_ref.filter_h_kernel(npad, float(np.float32(time_step)), float(np.float32(10 * time_step)), sigma)
        pad = (npad - T) // 2
        Kf = torch.fft.fft(torch.from_numpy(K.astype(np.complex64)).to(cube.device))
        Hs = torch.zeros((Ls, npad), dtype=torch.complex64, device=cube.device)
        src = cube.reshape(Ls, T)
        ref_c = torch.empty_like(src)

        def cufft_filter_h():
            Hs.zero_()
            Hs[:, pad:pad + T] = src
            ref_c.copy_(torch.fft.ifft(torch.fft.fft(Hs, dim=1) * Kf[None], dim=1, norm="forward")[:, pad:pad + T].real)

        _, rf_ms = timed_ms(cufft_filter_h)
        once = cube.clone()  # one application (the timed loop above filters c in place repeatedly)
        ctx.filter_h_(once, time_step)
        res["filter_h"]["reference_cufft_c2c_ms"] = rf_ms
        res["filter_h"]["speedup_vs_cufft_pipeline"] = rf_ms / fh_ms
        res["filter_h"]["rel_l2_vs_cufft_pipeline"] = float(
            torch.linalg.vector_norm((once.reshape(Ls, T) - ref_c).double()) / torch.linalg.vector_norm(ref_c.double()))
        del once
        del Hs
    except RuntimeError as e:  # pragma: no cover
        res["filter_h"]["reference_cufft_unavailable"] = str(e)
    # LoG-FFT (LoGFFT::compute): ours against the reference's own arithmetic
    # path, an R2C FFT, the half-grid response and a C2R FFT through cuFFT
    # (the library the reference calls), on the same volume.
    from fasterbackprojection_gb300 import FBP_FILTER_LOG_FFT

    n = vol.shape[0]
    _, lf_ms = timed_ms(lambda: ctx.postfilter(FBP_FILTER_LOG_FFT, vol, 5, 1.0, out=out), reps=20)
    f = torch.fft.fftfreq(n, device=vol.device).float()
    fz, fy, fx = torch.meshgrid(f, f, f[: n // 2 + 1].abs(), indexing="ij")
    k2 = fx * fx + fy * fy + fz * fz
    resp = (-4 * math.pi ** 2 * k2 * torch.exp(-2 * math.pi ** 2 * k2)).contiguous()
    ref_out = torch.empty_like(vol)

    def cufft_path():
        ref_out.copy_(torch.fft.irfftn(torch.fft.rfftn(vol) * resp, s=vol.shape, norm="forward"))

    cf_ms = 0.0
    try:
        _, cf_ms = timed_ms(cufft_path, reps=20)
        rel = float(torch.linalg.vector_norm((out - ref_out).double()) / torch.linalg.vector_norm(ref_out.double()))
    except RuntimeError as e:  # pragma: no cover
        rel = None
        cf_ms = None
        res["log_fft_cufft_unavailable"] = str(e)
    res["log_fft"] = {"ms": lf_ms, "cufft_r2c_c2r_ms": cf_ms, "rel_l2_vs_cufft": rel,
                      "bytes": 8 * V, "frac": 8 * V / (lf_ms / 1e3) / 1e9 / peak}
    return res


def learned_mis_leg(ctx, dev, info, cube, lx, n_train=2000, ks=(4, 5, 6, 8, 12, 16, 32, 64), seeds=(0, 1, 2)):
    """Learned MIS on the benchmark capture in BF16: train the proposal MLP on
    the device (2000 seeded point scenes, 64^2 x 512 x 32 ps, seeds 10000..),
    then for K cluster samples per voxel tile (clusters of 16 x 16 scan
    points, 256 per capture) compare learned and uniform cluster proposals
    with the full backprojection of the same BF16 cube: rel-L2 and time.
    Time-to-1% = wall time (CUDA events) of the smallest K reaching <= 1 %
    rel-L2, the learned arm including its feature + MLP pass."""
    import numpy as np
    import torch

    from fasterbackprojection_gb300 import FBP_MIS_LEARNED, Mlp, learned

    n = int(round(info.num_laser_targets ** 0.5))
    cs = n // 16
    stream = torch.cuda.current_stream()
    cube16 = cube.to(torch.bfloat16)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def timed(fn, reps=3):
        fn()
        a, b = ev(), ev()
        a.record(stream)
        for _ in range(reps):
            out = fn()
        b.record(stream)
        torch.cuda.synchronize()
        return out, a.elapsed_time(b) / reps

    full, full_ms = timed(lambda: ctx.backproject_confocal(info, cube16, lx))
    data = learned.build_training_set(ctx, range(10000, 10000 + n_train), vres=tuple(info.voxel_res), device=dev)
    mlp = Mlp(ctx, seed=7)
    losses, train_s = learned.train(ctx, mlp, data, epochs=4, batch=256, lr=2e-3)
    cdf, prop_ms = timed(lambda: learned.proposal(ctx, mlp, info, cube16, lx, cs, n, defensive=0.1))

    full_d = full.double()
    full_n = torch.linalg.vector_norm(full_d)

    def rel(v):
        return float(torch.linalg.vector_norm(v.double() - full_d) / full_n)

    cv = cs // 4  # control variate: 4 x 4-point blocks (1/16 of the scan points)
    arms = (("learned_cv", cdf, cv), ("uniform_cv", None, cv), ("learned", cdf, 0), ("uniform", None, 0))
    rows = []
    for K in ks:
        r = {"K": K}
        for name, tc, cvs in arms:
            def run(sd):
                return ctx.mis_backproject(info, cube16, lx, FBP_MIS_LEARNED, K, seed=sd, tile_cluster_cdf=tc,
                                           cluster_side=cs, scan_side=n, cv_side=cvs)
            est, t = timed(lambda: run(seeds[0]), reps=2)  # time (the same work for every seed)
            errs = [rel(est)] + [rel(run(sd)) for sd in seeds[1:]]
            r[name] = {"rel_l2": float(np.mean(errs)), "ms": float(t)}
        rows.append(r)
    ctx.check_device_status()

    def ttt(name, extra_ms):
        for r in rows:
            if r[name]["rel_l2"] <= 0.01:
                return r[name]["ms"] + extra_ms
        return None

    t_l, t_u = ttt("learned_cv", prop_ms), ttt("uniform_cv", 0.0)
    t_lp, t_up = ttt("learned", prop_ms), ttt("uniform", 0.0)
    best = min((t, n) for t, n in ((t_l, "learned_cv"), (t_lp, "learned")) if t) if any((t_l, t_lp)) else (None, None)
    mlp.close()
    data_s = data.seconds
    del data
    return {
        "workload": "256^2 x 1024 confocal patch capture in BF16 (-> 256^3); K clusters of 16x16 scan points per "
                    "8x16x16-voxel tile, systematic sampling, whole clusters gathered",
        "training": {"scenes": n_train, "tiles": int(n_train * 64), "epochs": 4, "losses": losses,
                     "data_s": data_s, "train_s": train_s},
        "full_bp_ms": full_ms, "proposal_ms": prop_ms, "per_k": rows,
        "time_to_1pct_ms": {"learned_cv": t_l, "uniform_cv": t_u, "learned": t_lp, "uniform": t_up,
                            "full_bp": full_ms},
        "learned_gain_vs_uniform_cv": (t_u / t_l) if (t_u and t_l) else None,
        "learned_vs_full_time": (best[0] / full_ms) if best[0] else None, "best_learned_arm": best[1],
        "estimators": "learned_cv / uniform_cv: block-summed control variate (4x4 scan points) + sampled "
                      "clusters' residuals; learned / uniform: plain cluster sampling; all unbiased",
        "samples": "K clusters of 256 scan points per 8x16x16-voxel tile (K = 4..64); rel-L2 the mean over "
                   "MIS seeds, time of one estimate (CUDA events; time to 1 % = the smallest K whose mean "
                   "reaches 1 %, plus the proposal for the learned arms)",
        "note": "rel-L2 vs the full backprojection of the same BF16 cube; mean over MIS seeds " + str(list(seeds)),
    }


def cpu_baseline(info, cube, lx):
    # All host threads, whatever OMP_NUM_THREADS a launcher set (torchrun sets 1).
    rate, desc, dt = cpu_sample_rate(info, cube.cpu().numpy(), lx.cpu().numpy(), target_s=12.0,
                                     threads=os.cpu_count() or 1)
    return {"value": rate, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": desc + f" ({dt:.1f} s)"}


# ------------------------------------------------------- reference arm

def run_reference(args):
    ws, rank, local = dist_setup("gloo")
    if rank != 0:
        return
    import torch

    from fasterbackprojection_gb300 import make_info, scenes

    # The capture itself comes from the same generator; it needs a device for
    # the patch scene, otherwise fall back to a point scene of the same shape.
    if torch.cuda.is_available():
        cap, info = make_workload(torch.device("cuda", local), 2, args.size)
        cube = cap.cube.cpu().numpy()
        lx = cap.laser_xyz.cpu().numpy()
    else:
        n = SIZES[args.size][0]
        capn = scenes.confocal_points(n, N_BINS, DT, n_points=200, seed=2)
        hmin, vs = scenes.volume_geometry(VRES, depth_range=(0.0, 1.5))
        info = make_info(num_laser_targets=n * n, num_time_bins=N_BINS, time_step=capn.time_step, voxel_res=VRES,
                         hidden_min=hmin, voxel_size=vs)
        cube, lx = capn.cube, capn.laser_xyz
    rates = []
    desc = ""
    for k in range(args.warmup + args.steps):
        r, desc, dt = cpu_sample_rate(info, cube, lx, target_s=4.0, threads=os.cpu_count() or 1)
        if k >= args.warmup:
            rates.append(r)
    value = statistics.mean(rates)
    L = info.num_laser_targets
    V = info.voxel_res[0] * info.voxel_res[1] * info.voxel_res[2]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": V * L / value * 1e3, "ms_per_step_kind":
            "extrapolated: each step times a bounded voxel sample (cpu_baseline.sample) and scales its rate to "
            "the full workload; no full step ran",
        "measured_wall_s_per_step": dt, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "volume": list(info.voxel_res), "scan": [int(round(L ** 0.5))] * 2,
                   "bins": N_BINS},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                         "sample": desc + " per step; the reference has no CPU backprojection, this is the "
                                          "oracle's FP32 restatement of backprojectConfocalVoxel"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_only(args):
    """One extra leg alone (for profiling command lines)."""
    import torch

    from fasterbackprojection_gb300 import Context

    dev = torch.device("cuda", 0)
    cap, info = make_workload(dev, 2, args.size)
    ctx = Context(0)
    cube, lx = cap.cube.contiguous(), cap.laser_xyz.contiguous()
    vx, vy, vz = info.voxel_res
    vol = torch.empty((vz, vy, vx), device=dev)
    ctx.backproject_confocal(info, cube, lx, out=vol)
    pk = measured_peaks()[0]
    legs = {
        "exhaustive": lambda: exhaustive_leg(ctx, dev),
        "filters": lambda: filters_leg(ctx, dev, vol, cube, info.time_step, pk),
        "lct": lambda: lct_leg(ctx, dev, pk),
        "scatter_forms": lambda: scatter_forms_leg(ctx, dev, info, cube, lx),
        "batched": lambda: batched_leg(ctx, dev, max(1, args.steps)),
        "reference_kernels": lambda: reference_kernels_leg(ctx, dev, info, cube, lx, vol),
        "learned": lambda: learned_mis_leg(ctx, dev, info, cube, lx),
    }
    res = legs[args.only]()
    ctx.check_device_status()
    print(json.dumps({"only": args.only, args.only: res}), flush=True)
    ctx.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.only:
        run_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
