"""Seeded synthetic NLOS captures with the shapes of the benchmark configurations.

No public capture ships with the reference (its HDF5 and .mat inputs are
absent), so these stand in for them.  Conventions:

* relay wall: the plane y = 0, scan points at cell centres of an n x n grid over
  x, z in [-1, 1] m; scan point l = iz * n + ix; wall normal (0, -1, 0); the
  hidden scene lies at negative y (depth = -y).
* time_step (metres of path per bin) = c * dt.
* confocal contribution of a scene point at distance r: albedo / r^4 at bin
  round(2 r / time_step); exhaustive: albedo / (r_l^2 r_s^2) at
  round((r_l + r_s) / time_step).
* noise: the cube is scaled so the mean total count per scan point (or pair)
  is `photons`, then Poisson-sampled with numpy PCG64(seed) (torch's generator
  for the on-device path).
* cubes are time-innermost: confocal [L][T], exhaustive [L][S][T].
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

LIGHT_SPEED = 299792458.0


@dataclass
class Capture:
    cube: object  # numpy array or torch tensor, float32, time innermost
    laser_xyz: object  # [L][3] float32
    sensor_xyz: object | None  # [S][3] float32 (exhaustive only)
    time_step: float
    n_scan: int  # scan grid side (laser grid side for exhaustive)
    num_bins: int


def wall_grid(n: int, half: float = 1.0) -> np.ndarray:
    c = -half + (np.arange(n) + 0.5) * (2 * half / n)
    gz, gx = np.meshgrid(c, c, indexing="ij")
    xyz = np.stack([gx.ravel(), np.zeros(n * n), gz.ravel()], axis=1)
    return xyz.astype(np.float32)


def _poisson(cube: np.ndarray, photons: float, rng: np.random.Generator, per_axis: int = -1) -> np.ndarray:
    tot = cube.sum(axis=per_axis)
    mean_tot = float(tot.mean())
    if mean_tot <= 0:
        return cube.astype(np.float32)
    scale = photons / mean_tot
    return rng.poisson(cube * scale).astype(np.float32)


def random_points(n_points: int, depth_range, seed: int, xz_range=(-1.0, 1.0)):
    rng = np.random.default_rng(seed)
    x = rng.uniform(*xz_range, n_points)
    z = rng.uniform(*xz_range, n_points)
    depth = rng.uniform(*depth_range, n_points)
    albedo = rng.uniform(0.2, 1.0, n_points)
    return np.stack([x, -depth, z], axis=1), albedo, rng


def confocal_points(n: int, T: int, dt_s: float, n_points: int = 200, depth_range=(0.4, 1.2), seed: int = 1,
                    photons: float = 1e4, noise: bool = True) -> Capture:
    """Confocal point-scene capture (the 64^2 x 512 LCT shape and small test cases):
    seeded points, albedo / r^4 at round(2r / (c dt))."""
    step = LIGHT_SPEED * dt_s
    lx = wall_grid(n)
    pts, alb, rng = random_points(n_points, depth_range, seed)
    cube = np.zeros((n * n, T), dtype=np.float64)
    L = n * n
    for i in range(0, n_points, 64):
        p = pts[i:i + 64]
        a = alb[i:i + 64]
        r = np.linalg.norm(lx[:, None, :].astype(np.float64) - p[None, :, :], axis=2)  # [L, P]
        b = np.rint(2 * r / step).astype(np.int64)
        ok = b < T
        li = np.broadcast_to(np.arange(L)[:, None], b.shape)
        np.add.at(cube, (li[ok], b[ok]), (a[None, :] / r ** 4)[ok])
    cube = _poisson(cube, photons, rng) if noise else cube.astype(np.float32)
    return Capture(cube, lx, None, step, n, T)


def confocal_points_torch(n: int, T: int, dt_s: float, n_points: int = 200, depth_range=(0.4, 1.2), seed: int = 1,
                          photons: float = 1e4, device="cuda", noise: bool = True) -> Capture:
    """confocal_points generated on the device (same scene and contribution
    rule; Poisson noise from torch's generator seeded with `seed`)."""
    import torch

    step = LIGHT_SPEED * dt_s
    lx = torch.from_numpy(wall_grid(n)).to(device)
    pts, alb, _ = random_points(n_points, depth_range, seed)
    L = n * n
    r = torch.cdist(lx.double(), torch.from_numpy(pts).to(device))  # [L, P]
    b = torch.round(2 * r / step).to(torch.int64)
    ok = b < T
    val = (torch.from_numpy(alb).to(device)[None, :] / r ** 4)
    flat = (torch.arange(L, device=device, dtype=torch.int64)[:, None] * T + b)[ok]
    cube = torch.zeros(L * T, dtype=torch.float64, device=device)
    cube.index_add_(0, flat, val[ok])
    cube = cube.view(L, T)
    if noise:
        tot = cube.sum(dim=1).mean().item()
        if tot > 0:
            g = torch.Generator(device=device)
            g.manual_seed(seed)
            cube = torch.poisson(cube * (photons / tot), generator=g)
    return Capture(cube.float().contiguous(), lx.contiguous(), None, step, n, T)


def exhaustive_points(nl: int, ns: int, T: int, dt_s: float, n_points: int = 500, depth_range=(0.4, 1.4),
                      seed: int = 3, photons: float = 1e4, noise: bool = True) -> Capture:
    """Exhaustive (laser x SPAD) point-scene capture: [L][S][T], albedo / (r_l^2 r_s^2)
    at round((r_l + r_s) / (c dt))."""
    step = LIGHT_SPEED * dt_s
    lx = wall_grid(nl)
    sx = wall_grid(ns)
    pts, alb, rng = random_points(n_points, depth_range, seed)
    L, S = nl * nl, ns * ns
    cube = np.zeros((L, S, T), dtype=np.float64)
    rl_all = np.linalg.norm(lx[:, None, :].astype(np.float64) - pts[None], axis=2)  # [L, P]
    rs_all = np.linalg.norm(sx[:, None, :].astype(np.float64) - pts[None], axis=2)  # [S, P]
    for pi in range(n_points):
        rl = rl_all[:, pi][:, None]
        rs = rs_all[:, pi][None, :]
        b = np.rint((rl + rs) / step).astype(np.int64)
        ok = b < T
        li, si = np.nonzero(ok)
        np.add.at(cube, (li, si, b[ok]), (alb[pi] / (rl ** 2 * rs ** 2))[ok])
    cube = cube.reshape(L * S, T)
    cube = _poisson(cube, photons, rng) if noise else cube.astype(np.float32)
    return Capture(cube.reshape(L, S, T), lx, sx, step, nl, T)


def exhaustive_points_torch(nl: int, ns: int, T: int, dt_s: float, n_points: int = 500, depth_range=(0.4, 1.4),
                            seed: int = 3, photons: float = 1e4, device="cuda", noise: bool = True) -> Capture:
    """exhaustive_points generated on the device: cube [L][S][T] float32."""
    import torch

    step = LIGHT_SPEED * dt_s
    lx = torch.from_numpy(wall_grid(nl)).to(device)
    sx = torch.from_numpy(wall_grid(ns)).to(device)
    pts, alb, _ = random_points(n_points, depth_range, seed)
    L, S = nl * nl, ns * ns
    P = torch.from_numpy(pts).to(device)
    A = torch.from_numpy(alb).to(device)
    rl_all = torch.cdist(lx.double(), P)  # [L, P]
    rs_all = torch.cdist(sx.double(), P)  # [S, P]
    cube = torch.zeros(L * S * T, dtype=torch.float64, device=device)
    base = (torch.arange(L, device=device, dtype=torch.int64)[:, None] * S +
            torch.arange(S, device=device, dtype=torch.int64)[None, :]) * T
    for pi in range(n_points):
        rl = rl_all[:, pi][:, None]
        rs = rs_all[:, pi][None, :]
        b = torch.round((rl + rs) / step).to(torch.int64)
        ok = b < T
        cube.index_add_(0, (base + b)[ok], (A[pi] / (rl ** 2 * rs ** 2)).expand(L, S)[ok])
    cube = cube.view(L * S, T)
    if noise:
        tot = cube.sum(dim=1).mean().item()
        if tot > 0:
            g = torch.Generator(device=device)
            g.manual_seed(seed)
            cube = torch.poisson(cube * (photons / tot), generator=g)
    return Capture(cube.float().view(L, S, T).contiguous(), lx.contiguous(), sx.contiguous(), step, nl, T)


def patch_points(n_patches: int, depth_range, seed: int, sample: float = 0.004):
    """Patch scene of the 256^2 x 1024 confocal workload: planar patches (edge U[0.1, 0.4] m, normal uniform on
    the hemisphere facing the wall) sampled every `sample` metres."""
    rng = np.random.default_rng(seed)
    pts, alb = [], []
    for _ in range(n_patches):
        edge = rng.uniform(0.1, 0.4)
        c = np.array([rng.uniform(-0.8, 0.8), -rng.uniform(*depth_range), rng.uniform(-0.8, 0.8)])
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        if v[1] < 0:  # face the wall (+y)
            v[1] = -v[1]
        t1 = np.cross(v, [1.0, 0.0, 0.0] if abs(v[0]) < 0.9 else [0.0, 0.0, 1.0])
        t1 /= np.linalg.norm(t1)
        t2 = np.cross(v, t1)
        k = max(1, int(round(edge / sample)))
        u = (np.arange(k) + 0.5) / k * edge - edge / 2
        uu, vv = np.meshgrid(u, u, indexing="ij")
        p = c[None] + uu.reshape(-1, 1) * t1[None] + vv.reshape(-1, 1) * t2[None]
        p[:, 1] = np.minimum(p[:, 1], -0.05)
        pts.append(p)
        alb.append(np.full(p.shape[0], rng.uniform(0.2, 1.0)))
    return np.concatenate(pts), np.concatenate(alb), rng


def confocal_patches_torch(n: int, T: int, dt_s: float, n_patches: int = 8, depth_range=(0.3, 1.5), seed: int = 2,
                           photons: float = 1e4, device="cuda", sample: float = 0.004, noise: bool = True) -> Capture:
    """The 256^2 x 1024 confocal patch capture generated on the device (65536 scan points x ~10^5
    scene samples is too slow in NumPy).  Returns torch tensors on `device`."""
    import torch

    step = LIGHT_SPEED * dt_s
    pts, alb, _ = patch_points(n_patches, depth_range, seed, sample)
    lx = torch.from_numpy(wall_grid(n)).to(device)
    L = n * n
    cube = torch.zeros(L * T, dtype=torch.float32, device=device)
    p_all = torch.from_numpy(pts).to(device=device, dtype=torch.float32)
    a_all = torch.from_numpy(alb).to(device=device, dtype=torch.float32)
    lidx = torch.arange(L, device=device, dtype=torch.int64)[:, None]
    chunk = max(1, (1 << 26) // L)
    for i in range(0, p_all.shape[0], chunk):
        p = p_all[i:i + chunk]
        r = torch.cdist(lx.double(), p.double()).float()  # [L, P]
        b = torch.round(2 * r / step).to(torch.int64)
        ok = b < T
        val = (a_all[i:i + chunk][None, :] / r ** 4)
        flat = (lidx * T + b)[ok]
        cube.index_add_(0, flat, val[ok])
    cube = cube.view(L, T)
    if noise:
        tot = cube.sum(dim=1).double().mean().item()
        if tot > 0:
            g = torch.Generator(device=device)
            g.manual_seed(seed)
            cube = torch.poisson(cube * (photons / tot), generator=g)
    return Capture(cube.contiguous(), lx.contiguous(), None, step, n, T)


# ------------------------------------------------------------ configurations


def volume_geometry(vres, x_range=(-1.0, 1.0), depth_range=(0.0, 1.5), z_range=(-1.0, 1.0)):
    """(hidden_min, voxel_size) so that voxel (vx, vy, vz) of a volume with
    voxel_res (Vx, Vy, Vz) covers x in x_range, world z in z_range (vy) and
    depth in depth_range (vz, world y = -depth), the axis mapping of the
    reference kernels (hiddenMin + (vx, vz, vy) * voxelSize)."""
    Vx, Vy, Vz = vres
    hmin = (x_range[0], -depth_range[1], z_range[0])
    vs = ((x_range[1] - x_range[0]) / Vx, (depth_range[1] - depth_range[0]) / Vz, (z_range[1] - z_range[0]) / Vy)
    return hmin, vs


CONFIGS = {
    # name: description of the workload (sizes mirror the benchmark configurations)
    "lct_64x64x512": dict(n=64, T=512, dt=32e-12, vres=(64, 64, 512)),
    "confocal_256x256x1024": dict(n=256, T=1024, dt=16e-12, vres=(256, 256, 256)),
    "exhaustive_16x16_32x32x1024": dict(nl=16, ns=32, T=1024, dt=16e-12, vres=(128, 128, 128)),
}


def batched_configs(seed0: int = 100, count: int = 64):
    """Uneven capture sizes of the batched workload: N in {32,64,128,256},
    T in {256,512,1024,2048}, volume N^3, seeds seed0..seed0+count-1."""
    rng = np.random.default_rng(12345)
    out = []
    for i in range(count):
        N = int(rng.choice([32, 64, 128, 256]))
        T = int(rng.choice([256, 512, 1024, 2048]))
        out.append(dict(n=N, T=T, vres=(N, N, N), seed=seed0 + i))
    return out


def bins_for_depth(T: int, depth_max: float) -> float:
    """time_step (m) so T bins cover round trips to depth_max."""
    return 2.0 * depth_max / T


def to_bits_bf16(a: np.ndarray) -> np.ndarray:
    """float32 -> bfloat16 bit pattern (round to nearest even), as uint16."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def from_bits_bf16(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32)


def math_dt_for(step_m: float) -> float:
    return step_m / LIGHT_SPEED


__all__ = [n for n in dir() if not n.startswith("_") and n not in ("math",)]
