"""CPU oracle of the learned MIS proposal (test infrastructure only: the tests
use it to check the GPU kernels; nothing in the product calls it).

There is no reference implementation to follow: the reference's MIS
proposal is a spatial alias table over scan points (FasterBackprojection/
Laser.cu:253-315) and it has no learned component.  This restates, in FP64
NumPy, what the GPU computes (fasterbackprojection_gb300/csrc/mlp.cu):

  * features of (tile, cluster) rows from a capture;
  * the training target q_c ~ sqrt(sum_v F_vc^2) of a tile;
  * the MLP 19 -> 64 -> 64 -> 64 -> 1 (GELU, tanh form) forward pass and the
    gradient of the per-tile softmax cross-entropy, with the GPU's BF16
    rounding points (every tensor-core operand) when ``rounding`` is set, or
    exact FP64 maths when it is not (for finite-difference checks).
"""
from __future__ import annotations

import numpy as np

IN, IN_PAD, FEAT, H = 19, 32, 20, 64
OW1 = 0
OB1 = OW1 + H * IN_PAD
OW2 = OB1 + H
OB2 = OW2 + H * H
OW3 = OB2 + H
OB3 = OW3 + H * H
OW4 = OB3 + H
OB4 = OW4 + H
NPARAM = OB4 + 1
POOL_M = 0.0384
WINDOW = 16
C = np.sqrt(2.0 / np.pi)


def bf16(x) -> np.ndarray:
    """Round to bfloat16 (nearest even) through float32; returned as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    b = ((u + r) & 0xFFFF0000).astype(np.uint32)
    return b.view(np.float32).astype(np.float64)


def _r(x, rounding):
    return bf16(x) if rounding else np.asarray(x, dtype=np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(C * (x + 0.044715 * x ** 3)))


def gelu_d(x):
    t = np.tanh(C * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * C * (1.0 + 3 * 0.044715 * x * x)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return dict(W1=p[OW1:OB1].reshape(H, IN_PAD), b1=p[OB1:OW2], W2=p[OW2:OB2].reshape(H, H), b2=p[OB2:OW3],
                W3=p[OW3:OB3].reshape(H, H), b3=p[OB3:OW4], w4=p[OW4:OB4], b4=p[OB4])


def forward(p, feats, rounding=True):
    """Logits [..., G] of feature rows [..., G, FEAT] and the cache for backward."""
    w = unpack(p)
    a0 = np.zeros(feats.shape[:-1] + (IN_PAD,))
    a0[..., :IN] = feats[..., :IN]
    a0r = _r(a0, rounding)
    x1 = a0r @ _r(w["W1"], rounding).T + w["b1"]
    a1r = _r(gelu(x1), rounding)
    x2 = a1r @ _r(w["W2"], rounding).T + w["b2"]
    a2r = _r(gelu(x2), rounding)
    x3 = a2r @ _r(w["W3"], rounding).T + w["b3"]
    a3 = gelu(x3)
    o = a3 @ w["w4"] + w["b4"]
    return o, dict(a0r=a0r, x1=x1, a1r=a1r, x2=x2, a2r=a2r, x3=x3, a3=a3, w=w)


def loss_and_grad(p, feats, labels, rounding=True):
    """Mean over tiles of -sum_c q_c log softmax(o)_c and its gradient (flat,
    NPARAM).  feats [B, G, FEAT], labels [B, G]."""
    o, k = forward(p, feats, rounding)
    w = k["w"]
    B = o.shape[0]
    m = o.max(axis=1, keepdims=True)
    lse = m + np.log(np.exp(o - m).sum(axis=1, keepdims=True))
    logp = o - lse
    loss = float(-(labels * logp).sum() / B)
    g = (np.exp(logp) - labels) / B
    grad = np.zeros(NPARAM)
    grad[OW4:OB4] = np.einsum("bc,bck->k", g, k["a3"])
    grad[OB4] = g.sum()
    dx3 = g[..., None] * w["w4"] * gelu_d(k["x3"])
    grad[OB3:OW4] = dx3.sum(axis=(0, 1))
    d3 = _r(dx3, rounding)
    grad[OW3:OB3] = np.einsum("bcn,bck->nk", d3, k["a2r"]).ravel()
    da2 = d3 @ _r(w["W3"], rounding)
    dx2 = da2 * gelu_d(k["x2"])
    grad[OB2:OW3] = dx2.sum(axis=(0, 1))
    d2 = _r(dx2, rounding)
    grad[OW2:OB2] = np.einsum("bcn,bck->nk", d2, k["a1r"]).ravel()
    da1 = d2 @ _r(w["W2"], rounding)
    dx1 = da1 * gelu_d(k["x1"])
    grad[OB1:OW2] = dx1.sum(axis=(0, 1))
    d1 = _r(dx1, rounding)
    grad[OW1:OB1] = np.einsum("bcn,bck->nk", d1, k["a0r"]).ravel()
    return loss, grad


# ------------------------------------------------------------ features/labels

def pool_bins(time_step: float) -> int:
    r = np.float32(POOL_M) / np.float32(time_step)
    return 1 if r < 1.5 else int(r + np.float32(0.5))


def cluster_summary(cube, laser_xyz, scan_side: int, cluster_side: int, time_step: float):
    """Pooled mean profiles [G][J], centres [G][4] and the profile mean of a
    capture cube[l][t] (time innermost), in float32 like the GPU."""
    cube = np.asarray(cube, dtype=np.float32)
    L, T = cube.shape
    pool = pool_bins(time_step)
    J = -(-T // pool)
    cpr = -(-scan_side // cluster_side)
    G = cpr * cpr
    prof = np.zeros((G, J), np.float32)
    centre = np.zeros((G, 4), np.float32)
    padded = np.zeros((L, J * pool), np.float32)
    padded[:, :T] = cube
    pooled = padded.reshape(L, J, pool).sum(axis=2, dtype=np.float64)
    for c in range(G):
        cx, cz = c % cpr, c // cpr
        xs = np.arange(cx * cluster_side, min((cx + 1) * cluster_side, scan_side))
        zs = np.arange(cz * cluster_side, min((cz + 1) * cluster_side, scan_side))
        ls = (zs[:, None] * scan_side + xs[None, :]).ravel()
        prof[c] = (pooled[ls].sum(axis=0) / len(ls)).astype(np.float32)
        centre[c, :3] = laser_xyz[ls].astype(np.float64).mean(axis=0)
        centre[c, 3] = len(ls)
    mean = np.float32(prof.astype(np.float64).mean()) + np.float32(1e-30)
    return prof, centre, mean


def tile_centres(info, tiles):
    gx = -(-info.voxel_res[0] // 8)
    gy = -(-info.voxel_res[1] // 16)
    out = []
    for t in tiles:
        bx, by, bz = t % gx, (t // gx) % gy, t // (gx * gy)
        x0, y0, z0 = bx * 8, by * 16, bz * 16
        nx = min(8, info.voxel_res[0] - x0)
        ny = min(16, info.voxel_res[1] - y0)
        nz = min(16, info.voxel_res[2] - z0)
        out.append((info.hidden_min[0] + info.voxel_size[0] * (x0 + 0.5 * nx),
                    info.hidden_min[1] + info.voxel_size[1] * (z0 + 0.5 * nz),
                    info.hidden_min[2] + info.voxel_size[2] * (y0 + 0.5 * ny)))
    return np.asarray(out, dtype=np.float64)


def features(info, cube, laser_xyz, scan_side: int, cluster_side: int, tiles) -> np.ndarray:
    """Feature rows [len(tiles)][G][FEAT] (discarded first/last bounces)."""
    prof, centre, mean = cluster_summary(cube, laser_xyz, scan_side, cluster_side, info.time_step)
    G, J = prof.shape
    ppb = np.float32(info.time_step) * np.float32(pool_bins(info.time_step))
    tc = tile_centres(info, tiles)
    out = np.zeros((len(tiles), G, FEAT), np.float32)
    for i in range(len(tiles)):
        d = tc[i][None, :] - centre[:, :3]
        out[i, :, 0:3] = 0.5 * d
        path = 2.0 * np.sqrt((d * d).sum(axis=1)) - info.time_offset
        j0 = np.floor(path / ppb).astype(np.int64) - WINDOW // 2
        for k in range(WINDOW):
            j = j0 + k
            ok = (j >= 0) & (j < J)
            v = np.where(ok, prof[np.arange(G), np.clip(j, 0, J - 1)], 0.0)
            out[i, :, 3 + k] = np.log1p(np.maximum(v, 0.0) / mean)
    return out


def labels(info, cube, laser_xyz, scan_side: int, cluster_side: int, tiles) -> np.ndarray:
    """FP64 training targets [len(tiles)][G] with FP64 bins (cube[l][t])."""
    cube = np.asarray(cube, dtype=np.float32)
    L, T = cube.shape
    Vx, Vy, Vz = info.voxel_res
    gx, gy = -(-Vx // 8), -(-Vy // 16)
    cpr = -(-scan_side // cluster_side)
    G = cpr * cpr
    dt = float(info.time_step)
    lx = laser_xyz.astype(np.float64)
    out = np.zeros((len(tiles), G))
    for i, t in enumerate(tiles):
        bx, by, bz = t % gx, (t // gx) % gy, t // (gx * gy)
        vx = np.arange(bx * 8, min(bx * 8 + 8, Vx))
        vy = np.arange(by * 16, min(by * 16 + 16, Vy))
        vz = np.arange(bz * 16, min(bz * 16 + 16, Vz))
        X, Yr, Zd = np.meshgrid(vx, vy, vz, indexing="ij")
        px = info.hidden_min[0] + (X.ravel() + 0.5) * info.voxel_size[0]
        py = info.hidden_min[1] + (Zd.ravel() + 0.5) * info.voxel_size[1]
        pz = info.hidden_min[2] + (Yr.ravel() + 0.5) * info.voxel_size[2]
        P = np.stack([px, py, pz], 1)
        F = np.zeros((P.shape[0], G))
        for c in range(G):
            cx, cz = c % cpr, c // cpr
            xs = np.arange(cx * cluster_side, min((cx + 1) * cluster_side, scan_side))
            zs = np.arange(cz * cluster_side, min((cz + 1) * cluster_side, scan_side))
            for l in (zs[:, None] * scan_side + xs[None, :]).ravel():
                dist = 2.0 * np.sqrt(((P - lx[l]) ** 2).sum(axis=1)) - info.time_offset
                b = np.floor(dist / dt).astype(np.int64)
                ok = (b >= 0) & (b < T)
                I = np.where(ok, cube[l, np.clip(b, 0, T - 1)], 0.0)
                I = np.where(I > 1e-5, I, 0.0)
                F[:, c] += I / (dist * dist)
        s = np.sqrt((F * F).sum(axis=0))
        out[i] = s / s.sum() if s.sum() > 0 else 1.0 / G
    return out
