"""FP64 NumPy restatements of the temporal filter and the LCT pipeline.

TEST INFRASTRUCTURE ONLY — see oracle/__init__.py.

filter_h       Laser::filter_H_cuda + padIntensity (FasterBackprojection/Laser.cu:80-240),
               the literal padded-FFT computation in float64.
define_psf     python/lct.py:295-347
resampling_operator  python/lct.py:350-419, built directly as the pooled M x M
               matrix instead of the dense M^2 x M intermediate (same values).
lct            python/lct.py:97-211 steps 1-4 for an already-loaded capture
               (no downsampling, no z_trim: synthetic input).
Pinned against the reference's own lct.py functions through the fixtures in
tests/golden/ (made by tests/golden/make_golden.py).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp

LIGHT_SPEED = 299792458.0  # math.cuh:10


def filter_h_params(nt: int, delta_t: float, wl_mean: float, wl_sigma: float = 0.0):
    f32 = np.float32
    wl_sigma = f32(wl_sigma)
    wl_mean = f32(wl_mean)
    if abs(float(wl_sigma) - 0.0) < float(np.finfo(np.float32).eps):
        wl_sigma = f32(wl_mean / f32(math.sqrt(2.0)))
    r = f32(f32(6) * wl_sigma / f32(delta_t))
    t6 = int(math.floor(float(r) + 0.5)) if r >= 0 else -int(math.floor(-float(r) + 0.5))
    if t6 % 2 == 1:
        t6 += 1
    nt_pad = nt + 2 * (t6 - 1)
    return float(wl_sigma), t6, nt_pad


def filter_h_kernel(nt_pad: int, delta_t: float, wl_mean: float, wl_sigma: float) -> np.ndarray:
    """The ifft-shifted complex kernel K (Laser.cu:142-172), float64."""
    t = np.arange(nt_pad, dtype=np.float64) * delta_t
    tmax = delta_t * (nt_pad - 1)
    env = np.exp(-(((t - tmax * 0.5) / wl_sigma) ** 2) * 0.5)
    phase = 2.0 * np.pi * t / wl_mean
    K = env * (np.cos(phase) + 1j * np.sin(phase)) / env.sum()
    shift = nt_pad // 2
    return K[(np.arange(nt_pad) + shift) % nt_pad]


def filter_h(data: np.ndarray, delta_t: float, wl_mean: float | None = None, wl_sigma: float = 0.0,
             border: str = "zero") -> np.ndarray:
    """data[..., T] float -> filtered float64, same shape."""
    data = np.asarray(data)
    T = data.shape[-1]
    flat = data.reshape(-1, T).astype(np.float64)
    wl_mean = delta_t * 10.0 if wl_mean is None else wl_mean
    sigma, t6, n = filter_h_params(T, delta_t, wl_mean, wl_sigma)
    K = filter_h_kernel(n, float(np.float32(delta_t)), float(np.float32(wl_mean)), sigma)
    pad = (n - T) // 2
    H = np.zeros((flat.shape[0], n), dtype=np.complex128)
    H[:, pad:pad + T] = flat
    if border == "edge":
        H[:, :pad] = flat[:, :1]
        H[:, pad + T:] = flat[:, -1:]
    elif border not in ("zero", "constant"):
        raise ValueError(border)
    # cuFFT's inverse is unnormalised: n * ifft.
    out = np.fft.ifft(np.fft.fft(H, axis=1) * np.fft.fft(K)[None, :], axis=1) * n
    return out[:, pad:pad + T].real.reshape(data.shape)


def define_psf(U: int, V: int, slope: float, center: int | None = None) -> np.ndarray:
    """python/lct.py:295-347; center: the column whose sum normalises the PSF
    before its L2 normalisation, U - 1 in lct.py (default), U in lct_2.py:202."""
    x = np.linspace(-1, 1, 2 * U)
    y = np.linspace(-1, 1, 2 * U)
    z = np.linspace(0, 2, 2 * V)
    gz, gy, gx = np.meshgrid(z, y, x, indexing="ij")
    psf = np.abs(((4.0 * slope) ** 2) * (gx ** 2 + gy ** 2) - gz)
    psf = (psf == np.min(psf, axis=0, keepdims=True)).astype(np.float64)
    c = U - 1 if center is None else center
    psf = psf / np.sum(psf[:, c, c])
    psf = psf / np.linalg.norm(psf.ravel())
    return np.roll(psf, shift=(0, U, U), axis=(0, 1, 2))


def resampling_operator(M: int):
    """(mtx, mtxi) as sparse M x M matrices; mtxi == mtx.T."""
    K = int(round(math.log2(M)))
    if 2 ** K != M:
        raise ValueError("resampling operator needs a power-of-two bin count")
    i = np.arange(M * M, dtype=np.float64)
    col = np.clip(np.ceil(np.sqrt(i + 1)) - 1, 0, M - 1).astype(np.int64)
    val = 1.0 / np.sqrt(i + 1)
    row = (np.arange(M * M) // M).astype(np.int64)  # pooled 2^K = M rows into one, weight 1/M
    mtx = sp.coo_matrix((val / M, (row, col)), shape=(M, M)).tocsr()
    mtx.sum_duplicates()
    return mtx, mtx.T.tocsr()


def radiometric_grid(M: int, N: int, mode: str = "reference") -> np.ndarray:
    """grid_z of python/lct.py:134-136.  The reference tiles linspace(0, 1, M)
    with np.tile(col, (1, N, N)).reshape(M, N, N), which gives
    grid_z[a, b, c] = linspace[(a*N + b) % M]; mode "depth" is the per-depth
    grid the comment there describes (grid_z[a] = linspace[a])."""
    lin = np.linspace(0, 1, M)
    if mode == "reference":
        a = np.arange(M)[:, None, None]
        b = np.arange(N)[None, :, None]
        return np.broadcast_to(lin[(a * N + b) % M], (M, N, N))
    if mode == "depth":
        return np.broadcast_to(lin[:, None, None], (M, N, N))
    raise ValueError(mode)


def lct(data_tmajor: np.ndarray, width: float, bin_length: float, snr: float = 0.8, diffuse: bool = True,
        psf: np.ndarray | None = None, mtx=None, mtxi=None, grid: str = "reference",
        output: str = "clamped_real") -> np.ndarray:
    """Confocal LCT of data[M][N][N] (time-major; python/lct.py:129 order).

    bin_length: path length per bin in metres (c * bin_resolution).
    output: "clamped_real" max(real(vol), 0) (python/lct.py:154) or
    "magnitude" abs(vol) (python/lct_2.py:154; lct_2.py also uses the per-depth
    grid, grid="depth", lct_2.py:103).
    Returns vol[M][N][N] float64 (depth, y, x)."""
    M, N, N2 = data_tmajor.shape
    assert N == N2
    range_max = M * bin_length
    if psf is None:
        psf = define_psf(N, M, width / range_max)
    fpsf = np.fft.fftn(psf)
    invpsf = np.conj(fpsf) / (np.abs(fpsf) ** 2 + 1.0 / snr)
    if mtx is None:
        mtx, mtxi = resampling_operator(M)
    grid_z = radiometric_grid(M, N, grid)
    data = data_tmajor.astype(np.float64) * (grid_z ** 4 if diffuse else grid_z ** 2)
    tdata = np.zeros((2 * M, 2 * N, 2 * N), dtype=np.complex128)
    tdata[:M, :N, :N] = (mtx @ data.reshape(M, N * N)).reshape(M, N, N)
    tvol = np.fft.ifftn(np.fft.fftn(tdata) * invpsf)[:M, :N, :N]
    vol = (mtxi @ tvol.reshape(M, N * N)).reshape(M, N, N)
    if output == "magnitude":
        return np.abs(vol)
    return np.maximum(np.real(vol), 0)


# ------------------------------------------------------------ ellipsoid splat

def splat_backproject(info, cube, laser_xyz, max_bins=700, grid=(256, 256)) -> np.ndarray:
    """The rasterised ellipsoid splat (FasterBackprojection/DrawEllipsoids.cpp:
    12-114, 332-440; backprojection-vs/fs.glsl) as fasterbackprojection_gb300's
    fbp_splat_backproject samples it: exact hemispheres towards -y at a grid of
    pixel centres over the volume's x / z extent, every operation in IEEE
    float32 in the same order (so voxel indices are the GPU's), sums in FP64.
    Bounce terms are not supported here (discard_first_last_bounces = 1).
    cube: [L][T] (time innermost).  Returns vol[Vz][Vy][Vx] float64."""
    f = np.float32
    cube = np.asarray(cube, dtype=np.float32)
    L, T = cube.shape
    nb = min(T, max_bins) if max_bins else T
    Vx, Vy, Vz = (int(v) for v in info.voxel_res)
    vs = [f(v) for v in info.voxel_size]
    hm = [f(v) for v in info.hidden_min]
    gw, gh = grid
    px = f(vs[0] * f(Vx)) / f(gw)
    pz = f(vs[2] * f(Vy)) / f(gh)
    x0 = f(hm[0] + f(f(0.5) * px))
    z0 = f(hm[2] + f(f(0.5) * pz))
    xs = (x0 + np.arange(gw, dtype=np.float32) * px).astype(np.float32)
    zs = (z0 + np.arange(gh, dtype=np.float32) * pz).astype(np.float32)
    X, Z = np.meshgrid(xs, zs, indexing="xy")
    vol = np.zeros((Vz, Vy, Vx), dtype=np.float64)
    ls, ts = np.nonzero(cube[:, :nb] > f(1.1920929e-7))
    lx = np.asarray(laser_xyz, dtype=np.float32)
    for l, t in zip(ls, ts):
        path = f(f(f(t) * f(info.time_step)) + f(info.time_offset))
        r = f(f(0.5) * path)
        if not r > 0:
            continue
        c = lx[l]
        dx = (X - c[0]).astype(np.float32)
        dz = (Z - c[2]).astype(np.float32)
        h2 = ((f(r * r) - (dx * dx).astype(np.float32)).astype(np.float32) - (dz * dz).astype(np.float32))
        h2 = h2.astype(np.float32)
        ok = h2 >= 0
        y = (c[1] - np.sqrt(np.where(ok, h2, f(0)))).astype(np.float32)
        fx = ((X - hm[0]).astype(np.float32) / vs[0]).astype(np.float32)
        fy = ((y - hm[1]).astype(np.float32) / vs[1]).astype(np.float32)
        fz = ((Z - hm[2]).astype(np.float32) / vs[2]).astype(np.float32)
        ok &= (fx >= 0) & (fy >= 0) & (fz >= 0)
        vx, vz, vy = fx.astype(np.int64), fy.astype(np.int64), fz.astype(np.int64)
        ok &= (vx < Vx) & (vy < Vy) & (vz < Vz)
        np.add.at(vol, (vz[ok], vy[ok], vx[ok]), float(cube[l, t]))
    return vol


def transient_image(slice_, width, height, size, stride=1, offset=0, normalize=False) -> np.ndarray:
    """TransientImage::save (FasterBackprojection/TransientImage.cpp:46-64) of
    one plane: grey RGBA8 clamp(uint(v * 255), 0, 255) of
    slice[offset + idx * stride], rows flipped (Image.h:160-178), then the
    bilinear Image::resize (Image.h:45-66, 92-138) to size = (w, h) when it
    differs, every operation in IEEE float32 in the reference's order.
    normalize divides the plane by max(0, its maximum) (the reference divides
    the first width * height floats, the same plane for stride 1, offset 0).
    Negative or NaN products become 0.  Returns uint8 [h][w][4], rows top first."""
    f = np.float32
    s = np.asarray(slice_, dtype=np.float32)
    n = width * height
    v = s[offset + np.arange(n, dtype=np.int64) * stride].astype(np.float32)
    if normalize:
        m = f(max(0.0, float(np.nanmax(v)) if np.any(~np.isnan(v)) else 0.0))
        with np.errstate(divide="ignore", invalid="ignore"):
            v = (v / m).astype(np.float32)
    with np.errstate(invalid="ignore", over="ignore"):
        p = (v * f(255.0)).astype(np.float32)
        p = np.where(np.isnan(p) | (p < 0), f(0), np.minimum(np.trunc(p), f(255)))
    grey = p.reshape(height, width)[::-1].astype(np.float32)  # flipped, values 0..255
    ow, oh = size
    if (ow, oh) == (width, height):
        out = np.empty((height, width, 4), np.uint8)
        out[..., :3] = grey.astype(np.uint8)[..., None]
        out[..., 3] = 255
        return out
    xr = f(f(width - 1) / f(ow - 1))
    yr = f(f(height - 1) / f(oh - 1))
    xs = (np.arange(ow, dtype=np.float32) * xr).astype(np.float32)
    ys = (np.arange(oh, dtype=np.float32) * yr).astype(np.float32)
    x0 = np.minimum(xs.astype(np.int64), width - 1)
    y0 = np.minimum(ys.astype(np.int64), height - 1)
    x1 = np.minimum(x0 + 1, width - 1)
    y1 = np.minimum(y0 + 1, height - 1)
    dx = (xs - x0.astype(np.float32)).astype(np.float32)[None, :]
    dy = (ys - y0.astype(np.float32)).astype(np.float32)[:, None]
    ex = (f(1) - dx).astype(np.float32)
    ey = (f(1) - dy).astype(np.float32)

    def lerp(p00, p01, p10, p11):
        a = ((ex * ey).astype(np.float32) * p00).astype(np.float32)
        a = (a + ((dx * ey).astype(np.float32) * p01).astype(np.float32)).astype(np.float32)
        a = (a + ((ex * dy).astype(np.float32) * p10).astype(np.float32)).astype(np.float32)
        return (a + ((dx * dy).astype(np.float32) * p11).astype(np.float32)).astype(np.float32)

    g = lerp(grey[y0][:, x0], grey[y0][:, x1], grey[y1][:, x0], grey[y1][:, x1])
    a = lerp(f(255), f(255), f(255), f(255))
    out = np.empty((oh, ow, 4), np.uint8)
    out[..., :3] = np.minimum(np.trunc(g), 255).astype(np.uint8)[..., None]
    out[..., 3] = np.broadcast_to(np.minimum(np.trunc(a), 255).astype(np.uint8), (oh, ow))
    return out


def _mis_scatter_walk(cube, l, w, dist, vs, dt, T) -> np.ndarray:
    """transient_reconstruction.cuh:235-250 for one sample of every voxel:
    the terms w * I / dist^2 over the walk's bins (I > 1e-5), FP64."""
    ext = 0.5 * float(np.sqrt(vs @ vs))
    step = dt + float(np.float32(1e-5))
    d = np.maximum(0.0, dist - ext)
    dmax = dist + ext
    wt = w / (dist * dist)
    acc = np.zeros(dist.shape[0])
    alive = d < dmax
    while alive.any():
        x = d / dt
        inside = (x > -1) & (x < T)
        alive &= inside  # the reference's thread returns at the first bin outside [0, T)
        b = np.clip(x, 0, T - 1).astype(np.int64)
        I = np.where(alive, cube[l, b], 0.0)
        acc += np.where(alive & (I > 1e-5), wt * I, 0.0)
        d = np.where(alive, d + step, d)
        alive &= d < dmax
    return acc


def scatter_walk_f32(cube, l, dist, rcp_dt: float, ext: float, dt: float, T: int) -> np.ndarray:
    """The voxel-scattering walk (transient_reconstruction.cuh:112-126, 235-250)
    replayed in float32 from given FP32 paths `dist` (the GPU's, from
    fbp_debug_confocal_paths) and the GPU's rcp.approx(timeStep) and half
    voxel diagonal: d = max(0, dist - ext), d += timeStep + EPS while
    d < dist + ext, bin = int(d * rcp_dt), stop at the first bin outside
    [0, T).  Every step is an IEEE float32 operation, so the bins are the
    GPU's bit for bit.  Returns the sum of I (> 1e-5) over each walk, FP64
    (the caller applies the weight)."""
    f = np.float32
    dist = np.asarray(dist, dtype=np.float32)
    step = f(f(dt) + f(1e-5))
    d = np.maximum(f(0), (dist - f(ext)).astype(np.float32))
    dmax = (dist + f(ext)).astype(np.float32)
    acc = np.zeros(dist.shape, dtype=np.float64)
    alive = d < dmax
    while alive.any():
        b = np.trunc((d * f(rcp_dt)).astype(np.float32)).astype(np.int64)
        alive &= (b >= 0) & (b < T)  # the reference's thread returns at the first bin outside [0, T)
        I = np.where(alive, cube[l, np.clip(b, 0, T - 1)], 0.0)
        acc += np.where(alive & (I > 1e-5), I, 0.0)
        d = np.where(alive, (d + step).astype(np.float32), d)
        alive &= d < dmax
    return acc


def safe_rcp_sq(dist) -> np.ndarray:
    """safeRCP(dist^2) (math.cuh:23-29) in FP64."""
    dd = np.asarray(dist, dtype=np.float64) ** 2
    return np.where(dd > 1e-5, 1.0 / np.where(dd > 1e-5, dd, 1.0), float(np.finfo(np.float32).max))


def confocal_scatter_given_paths(cube, paths, rcp_dt: float, ext: float, dt: float) -> np.ndarray:
    """backprojectConfocalVoxel of the ACCUMULATE_VOXEL_SCATTERING build for
    the voxels whose GPU paths [n][L] are given: sum over scan points of
    I(bin) * safeRCP(dist^2) over each walk, FP64 sums of the FP32 walk."""
    cube = np.asarray(cube, dtype=np.float32)
    L, T = cube.shape
    paths = np.asarray(paths, dtype=np.float32).reshape(-1, L)
    l = np.broadcast_to(np.arange(L), paths.shape)
    return (scatter_walk_f32(cube, l, paths, rcp_dt, ext, dt, T) * safe_rcp_sq(paths)).sum(axis=1)


def mis_reference(info, cube, laser_xyz, cdf, alias, prob, noise, samples, bins=None,
                  scatter: bool = False, paths=None, consts=None) -> np.ndarray:
    """Sum over samples s < `samples` of backprojectConfocalVoxelMIS
    (FasterBackprojection/transient_reconstruction.cuh:194-260, without the
    race of its `+=`): voxel v, sample s starts its generator at state v + s
    (uint32, :209), draws from the noise buffer with
    getUniformRandom / getMISIndexAlias (transient_utils.cuh:18-53) and picks
    the alias or the uniform proposal with the balance weight, all in float32
    as the kernel does; the term weight * I / dist^2 is summed in FP64.
    bins: [V][L] int32 time bins (the GPU's, from fbp_debug_confocal_bins),
    else FP64 bins.  scatter: the ACCUMULATE_VOXEL_SCATTERING build
    (transient_reconstruction.cuh:235-250): each sample adds every bin of the
    path d = max(0, dist - ext) .. dist + ext (exclusive, steps of
    timeStep + EPS, ext = |voxelSize| / 2) until a bin leaves [0, T); in FP64
    by default, or, with the GPU's FP32 paths [V][L] and consts
    (rcp_dt, ext) from fbp_debug_confocal_paths, replayed in float32 with the
    GPU's bins (scatter_walk_f32).
    cube: [L][T].  Returns vol[Vz][Vy][Vx] float64."""
    if scatter and bins is not None:
        raise ValueError("mis_reference: given bins and the scattering walk exclude each other")
    if int(info.discard_first_last_bounces) == 0:
        raise NotImplementedError("mis_reference: bounce terms are not restated here")
    f = np.float32
    cube = np.asarray(cube, dtype=np.float32)
    L, T = cube.shape
    Vx, Vy, Vz = (int(v) for v in info.voxel_res)
    V = Vx * Vy * Vz
    noise = np.asarray(noise, dtype=np.float32)
    n = np.uint64(noise.shape[0])
    cdf = np.asarray(cdf, dtype=np.float32)
    alias = np.asarray(alias, dtype=np.int64)
    prob = np.asarray(prob, dtype=np.float32)
    spatial_pdf = np.concatenate([cdf[:1], (cdf[1:] - cdf[:-1]).astype(np.float32)]).astype(np.float32)
    inv_l = f(1.0) / f(L) if f(L) > f(1e-5) else np.finfo(np.float32).max
    v = np.arange(V, dtype=np.int64)
    vz, rem = v // (Vx * Vy), v % (Vx * Vy)
    vy, vx = rem // Vx, rem % Vx
    hm = np.asarray(info.hidden_min, dtype=np.float64)
    vs = np.asarray(info.voxel_size, dtype=np.float64)
    p = np.stack([hm[0] + (vx + 0.5) * vs[0], hm[1] + (vz + 0.5) * vs[1], hm[2] + (vy + 0.5) * vs[2]], axis=1)
    lx = np.asarray(laser_xyz, dtype=np.float64)
    out = np.zeros(V, dtype=np.float64)

    def draw(state):
        state = (state * np.uint64(747796405) + np.uint64(2891336453)) & np.uint64(0xFFFFFFFF)
        return state, noise[(state % n).astype(np.int64)]

    for s in range(samples):
        state = ((v + s) & 0xFFFFFFFF).astype(np.uint64)
        state, r0 = draw(state)
        use_alias = r0 < f(0.5)
        state_a, r1 = draw(state)
        state_a, r2 = draw(state_a)
        k = np.minimum((r1 * f(L)).astype(np.float32).astype(np.int64), L - 1)
        l_alias = np.where(r2 < prob[k], k, alias[k])
        _, ru = draw(state)
        l_unif = np.minimum((ru * f(L)).astype(np.float32).astype(np.int64), L - 1)
        l = np.where(use_alias, l_alias, l_unif)
        pdf = np.where(use_alias, spatial_pdf[l], inv_l).astype(np.float32)
        gpdf = np.where(use_alias, (spatial_pdf[l] + inv_l).astype(np.float32),
                        (inv_l + spatial_pdf[l]).astype(np.float32)).astype(np.float32)
        w = pdf.astype(np.float64) / gpdf.astype(np.float64)
        dist = 2.0 * np.linalg.norm(p - lx[l], axis=1) - float(info.time_offset)
        if scatter and paths is not None:
            d32 = np.asarray(paths, dtype=np.float32).reshape(V, L)[v, l]
            out += w * safe_rcp_sq(d32) * scatter_walk_f32(cube, l, d32, consts[0], consts[1],
                                                           float(info.time_step), T)
            continue
        if scatter:
            out += _mis_scatter_walk(cube, l, w, dist, vs, float(info.time_step), T)
            continue
        if bins is None:
            b = np.floor(dist / float(info.time_step)).astype(np.int64)
        else:
            b = np.asarray(bins, dtype=np.int64).reshape(V, L)[v, l]
        ok = (b >= 0) & (b < T)
        I = np.where(ok, cube[l, np.clip(b, 0, T - 1)], 0.0)
        ok &= I > 1e-5
        out += np.where(ok, w * I / (dist * dist), 0.0)
    return out.reshape(Vz, Vy, Vx)
