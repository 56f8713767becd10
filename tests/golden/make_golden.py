"""Generates tests/golden/lct_golden.npz from the reference's own python/lct.py.

Run where the reference tree is present:
    python tests/golden/make_golden.py [/path/to/reference]
It imports python/lct.py (matplotlib is stubbed: lct.py imports it at module
level but the functions used here never call it) and records:
  * define_psf(U, V, slope) for small grids,
  * resampling_operator(M) for small power-of-two M,
  * a full confocal LCT of a small seeded synthetic capture, computed with the
    reference's define_psf / resampling_operator and the steps of
    cnlos_reconstruction (lct.py:142-211; no downsampling, no z_trim).
The fixtures pin oracle/numpy_ref.py and the GPU LCT.
"""
from __future__ import annotations

import importlib.util
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def import_reference_lct(ref_root: Path):
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", plt)
    spec = importlib.util.spec_from_file_location("reference_lct", ref_root / "python" / "lct.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def synthetic_capture(N: int, M: int, bin_length: float, seed: int) -> np.ndarray:
    """Small seeded confocal capture data[M][N][N] (time-major): 12 points,
    contribution albedo / r^4 at bin round(2r / bin_length)."""
    rng = np.random.default_rng(seed)
    xs = -1 + (np.arange(N) + 0.5) * 2.0 / N
    gx, gy = np.meshgrid(xs, xs, indexing="xy")  # data[t][iy][ix]
    pts = np.stack([rng.uniform(-0.8, 0.8, 12), rng.uniform(-0.8, 0.8, 12), rng.uniform(0.3, 0.9, 12)], 1)
    alb = rng.uniform(0.2, 1.0, 12)
    data = np.zeros((M, N, N))
    for (px, py, pz), a in zip(pts, alb):
        r = np.sqrt((gx - px) ** 2 + (gy - py) ** 2 + pz ** 2)
        b = np.rint(2 * r / bin_length).astype(int)
        ok = b < M
        np.add.at(data, (b[ok], np.nonzero(ok)[0], np.nonzero(ok)[1]), a / r[ok] ** 4)
    return data


def reference_lct(lct, data: np.ndarray, width: float, bin_length: float, snr: float, diffuse: bool) -> np.ndarray:
    M, N, _ = data.shape
    range_max = M * bin_length
    psf = lct.define_psf(N, M, width / range_max)
    fpsf = np.fft.fftn(psf)
    invpsf = np.conj(fpsf) / (np.abs(fpsf) ** 2 + 1.0 / snr)
    mtx, mtxi = lct.resampling_operator(M)
    grid_z = np.tile(np.linspace(0, 1, M)[:, np.newaxis], (1, N, N)).reshape(M, N, N)
    d = data * (grid_z ** 4 if diffuse else grid_z ** 2)
    tdata = np.zeros((2 * M, 2 * N, 2 * N), dtype=np.complex128)
    tdata[:M, :N, :N] = (mtx @ d.reshape(M, N * N)).reshape(M, N, N)
    tvol = np.fft.ifftn(np.fft.fftn(tdata) * invpsf)[:M, :N, :N]
    vol = (mtxi @ tvol.reshape(M, N * N)).reshape(M, N, N)
    return np.maximum(np.real(vol), 0)


def main() -> None:
    # The reference checkout beside this repository unless given.
    ref_root = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parents[3] / "reference"
    lct = import_reference_lct(ref_root)
    out = {}
    for U, V, slope in [(4, 8, 0.3), (8, 16, 0.1), (8, 32, 0.05), (16, 16, 0.25)]:
        out[f"psf_{U}_{V}"] = lct.define_psf(U, V, slope)
        out[f"psf_{U}_{V}_slope"] = np.array(slope)
    for M in (8, 16, 32, 64):
        mtx, mtxi = lct.resampling_operator(M)
        out[f"mtx_{M}"] = np.asarray(mtx)
        out[f"mtxi_{M}"] = np.asarray(mtxi)
    for name, (N, M, bl, snr, diffuse, seed) in {
        "lct_a": (16, 64, 0.03, 0.8, True, 7),
        "lct_b": (8, 32, 0.06, 0.5, False, 11),
    }.items():
        data = synthetic_capture(N, M, bl, seed)
        out[f"{name}_data"] = data.astype(np.float32)
        out[f"{name}_params"] = np.array([1.0, bl, snr, float(diffuse)])
        out[f"{name}_vol"] = reference_lct(lct, data.astype(np.float32).astype(np.float64), 1.0, bl, snr, diffuse)
    np.savez_compressed(HERE / "lct_golden.npz", **out)
    print("wrote", HERE / "lct_golden.npz", sorted(out))


if __name__ == "__main__":
    main()
