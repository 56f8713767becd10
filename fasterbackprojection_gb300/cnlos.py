"""The host side of python/lct.py's confocal NLOS reconstruction
(cnlos_reconstruction, lct.py:8-236) around the GPU light-cone transform.

lct.py loads a capture (.mat: rect_data [N][N][M] and width), halves the
temporal resolution K times by summing bin pairs, zeroes the first z_trim bins
(the direct component), runs the LCT (steps 1-4: fbp_lct here) and crops and
flips the volume for display.  Everything but the LCT is host-side array
bookkeeping and stays in NumPy, as in lct.py; plotting is left to the caller
(`views` gives the three projections lct.py draws).
"""
from __future__ import annotations

from dataclasses import dataclass, replace

import numpy as np

from . import _lib

C_LIGHT = 3e8  # lct.py:26 (the script's speed of light)
NATIVE_BIN_S = 4e-12  # lct.py:25: native SPAD bin of the captures

# lct.py:39-71: scene number -> capture file, first displayed depth bin, diffuse.
SCENES = {
    1: ("data_resolution_chart_40cm.mat", 350, False),
    2: ("data_resolution_chart_65cm.mat", 700, False),
    3: ("data_dot_chart_40cm.mat", 350, False),
    4: ("data_dot_chart_65cm.mat", 700, False),
    5: ("data_mannequin.mat", 300, False),
    6: ("data_exit_sign.mat", 600, False),
    7: ("data_s_u.mat", 800, False),
    8: ("data_outdoor_s.mat", 700, False),
    9: ("data_diffuse_s.mat", 100, True),
}


@dataclass(frozen=True)
class Settings:
    """The adjustable parameters of lct.py:24-33.  lct.py's isbackprop
    (conj(F) instead of the Wiener filter) is not offered: fbp_lct always
    applies the Wiener filter."""

    bin_resolution: float = NATIVE_BIN_S  # seconds per bin of the capture
    K: int = 1  # halvings of the temporal resolution
    snr: float = 0.8
    z_trim: int = 600  # capture bins zeroed from the start
    z_offset: int = 0  # first displayed depth bin (capture bins)
    isdiffuse: bool = False


def scene_settings(scene: int, base: Settings = Settings()) -> tuple[str, Settings]:
    """lct.py:39-71: the capture file of scene 1..9 and its settings (scene 9
    is diffuse: grid_z^4 radiometry and a tenth of the SNR)."""
    if scene not in SCENES:
        raise ValueError("Invalid scene number. Choose between 1 and 9.")
    name, z_offset, diffuse = SCENES[scene]
    s = replace(base, z_offset=z_offset)
    if diffuse:
        s = replace(s, isdiffuse=True, snr=s.snr * 1e-1)
    return "lct/" + name, s


def load_capture(path) -> tuple[np.ndarray, float]:
    """lct.py:79-90: rect_data [N][N][M] and width (0.4 m when the file has
    none, lct.py's stand-in)."""
    import scipy.io

    m = scipy.io.loadmat(str(path))
    if "rect_data" not in m:
        raise ValueError(f"{path}: no rect_data")
    rect = np.asarray(m["rect_data"])
    if rect.ndim != 3 or rect.shape[0] != rect.shape[1]:
        raise ValueError(f"{path}: rect_data must be N x N x M, got {rect.shape}")
    width = float(m["width"].item()) if "width" in m else 0.4
    return rect, width


@dataclass(frozen=True)
class Prepared:
    data: np.ndarray  # [M][N][N] float32, time-major (lct.py:129 order)
    bin_resolution: float  # seconds per bin after downsampling
    range_max: float  # M * c * bin_resolution of the capture (lct.py:95)
    z_trim: int  # in downsampled bins
    z_offset: int  # in downsampled bins

    @property
    def bin_length(self) -> float:
        """Metres of path per (downsampled) bin: fbp_lct's bin_length."""
        return C_LIGHT * self.bin_resolution


def prepare(rect_data, s: Settings = Settings()) -> Prepared:
    """lct.py:93-129 up to the LCT: the range of the capture, K pair-sum
    downsamplings (z_trim and z_offset halved with round() each time), the
    first z_trim bins zeroed, and the permutation to [M][N][N].  The caller's
    array is not modified; sums keep its element type, as in lct.py."""
    rect = np.array(rect_data, copy=True)
    if rect.ndim != 3 or rect.shape[0] != rect.shape[1]:
        raise ValueError(f"rect_data must be N x N x M, got {rect.shape}")
    M = rect.shape[2]
    bin_res = s.bin_resolution
    range_max = M * C_LIGHT * bin_res
    z_trim, z_offset = s.z_trim, s.z_offset
    for _ in range(s.K):
        if rect.shape[2] % 2:
            raise ValueError(f"cannot halve {rect.shape[2]} bins")
        bin_res = 2 * bin_res
        rect = rect[:, :, 0::2] + rect[:, :, 1::2]
        z_trim = round(z_trim / 2)
        z_offset = round(z_offset / 2)
    rect[:, :, :z_trim] = 0
    data = np.ascontiguousarray(np.transpose(rect, (2, 1, 0)), dtype=np.float32)
    return Prepared(data, bin_res, range_max, z_trim, z_offset)


def display_depths(num_depths: int, prepared: Prepared, width: float) -> int:
    """lct.py:227: ind = round(M * 2 * width / (range / 2)) depth bins shown."""
    return round(num_depths * 2 * width / (prepared.range_max / 2))


def display_crop(vol, prepared: Prepared, width: float):
    """lct.py:229-236: x reversed, then depths z_offset .. z_offset + ind.
    NumPy arrays or torch tensors ([M][N][N])."""
    ind = display_depths(vol.shape[0], prepared, width)
    z0 = prepared.z_offset
    if isinstance(vol, np.ndarray):
        return vol[:, :, ::-1][z0:z0 + ind]
    import torch

    return torch.flip(vol, dims=[2])[z0:z0 + ind]


def axes(num_depths: int, n: int, prepared: Prepared, width: float):
    """lct.py:221-223, 235: tic_z (cropped), tic_y, tic_x in metres."""
    tic_z = np.linspace(0, prepared.range_max / 2, num_depths)
    ind = display_depths(num_depths, prepared, width)
    tic = np.linspace(-width, width, n)
    return tic_z[prepared.z_offset:prepared.z_offset + ind], tic, tic.copy()


def views(vol: np.ndarray) -> dict[str, np.ndarray]:
    """The three maximum projections lct.py plots (lct.py:241-287): front
    (over depth), top (over y) and side (over x, transposed)."""
    v = np.asarray(vol)
    return {"front": v.max(axis=0), "top": v.max(axis=1), "side": v.max(axis=2).T}


def reconstruct(ctx, rect_data, width: float, s: Settings = Settings(),
                grid_mode: int = _lib.FBP_LCT_GRID_REFERENCE, crop: bool = True, device=None, stream=None,
                variant: str = "lct"):
    """cnlos_reconstruction without the plots: the host preparation, the LCT
    on the GPU (fbp_lct on the [M][N][N] time-major data), then the display
    crop.  variant "lct_2" is python/lct_2.py's form: per-depth radiometry
    and abs(vol) (grid_mode is then ignored).  Returns a tensor on the
    context's device."""
    import torch

    if variant not in ("lct", "lct_2"):
        raise ValueError("variant must be 'lct' or 'lct_2'")
    p = prepare(rect_data, s)
    dev = device if device is not None else torch.device("cuda", ctx.device)
    data = torch.from_numpy(p.data).to(dev)
    if variant == "lct_2":
        grid_mode = _lib.FBP_LCT_GRID_DEPTH
    output = _lib.FBP_LCT_OUTPUT_MAGNITUDE if variant == "lct_2" else _lib.FBP_LCT_OUTPUT_CLAMPED_REAL
    vol = ctx.lct(data, width, p.bin_length, snr=s.snr, diffuse=s.isdiffuse, grid_mode=grid_mode,
                  layout=_lib.FBP_LAYOUT_TIME_MAJOR, stream=stream, output=output)
    return display_crop(vol, p, width) if crop else vol
