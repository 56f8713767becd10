"""Python-side handle on libfbp: a context plus one method per C entry point.

Device arguments are CUDA torch tensors (contiguous); the calls run on the
current torch stream unless one is given.  Every method raises FbpError on a
non-zero status.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_double, c_float, c_void_p

import numpy as np

from . import _lib
from ._lib import CaptureDesc, LctParams, MisParams, ReconInfo, ShapeParams, check, load


def make_info(*, num_laser_targets: int, num_time_bins: int, time_step: float, voxel_res, hidden_min, voxel_size,
              num_sensor_targets: int | None = None, capture_system: int = _lib.FBP_CONFOCAL,
              time_offset: float = 0.0, discard_first_last_bounces: int = 1, laser_position=(0.0, 0.0, 0.0),
              sensor_position=(0.0, 0.0, 0.0), wall_normal=(0.0, -1.0, 0.0), wall_min=(-1.0, 0.0, -1.0),
              wall_size=(2.0, 0.0, 2.0)) -> ReconInfo:
    """Build an fbp_recon_info.  voxel_res is (Vx, Vy, Vz) of a [Vz][Vy][Vx]
    volume; voxel (vx, vy, vz) sits at hidden_min + (vx, vz, vy)*voxel_size + voxel_size/2."""
    info = ReconInfo()
    info.capture_system = capture_system
    info.num_laser_targets = num_laser_targets
    info.num_sensor_targets = num_sensor_targets if num_sensor_targets is not None else num_laser_targets
    info.num_time_bins = num_time_bins
    info.time_step = time_step
    info.time_offset = time_offset
    info.discard_first_last_bounces = discard_first_last_bounces
    for k in range(3):
        info.laser_position[k] = laser_position[k]
        info.sensor_position[k] = sensor_position[k]
        info.hidden_min[k] = hidden_min[k]
        info.voxel_size[k] = voxel_size[k]
        info.voxel_res[k] = voxel_res[k]
        info.wall_normal[k] = wall_normal[k]
        info.wall_min[k] = wall_min[k]
        info.wall_size[k] = wall_size[k]
    # The reference derives voxel_size = size / res (NLosData.cpp:157), with
    # size = max - min; keep those fields consistent for callers reading them.
    for k in range(3):
        size = float(info.voxel_size[k]) * float(voxel_res[k])
        info.hidden_size[k] = size
        info.hidden_max[k] = float(info.hidden_min[k]) + size
    return info


def _dtype_code(t) -> int:
    import torch

    if t.dtype == torch.float32:
        return _lib.FBP_F32
    if t.dtype == torch.bfloat16:
        return _lib.FBP_BF16
    if t.dtype == torch.float16:
        return _lib.FBP_F16
    raise TypeError(f"unsupported cube dtype {t.dtype}")


def _np_dtype_code(a: np.ndarray) -> int:
    if a.dtype == np.float32:
        return _lib.FBP_F32
    if a.dtype == np.float16:
        return _lib.FBP_F16
    if a.dtype == np.uint16:  # raw bfloat16 bits
        return _lib.FBP_BF16
    raise TypeError(f"unsupported host cube dtype {a.dtype} (float32, float16, or uint16 bfloat16 bits)")


def _ptr(t, min_numel: int = 0, dtype=None, name: str = "tensor") -> c_void_p:
    """Device address of a contiguous CUDA tensor (NULL for None).  The kernels
    take plain pointers, so the sizes they will touch are checked here: a host
    tensor, a tensor smaller than `min_numel` elements or one of another
    element type than `dtype` raises before any launch."""
    if t is None:
        return c_void_p(0)
    if not getattr(t, "is_cuda", False):
        raise TypeError(f"{name} must be a CUDA tensor (got {type(t).__name__}"
                        f"{' on ' + str(t.device) if hasattr(t, 'device') else ''})")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype} (got {t.dtype})")
    if t.numel() < min_numel:
        raise ValueError(f"{name} has {t.numel()} elements, needs at least {min_numel}")
    return c_void_p(t.data_ptr())


def _f32():
    import torch

    return torch.float32


def _voxels(info: ReconInfo) -> int:
    vx, vy, vz = info.voxel_res
    return int(vx) * int(vy) * int(vz)


def _cube_elems(info: ReconInfo, exhaustive: bool = False) -> int:
    L, T = int(info.num_laser_targets), int(info.num_time_bins)
    return L * (int(info.num_sensor_targets) if exhaustive else 1) * T


def _plane_span(width: int, height: int, num_planes: int, pixel_stride: int, plane_stride: int) -> int:
    """Elements up to the last pixel read: plane p pixel i at p*plane_stride + i*pixel_stride."""
    if width <= 0 or height <= 0 or num_planes <= 0:
        return 0
    return (num_planes - 1) * plane_stride + (width * height - 1) * pixel_stride + 1


class Context:
    def __init__(self, device: int = 0):
        self._lib = load()
        h = c_void_p()
        check(self._lib.fbp_create(byref(h), device))
        self._h = h
        self.device = device

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.fbp_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @staticmethod
    def _stream(stream) -> c_void_p:
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        return c_void_p(s.cuda_stream)

    @property
    def launches(self) -> int:
        return int(self._lib.fbp_kernel_launch_count(self._h))

    def check_device_status(self, stream=None) -> None:
        check(self._lib.fbp_check_device_status(self._h, self._stream(stream)))

    @property
    def weight_mode(self) -> int:
        """fbp_weight_mode of the gathers: FBP_WEIGHTS_BATCHED (default) or FBP_WEIGHTS_REFERENCE."""
        m = ctypes.c_int()
        check(self._lib.fbp_get_weight_mode(self._h, byref(m)))
        return m.value

    @weight_mode.setter
    def weight_mode(self, mode: int) -> None:
        check(self._lib.fbp_set_weight_mode(self._h, int(mode)))

    # ---------------------------------------------------------- backprojection
    def backproject_confocal(self, info: ReconInfo, cube, laser_xyz, out=None, layout=_lib.FBP_LAYOUT_TIME_INNER,
                             stream=None):
        import torch

        vx, vy, vz = info.voxel_res
        if out is None:
            out = torch.empty((vz, vy, vx), dtype=torch.float32, device=cube.device)
        check(self._lib.fbp_backproject_confocal(self._h, byref(info), _ptr(cube, _cube_elems(info), name="cube"),
                                                 _dtype_code(cube), layout,
                                                 _ptr(laser_xyz, 3 * info.num_laser_targets, _f32(), "laser_xyz"),
                                                 _ptr(out, _voxels(info), _f32(), "out"), self._stream(stream)))
        return out

    def backproject_confocal_scatter(self, info: ReconInfo, cube, laser_xyz, out=None,
                                     layout=_lib.FBP_LAYOUT_TIME_INNER, stream=None):
        """The reference's ACCUMULATE_VOXEL_SCATTERING variant of the confocal backprojection."""
        import torch

        vx, vy, vz = info.voxel_res
        if out is None:
            out = torch.empty((vz, vy, vx), dtype=torch.float32, device=cube.device)
        check(self._lib.fbp_backproject_confocal_scatter(self._h, byref(info), _ptr(cube, _cube_elems(info), name="cube"),
                                                         _dtype_code(cube), layout,
                                                         _ptr(laser_xyz, 3 * info.num_laser_targets, _f32(), "laser_xyz"),
                                                         _ptr(out, _voxels(info), _f32(), "out"), self._stream(stream)))
        return out

    def splat_backproject(self, info: ReconInfo, cube, laser_xyz, max_bins: int = 700, grid=(256, 256), out=None,
                          layout=_lib.FBP_LAYOUT_TIME_INNER, stream=None):
        """Scatter-form (rasterised ellipsoid) backprojection, volume [Vz][Vy][Vx]."""
        import torch

        vx, vy, vz = info.voxel_res
        if out is None:
            out = torch.empty((vz, vy, vx), dtype=torch.float32, device=cube.device)
        check(self._lib.fbp_splat_backproject(self._h, byref(info), _ptr(cube, _cube_elems(info), name="cube"),
                                              _dtype_code(cube), layout,
                                              _ptr(laser_xyz, 3 * info.num_laser_targets, _f32(), "laser_xyz"),
                                              max_bins, grid[0], grid[1], _ptr(out, _voxels(info), _f32(), "out"),
                                              self._stream(stream)))
        return out

    def backproject_confocal_slab(self, info: ReconInfo, cube, laser_xyz, z_begin: int, z_end: int, out=None,
                                  layout=_lib.FBP_LAYOUT_TIME_INNER, stream=None):
        """Depth slices [z_begin, z_end) of the confocal volume: [z_end - z_begin][Vy][Vx]."""
        import torch

        vx, vy, _ = info.voxel_res
        if out is None:
            out = torch.empty((z_end - z_begin, vy, vx), dtype=torch.float32, device=cube.device)
        nz = max(0, min(int(z_end), int(info.voxel_res[2])) - int(z_begin))
        check(self._lib.fbp_backproject_confocal_slab(self._h, byref(info), _ptr(cube, _cube_elems(info), name="cube"),
                                                      _dtype_code(cube), layout,
                                                      _ptr(laser_xyz, 3 * info.num_laser_targets, _f32(), "laser_xyz"),
                                                      z_begin, z_end, _ptr(out, nz * vx * vy, _f32(), "out"),
                                                      self._stream(stream)))
        return out

    def backproject_exhaustive(self, info: ReconInfo, cube, laser_xyz, sensor_xyz, out=None, stream=None):
        import torch

        vx, vy, vz = info.voxel_res
        if out is None:
            out = torch.empty((vz, vy, vx), dtype=torch.float32, device=cube.device)
        check(self._lib.fbp_backproject_exhaustive(self._h, byref(info), _ptr(cube, _cube_elems(info, True), name="cube"),
                                                   _dtype_code(cube),
                                                   _ptr(laser_xyz, 3 * info.num_laser_targets, _f32(), "laser_xyz"),
                                                   _ptr(sensor_xyz, 3 * info.num_sensor_targets, _f32(), "sensor_xyz"),
                                                   _ptr(out, _voxels(info), _f32(), "out"), self._stream(stream)))
        return out

    def backproject_depths(self, info: ReconInfo, cube, laser_xyz, depths, sensor_xyz=None, out=None,
                           layout=_lib.FBP_LAYOUT_TIME_INNER, stream=None):
        import torch

        L = info.num_laser_targets
        D = int(depths.numel())
        if out is None:
            out = torch.empty((L, D), dtype=torch.float32, device=cube.device)
        import torch

        exhaustive = info.capture_system == _lib.FBP_EXHAUSTIVE
        check(self._lib.fbp_backproject_depths(self._h, byref(info),
                                               _ptr(cube, _cube_elems(info, exhaustive), name="cube"),
                                               _dtype_code(cube), layout,
                                               _ptr(laser_xyz, 3 * L, _f32(), "laser_xyz"),
                                               _ptr(sensor_xyz, 3 * info.num_sensor_targets if exhaustive else 0,
                                                    _f32(), "sensor_xyz"),
                                               _ptr(depths, D, torch.float64, "depths"), D,
                                               _ptr(out, L * D, _f32(), "out"), self._stream(stream)))
        return out

    def transient_images(self, data, width: int, height: int, num_planes: int, pixel_stride: int,
                         plane_stride: int, size=None, normalize: bool = False, out=None, stream=None):
        """RGBA8 images [planes][out_h][out_w][4] (TransientImage::save per
        plane); pixel idx of plane p is data[p*plane_stride + idx*pixel_stride];
        size = (out_w, out_h), default the plane's own size."""
        import torch

        ow, oh = size if size is not None else (width, height)
        if out is None:
            out = torch.empty((num_planes, oh, ow, 4), dtype=torch.uint8, device=data.device)
        check(self._lib.fbp_transient_images(self._h, _ptr(data, _plane_span(width, height, num_planes, pixel_stride,
                                                                              plane_stride), _f32(), "data"),
                                             width, height, num_planes, pixel_stride, plane_stride, ow, oh,
                                             int(normalize), _ptr(out, num_planes * oh * ow * 4, torch.uint8, "out"),
                                             self._stream(stream)))
        return out

    def depth_plane_images(self, activation, width: int, height: int, size=None, normalize: bool = False,
                           out=None, stream=None):
        """The images of every depth plane of an [width*height][D] activation."""
        D = int(activation.shape[-1])
        return self.transient_images(activation, width, height, D, D, 1, size, normalize, out, stream)

    def save_transient_images(self, data, width: int, height: int, num_planes: int, pixel_stride: int,
                              plane_stride: int, prefix: str, size=None, normalize: bool = False, stream=None):
        """Writes "<prefix>transient_<p>.png" for every plane."""
        ow, oh = size if size is not None else (width, height)
        span = _plane_span(width, height, num_planes, pixel_stride, plane_stride)
        check(self._lib.fbp_save_transient_images(self._h, _ptr(data, span, _f32(), "data"), width, height,
                                                  num_planes, pixel_stride,
                                                  plane_stride, ow, oh, int(normalize), prefix.encode(),
                                                  self._stream(stream)))

    def save_depth_planes(self, activation, width: int, height: int, prefix: str, size=None, normalize: bool = False,
                          stream=None):
        D = int(activation.shape[-1])
        self.save_transient_images(activation, width, height, D, D, 1, prefix, size, normalize, stream)

    def debug_confocal_bins(self, info: ReconInfo, laser_xyz, voxel_idx, stream=None):
        import torch

        out = torch.empty((voxel_idx.numel(), info.num_laser_targets), dtype=torch.int32, device=laser_xyz.device)
        check(self._lib.fbp_debug_confocal_bins(self._h, byref(info), _ptr(laser_xyz), _ptr(voxel_idx),
                                                voxel_idx.numel(), _ptr(out), self._stream(stream)))
        return out

    def debug_confocal_paths(self, info: ReconInfo, laser_xyz, voxel_idx, stream=None):
        """(paths [n][L] float32, (rcp_dt, half voxel diagonal)) in the gathers' FP32 arithmetic."""
        import torch

        out = torch.empty((voxel_idx.numel(), info.num_laser_targets), dtype=torch.float32, device=laser_xyz.device)
        consts = torch.empty(2, dtype=torch.float32, device=laser_xyz.device)
        check(self._lib.fbp_debug_confocal_paths(self._h, byref(info), _ptr(laser_xyz), _ptr(voxel_idx),
                                                 voxel_idx.numel(), _ptr(out), _ptr(consts), self._stream(stream)))
        c = consts.cpu()
        return out, (float(c[0]), float(c[1]))

    def debug_exhaustive_bins(self, info: ReconInfo, laser_xyz, sensor_xyz, voxel_idx, stream=None):
        import torch

        out = torch.empty((voxel_idx.numel(), info.num_laser_targets, info.num_sensor_targets), dtype=torch.int32,
                          device=laser_xyz.device)
        check(self._lib.fbp_debug_exhaustive_bins(self._h, byref(info), _ptr(laser_xyz), _ptr(sensor_xyz),
                                                  _ptr(voxel_idx), voxel_idx.numel(), _ptr(out),
                                                  self._stream(stream)))
        return out

    # --------------------------------------------------------- post-processing
    def postfilter(self, kind: int, vol, kernel_size: int = 5, sigma: float = 1.0, out=None, stream=None):
        import torch

        vz, vy, vx = vol.shape
        if out is None:
            out = torch.empty_like(vol)
        check(self._lib.fbp_postfilter(self._h, kind, kernel_size, sigma, _ptr(vol, 0, _f32(), "vol"),
                                       _ptr(out, vol.numel(), _f32(), "out"), vx, vy, vz,
                                       self._stream(stream)))
        return out

    def normalize_(self, v, stream=None):
        check(self._lib.fbp_normalize_minmax(self._h, _ptr(v, 0, _f32(), "v"), v.numel(), self._stream(stream)))
        return v

    def filter_h_(self, data, delta_t: float, wl_mean: float | None = None, wl_sigma: float = 0.0,
                  border: int = _lib.FBP_BORDER_ZERO, stream=None):
        """In-place temporal filter of data[num_series, T] (float32)."""
        n, T = data.shape[0] if data.dim() > 1 else 1, data.shape[-1]
        n = data.numel() // T
        wl = delta_t * 10.0 if wl_mean is None else wl_mean
        check(self._lib.fbp_filter_h(self._h, _ptr(data, 0, _f32(), "data"), n, T, delta_t, wl, wl_sigma, border,
                                     self._stream(stream)))
        return data

    # -------------------------------------------------------------------- MIS
    def mis_backproject(self, info: ReconInfo, cube, laser_xyz, proposal: int, samples: int, seed: int = 0,
                        noise=None, tile_cluster_cdf=None, cluster_side: int = 0, scan_side: int = 0, out=None,
                        layout=_lib.FBP_LAYOUT_TIME_INNER, cv_side: int = 0, stream=None):
        import torch

        vx, vy, vz = info.voxel_res
        if out is None:
            out = torch.empty((vz, vy, vx), dtype=torch.float32, device=cube.device)
        prm = MisParams(proposal, samples, seed, _ptr(noise, 0, _f32(), "noise"),
                        0 if noise is None else noise.numel(), _ptr(tile_cluster_cdf, 0, _f32(), "tile_cluster_cdf"),
                        cluster_side, scan_side, cv_side)
        check(self._lib.fbp_mis_backproject(self._h, byref(info), _ptr(cube, _cube_elems(info), name="cube"),
                                            _dtype_code(cube), layout,
                                            _ptr(laser_xyz, 3 * info.num_laser_targets, _f32(), "laser_xyz"),
                                            byref(prm), _ptr(out, _voxels(info), _f32(), "out"), self._stream(stream)))
        return out

    def mis_reference_tables(self, info: ReconInfo, cube, layout=_lib.FBP_LAYOUT_TIME_INNER, stream=None):
        L = info.num_laser_targets
        cdf = np.empty(L, np.float32)
        alias = np.empty(L, np.uint32)
        prob = np.empty(L, np.float32)
        check(self._lib.fbp_mis_reference_tables(self._h, byref(info), _ptr(cube), _dtype_code(cube), layout,
                                                 c_void_p(cdf.ctypes.data), c_void_p(alias.ctypes.data),
                                                 c_void_p(prob.ctypes.data), self._stream(stream)))
        return cdf, alias, prob

    # ------------------------------------------------------------------- LCT
    def lct(self, data, width: float, bin_length: float, snr: float = 0.8, diffuse: bool = True,
            grid_mode: int = _lib.FBP_LCT_GRID_REFERENCE, layout: int = _lib.FBP_LAYOUT_TIME_MAJOR, out=None,
            stream=None, output: int = _lib.FBP_LCT_OUTPUT_CLAMPED_REAL):
        """Confocal LCT.  data: [M][N][N] (time-major) or [N][N][M] (time-inner), float32.
        python/lct_2.py's variant: grid_mode=FBP_LCT_GRID_DEPTH, output=FBP_LCT_OUTPUT_MAGNITUDE."""
        import torch

        if layout == _lib.FBP_LAYOUT_TIME_MAJOR:
            M, N, _ = data.shape
        else:
            N, _, M = data.shape
        if out is None:
            out = torch.empty((M, N, N), dtype=torch.float32, device=data.device)
        prm = LctParams(width, bin_length, snr, int(diffuse), grid_mode, output)
        check(self._lib.fbp_lct(self._h, _ptr(data, M * N * N, _f32(), "data"), layout, N, M, byref(prm),
                                _ptr(out, M * N * N, _f32(), "out"), self._stream(stream)))
        return out

    # -------------------------------------------------------- learned proposal
    def mlp_tile_count(self, info: ReconInfo) -> int:
        n = ctypes.c_uint32()
        check(self._lib.fbp_mlp_tile_count(byref(info), byref(n)))
        return int(n.value)

    def mlp_features(self, info: ReconInfo, cube, laser_xyz, cluster_side: int, scan_side: int, tiles=None,
                     out=None, layout=_lib.FBP_LAYOUT_TIME_INNER, stream=None):
        """Feature rows [ntiles][G][FBP_MLP_FEATURES] of the listed tiles (int32 tensor) or of every tile."""
        import torch

        cpr = -(-scan_side // cluster_side)
        G = cpr * cpr
        nt = self.mlp_tile_count(info) if tiles is None else tiles.numel()
        if out is None:
            out = torch.empty((nt, G, _lib.FBP_MLP_FEATURES), dtype=torch.float32, device=cube.device)
        check(self._lib.fbp_mlp_features(self._h, byref(info), _ptr(cube), _dtype_code(cube), layout, _ptr(laser_xyz),
                                         cluster_side, scan_side, _ptr(tiles), 0 if tiles is None else nt, _ptr(out),
                                         self._stream(stream)))
        return out

    def mlp_labels(self, info: ReconInfo, cube, laser_xyz, cluster_side: int, scan_side: int, tiles, out=None,
                   layout=_lib.FBP_LAYOUT_TIME_INNER, stream=None):
        import torch

        cpr = -(-scan_side // cluster_side)
        G = cpr * cpr
        if out is None:
            out = torch.empty((tiles.numel(), G), dtype=torch.float32, device=cube.device)
        check(self._lib.fbp_mlp_labels(self._h, byref(info), _ptr(cube), _dtype_code(cube), layout, _ptr(laser_xyz),
                                       cluster_side, scan_side, _ptr(tiles), tiles.numel(), _ptr(out),
                                       self._stream(stream)))
        return out

    # ------------------------------------------------------------- end to end
    def reconstruct_shape_host(self, info: ReconInfo, cube: np.ndarray, laser_xyz: np.ndarray,
                               sensor_xyz: np.ndarray | None = None, use_fourier_filter: bool = True,
                               postfilter: int = _lib.FBP_FILTER_NONE, kernel_size: int = 5, sigma: float = 1.0,
                               normalize: bool = True, out: np.ndarray | None = None, stream=None) -> np.ndarray:
        vx, vy, vz = info.voxel_res
        if out is None:
            out = np.empty((vz, vy, vx), dtype=np.float32)
        params = ShapeParams(int(use_fourier_filter), postfilter, kernel_size, sigma, int(normalize))
        cube = np.ascontiguousarray(cube)
        laser_xyz = np.ascontiguousarray(laser_xyz, dtype=np.float32)
        sens = None if sensor_xyz is None else np.ascontiguousarray(sensor_xyz, dtype=np.float32)
        check(self._lib.fbp_reconstruct_shape_host(
            self._h, byref(info), c_void_p(cube.ctypes.data), _np_dtype_code(cube), c_void_p(laser_xyz.ctypes.data),
            c_void_p(0 if sens is None else sens.ctypes.data), byref(params), c_void_p(out.ctypes.data),
            self._stream(stream)))
        return out


class Batch:
    """Many confocal captures reconstructed together (fbp_batch_*).

    ``captures`` is a list of (info, cube, laser_xyz, volume, layout) with
    CUDA tensors; they are referenced, not copied, and must outlive the batch.
    Every ``run`` re-reads each cube and overwrites each volume.
    """

    def __init__(self, ctx: Context, captures):
        self._lib = ctx._lib
        self._ctx = ctx
        self._keep = []
        descs = (CaptureDesc * len(captures))()
        for i, (info, cube, laser_xyz, volume, layout) in enumerate(captures):
            d = descs[i]
            d.info = info
            d.cube = _ptr(cube).value
            d.dtype = _dtype_code(cube)
            d.layout = layout
            d.laser_xyz = _ptr(laser_xyz).value
            d.volume = _ptr(volume).value
            self._keep.append((cube, laser_xyz, volume))
        h = c_void_p()
        check(self._lib.fbp_batch_create(ctx._h, len(captures), descs, byref(h)))
        self._h = h

    def run(self, use_graph: bool = False, stream=None) -> None:
        check(self._lib.fbp_batch_run(self._h, int(use_graph), Context._stream(stream)))

    def autotune(self, stream=None) -> int:
        chosen = ctypes.c_int(-1)
        check(self._lib.fbp_batch_autotune(self._h, Context._stream(stream), byref(chosen)))
        return chosen.value

    def set_config(self, config: int, stream=None) -> None:
        check(self._lib.fbp_batch_set_config(self._h, config, Context._stream(stream)))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.fbp_batch_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass


class Mlp:
    """The learned MIS proposal network (fbp_mlp_*), parameters on the device."""

    def __init__(self, ctx: Context, seed: int = 0):
        self._lib = ctx._lib
        self._ctx = ctx
        h = c_void_p()
        check(self._lib.fbp_mlp_create(ctx._h, seed, byref(h)))
        self._h = h
        self.num_params = int(self._lib.fbp_mlp_num_params())

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        check(self._lib.fbp_mlp_get_params(self._h, out.ctypes.data_as(ctypes.POINTER(c_float)), self.num_params))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params
        check(self._lib.fbp_mlp_set_params(self._h, p.ctypes.data_as(ctypes.POINTER(c_float)), self.num_params))

    def forward(self, features, logits=True, defensive: float = 0.0, cdf=False, stream=None):
        """(logits [ntiles][G] or None, inclusive CDF [ntiles][G] or None)."""
        import torch

        nt, G = features.shape[0], features.shape[1]
        lo = torch.empty((nt, G), dtype=torch.float32, device=features.device) if logits else None
        cd = torch.empty((nt, G), dtype=torch.float32, device=features.device) if cdf else None
        check(self._lib.fbp_mlp_forward(self._ctx._h, self._h, _ptr(features), nt, G, _ptr(lo), defensive, _ptr(cd),
                                        Context._stream(stream)))
        return lo, cd

    def gradients(self, features, labels, idx, stream=None):
        """Gradient of the mean cross-entropy over rows idx, then the loss."""
        import torch

        out = torch.empty(self.num_params + 1, dtype=torch.float32, device=features.device)
        check(self._lib.fbp_mlp_gradients(self._ctx._h, self._h, _ptr(features), _ptr(labels), _ptr(idx), idx.numel(),
                                          features.shape[1], _ptr(out), Context._stream(stream)))
        return out

    def train_step(self, features, labels, idx, lr: float, loss=None, stream=None):
        check(self._lib.fbp_mlp_train_step(self._ctx._h, self._h, _ptr(features), _ptr(labels), _ptr(idx),
                                           idx.numel(), features.shape[1], lr, _ptr(loss), Context._stream(stream)))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.fbp_mlp_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass


def mis_tile_grid(info: ReconInfo):
    t = (ctypes.c_uint32 * 3)()
    check(load().fbp_mis_tile_grid(byref(info), t))
    return tuple(t)


def log_weights(size: int, sigma: float) -> np.ndarray:
    w = np.empty(size ** 3, dtype=np.float32)
    check(load().fbp_log_weights(size, sigma, w.ctypes.data_as(ctypes.POINTER(c_float))))
    return w


def linear_space(lo: float, hi: float, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    check(load().fbp_linear_space(lo, hi, n, out.ctypes.data_as(ctypes.POINTER(c_double))))
    return out


def write_png(path: str, rgba: np.ndarray) -> None:
    """PNG file of an RGBA8 host image [h][w][4] (rows top first)."""
    a = np.ascontiguousarray(rgba, dtype=np.uint8)
    if a.ndim != 3 or a.shape[2] != 4:
        raise ValueError("write_png: expected an [h][w][4] uint8 image")
    check(load().fbp_write_png(str(path).encode(), a.ctypes.data_as(c_void_p), a.shape[1], a.shape[0]))


def depth_image_size(side: int, exhaustive: bool = False) -> tuple[int, int]:
    """Output size of the depth-plane images: side * (256 // side) below 256
    for confocal captures (Laser.cu:420-422), 4 * side for exhaustive ones
    (Laser.cu:473)."""
    s = side * 4 if exhaustive else side * (256 // side if side < 256 else 1)
    return (s, s)
