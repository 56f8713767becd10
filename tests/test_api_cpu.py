"""The Python Context methods on the CPU: a stub library records the C calls,
fake device tensors stand in for CUDA memory.  Checks that every method
reaches its entry point with the sizes checked, and that short buffers are
refused before the call."""
from ctypes import c_void_p

import numpy as np
import pytest


class FakeCuda:
    """Enough of a contiguous CUDA tensor for the pointer checks."""

    is_cuda = True

    def __init__(self, shape, dtype=None):
        import torch

        self.shape = tuple(shape)
        self.dtype = dtype or torch.float32
        self.device = "cuda:0"

    def is_contiguous(self):
        return True

    def numel(self):
        return int(np.prod(self.shape)) if self.shape else 1

    def dim(self):
        return len(self.shape)

    def data_ptr(self):
        return 1 << 20


class StubLib:
    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def fn(*args):
            self.calls.append(name)
            return 0

        return fn


@pytest.fixture
def ctx():
    from fasterbackprojection_gb300.api import Context

    c = object.__new__(Context)
    c._lib = StubLib()
    c._h = c_void_p(1)
    c.device = 0
    c._stream = lambda stream=None: c_void_p(0)
    yield c
    c._h = None


def test_every_method_reaches_its_entry_point(ctx):
    import torch

    from fasterbackprojection_gb300 import FBP_EXHAUSTIVE, FBP_FILTER_LOG, FBP_MIS_REFERENCE, make_info

    L, S, T, V = 16, 9, 64, (4, 5, 6)
    nv = 4 * 5 * 6
    info = make_info(num_laser_targets=L, num_time_bins=T, time_step=0.01, voxel_res=V, hidden_min=(0, 0, 0),
                     voxel_size=(0.1, 0.1, 0.1))
    xinfo = make_info(num_laser_targets=L, num_sensor_targets=S, num_time_bins=T, time_step=0.01, voxel_res=V,
                      hidden_min=(0, 0, 0), voxel_size=(0.1, 0.1, 0.1), capture_system=FBP_EXHAUSTIVE)
    cube, lx, out = FakeCuda((L, T)), FakeCuda((L, 3)), FakeCuda((6, 5, 4))
    ctx.backproject_confocal(info, cube, lx, out=out)
    ctx.backproject_confocal_scatter(info, cube, lx, out=out)
    ctx.splat_backproject(info, cube, lx, out=out)
    ctx.backproject_confocal_slab(info, cube, lx, 2, 6, out=FakeCuda((4, 5, 4)))
    ctx.backproject_exhaustive(xinfo, FakeCuda((L, S, T)), lx, FakeCuda((S, 3)), out=out)
    ctx.backproject_depths(info, cube, lx, FakeCuda((7,), torch.float64), out=FakeCuda((L, 7)))
    ctx.transient_images(FakeCuda((L, 7)), 4, 4, 7, 7, 1, size=(8, 8), out=FakeCuda((7, 8, 8, 4), torch.uint8))
    ctx.save_transient_images(FakeCuda((L, 7)), 4, 4, 7, 7, 1, "x/")
    vol = FakeCuda((6, 5, 4))
    ctx.postfilter(FBP_FILTER_LOG, vol, out=FakeCuda((6, 5, 4)))
    ctx.normalize_(vol)
    ctx.filter_h_(FakeCuda((L, T)), 0.01)
    ctx.mis_backproject(info, cube, lx, FBP_MIS_REFERENCE, 0, noise=FakeCuda((nv,)), out=out)
    ctx.lct(FakeCuda((T, 4, 4)), 1.0, 0.01, out=FakeCuda((T, 4, 4)))
    assert ctx._lib.calls == [
        "fbp_backproject_confocal", "fbp_backproject_confocal_scatter", "fbp_splat_backproject",
        "fbp_backproject_confocal_slab", "fbp_backproject_exhaustive", "fbp_backproject_depths",
        "fbp_transient_images", "fbp_save_transient_images", "fbp_postfilter", "fbp_normalize_minmax",
        "fbp_filter_h", "fbp_mis_backproject", "fbp_lct"]


def test_short_or_host_buffers_never_reach_the_library(ctx):
    import torch

    from fasterbackprojection_gb300 import make_info

    L, T = 16, 64
    info = make_info(num_laser_targets=L, num_time_bins=T, time_step=0.01, voxel_res=(4, 5, 6), hidden_min=(0, 0, 0),
                     voxel_size=(0.1, 0.1, 0.1))
    cube, lx, out = FakeCuda((L, T)), FakeCuda((L, 3)), FakeCuda((6, 5, 4))
    with pytest.raises(ValueError, match="cube"):
        ctx.backproject_confocal(info, FakeCuda((L, T - 1)), lx, out=out)
    with pytest.raises(ValueError, match="laser_xyz"):
        ctx.backproject_confocal(info, cube, FakeCuda((L - 1, 3)), out=out)
    with pytest.raises(ValueError, match="out"):
        ctx.backproject_confocal(info, cube, lx, out=FakeCuda((6, 5, 3)))
    with pytest.raises(TypeError, match="out"):
        ctx.backproject_confocal(info, cube, lx, out=FakeCuda((6, 5, 4), torch.float16))
    with pytest.raises(TypeError, match="CUDA tensor"):
        ctx.backproject_confocal(info, torch.zeros((L, T)), lx, out=out)
    with pytest.raises(TypeError, match="depths"):
        ctx.backproject_depths(info, cube, lx, FakeCuda((7,)), out=FakeCuda((L, 7)))
    with pytest.raises(ValueError, match="data"):
        ctx.transient_images(FakeCuda((L, 6)), 4, 4, 7, 7, 1, out=FakeCuda((7, 4, 4, 4), torch.uint8))
    with pytest.raises(ValueError, match="out"):
        ctx.backproject_confocal_slab(info, cube, lx, 0, 6, out=FakeCuda((5, 5, 4)))
    assert ctx._lib.calls == []
