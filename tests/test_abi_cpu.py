"""C-ABI library checks that need no GPU: it loads, exports every symbol the
header declares, and its host-only functions match the oracle."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_functions():
    text = (ROOT / "include" / "fbp.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fbp_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built):
    from fasterbackprojection_gb300 import _lib

    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    names = header_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # The Python binding declares a signature for each of them.
    assert sorted(_lib.SIGNATURES) == names


def test_exports_are_plain_c_symbols(built):
    from fasterbackprojection_gb300 import _lib

    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (fbp_[a-z0-9_]+)$", out, flags=re.M))
    assert set(header_functions()) <= exported


def test_version_and_last_error(built):
    from fasterbackprojection_gb300 import _lib

    lib = _lib.load()
    assert b"sm_103a" in lib.fbp_version()
    assert lib.fbp_last_error() == b"" or isinstance(lib.fbp_last_error(), bytes)


def test_log_weights_match_oracle_bitwise(built):
    from fasterbackprojection_gb300.api import log_weights
    from oracle import cpu

    for k, s in [(5, 1.0), (3, 0.7), (7, 1.5), (9, 2.0)]:
        np.testing.assert_array_equal(log_weights(k, s), cpu.log_weights(k, s))


def test_linear_space_matches_reference_formula(built):
    from fasterbackprojection_gb300.api import linear_space

    got = linear_space(0.4, 0.6, 200)
    step = (0.6 - 0.4) / 200
    np.testing.assert_array_equal(got, 0.4 + step * np.arange(200))


def test_invalid_arguments_are_reported_not_raised(built):
    from fasterbackprojection_gb300 import _lib

    lib = _lib.load()
    assert lib.fbp_create(None, 0) == _lib.FBP_ERR_INVALID_ARG
    assert b"null" in lib.fbp_last_error()
    assert lib.fbp_linear_space(0.0, 1.0, 0, None) == _lib.FBP_ERR_INVALID_ARG
    w = (ctypes.c_float * 1)()
    assert lib.fbp_log_weights(0, 1.0, w) == _lib.FBP_ERR_INVALID_ARG


def test_create_without_gpu_fails_cleanly(built):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from fasterbackprojection_gb300 import _lib

    lib = _lib.load()
    h = ctypes.c_void_p()
    st = lib.fbp_create(ctypes.byref(h), 0)
    assert st in (_lib.FBP_ERR_CUDA, _lib.FBP_ERR_INVALID_ARG)
    assert lib.fbp_last_error() != b""


def test_product_never_imports_the_oracle():
    pkg = ROOT / "fasterbackprojection_gb300"
    for f in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cpp")) + list(pkg.rglob("*.hpp")):
        text = f.read_text()
        assert not re.search(r"^\s*(from|import)\s+oracle", text, flags=re.M), f
        assert "liboracle" not in text and "ref_kernels.cubin" not in text, f


def test_scene_generator_known_answer():
    from fasterbackprojection_gb300 import scenes

    w = scenes.wall_grid(4)
    assert w.shape == (16, 3) and w.dtype == np.float32
    np.testing.assert_allclose(w[0], [-0.75, 0, -0.75])
    np.testing.assert_allclose(w[1], [-0.25, 0, -0.75])  # l = iz * n + ix
    cap = scenes.confocal_points(4, 1024, 32e-12, n_points=1, seed=4, noise=False)
    pts, alb, _ = scenes.random_points(1, (0.4, 1.2), 4)
    r = np.linalg.norm(w.astype(np.float64) - pts[0], axis=1)
    b = np.rint(2 * r / cap.time_step).astype(int)
    for l in range(16):
        assert cap.cube[l, b[l]] == pytest.approx(alb[0] / r[l] ** 4, rel=1e-6)
        assert np.count_nonzero(cap.cube[l]) == 1


def test_bf16_bits_round_trip():
    from fasterbackprojection_gb300 import scenes

    a = np.array([0.0, 1.0, 3.0, 1e-3, 257.0, 65504.0], np.float32)
    back = scenes.from_bits_bf16(scenes.to_bits_bf16(a))
    np.testing.assert_allclose(back, a, rtol=2 ** -8)
    assert back[2] == 3.0 and back[4] == 256.0  # round to nearest even


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors have the C structs' sizes and field offsets."""
    from fasterbackprojection_gb300 import _lib

    structs = {
        "fbp_recon_info": _lib.ReconInfo,
        "fbp_lct_params": _lib.LctParams,
        "fbp_mis_params": _lib.MisParams,
        "fbp_shape_params": _lib.ShapeParams,
        "fbp_capture_desc": _lib.CaptureDesc,
    }
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "fbp.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        c, f, v = line.split()
        got[(c, f)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_device_pointer_checks_reject_host_and_short_tensors():
    """The Python layer hands kernels plain pointers: host memory, a wrong
    element type and (through the sizes each entry point needs) short
    buffers are refused before any launch."""
    import torch

    from fasterbackprojection_gb300.api import _plane_span, _ptr

    assert _ptr(None).value is None
    with pytest.raises(TypeError, match="CUDA tensor"):
        _ptr(torch.zeros(4), name="cube")
    with pytest.raises(TypeError, match="CUDA tensor"):
        _ptr(np.zeros(4, np.float32))

    class FakeCuda:  # stands in for a device tensor on a machine without one
        is_cuda = True
        dtype = torch.float32

        def __init__(self, n, contiguous=True):
            self.n, self.c = n, contiguous

        def is_contiguous(self):
            return self.c

        def numel(self):
            return self.n

        def data_ptr(self):
            return 4096

    assert _ptr(FakeCuda(12), 12, torch.float32).value == 4096
    with pytest.raises(ValueError, match="at least 13"):
        _ptr(FakeCuda(12), 13, name="out")
    with pytest.raises(ValueError, match="contiguous"):
        _ptr(FakeCuda(12, contiguous=False))
    with pytest.raises(TypeError, match="float64"):
        _ptr(FakeCuda(12), 0, torch.float64, "depths")
    # Plane p, pixel i at p * plane_stride + i * pixel_stride.
    assert _plane_span(16, 16, 200, 200, 1) == 256 * 200
    assert _plane_span(12, 40, 5, 1, 480) == 5 * 480
    assert _plane_span(0, 4, 4, 4, 1) == 0


def test_host_allocation_failure_is_a_status_not_an_abort(built, tmp_path):
    """No C++ exception crosses the C ABI: with the address space capped just
    above what the process uses, a 256 MB PNG encode must come back as
    FBP_ERR_OOM (an escaping std::bad_alloc would abort the process)."""
    import subprocess
    import sys

    resource = pytest.importorskip("resource")
    del resource
    code = f"""
import ctypes, resource, numpy as np
from fasterbackprojection_gb300 import _lib
lib = _lib.load()
img = np.zeros((8192, 8192, 4), np.uint8)
vm = [int(l.split()[1]) * 1024 for l in open('/proc/self/status') if l.startswith('VmSize')][0]
resource.setrlimit(resource.RLIMIT_AS, (vm + (96 << 20), resource.getrlimit(resource.RLIMIT_AS)[1]))
st = lib.fbp_write_png({str(tmp_path / 'big.png')!r}.encode(), img.ctypes.data_as(ctypes.c_void_p), 8192, 8192)
print(st, lib.fbp_last_error().decode())
"""
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=str(ROOT), timeout=120)
    assert out.returncode == 0, out.stderr[-2000:]
    st, msg = out.stdout.split(" ", 1)
    assert int(st) == 2 and "fbp_write_png" in msg  # FBP_ERR_OOM
