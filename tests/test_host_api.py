"""The reference-shaped C++ host classes (NLosData, Laser, LCT,
PostprocessingFilters) and the .nlos / .cube formats."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from tests.conftest import rel_l2

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def driver(built, tmp_path_factory):
    from fasterbackprojection_gb300 import _build

    exe = tmp_path_factory.mktemp("drv") / "host_api_test"
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", str(ROOT / "include"), "-I", str(_build.CPP),
                    "-I", "/usr/local/cuda/include", str(ROOT / "tests" / "cpp" / "host_api_test.cpp"), "-o", str(exe),
                    "-L", str(_build.LIBDIR), "-lfbp_host", "-lfbp", f"-Wl,-rpath,{_build.LIBDIR}",
                    "-L/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"], check=True)
    return exe


def _capture(n=8, T=256, seed=3):
    from fasterbackprojection_gb300 import nlos_io, scenes

    cap = scenes.confocal_points(n, T, 32e-12, n_points=30, seed=seed)
    L = n * n
    normals = np.tile(np.array([[0.0, -1.0, 0.0]], np.float32), (L, 1))
    c = nlos_io.NLosCapture(data=cap.cube.ravel(), dims=[n, n, T], camera_grid_positions=cap.laser_xyz,
                            camera_grid_normals=normals, laser_grid_positions=cap.laser_xyz,
                            laser_grid_normals=normals, camera_position=(0.0, -0.2, 0.1),
                            laser_position=(0.1, -0.2, 0.0), hidden_min=(-1.0, -2.0, -1.0),
                            hidden_max=(1.0, 0.0, 1.0), temporal_resolution=T, delta_t=cap.time_step, t0=0.0,
                            is_confocal=True)
    return cap, c


def test_nlos_python_round_trip(tmp_path):
    from fasterbackprojection_gb300 import nlos_io

    _, c = _capture()
    p = tmp_path / "a.nlos"
    nlos_io.write_nlos(p, c)
    r = nlos_io.read_nlos(p)
    np.testing.assert_array_equal(r.data, c.data)
    assert r.dims == c.dims and r.temporal_resolution == c.temporal_resolution and r.is_confocal
    np.testing.assert_allclose(r.hidden_min, c.hidden_min)
    # 12+12+4+4+4+1+32 header bytes, dims, two grids, data.
    L = 64
    assert p.stat().st_size == 69 + 8 + 3 * 8 + 2 * (8 + L * 24 + 8) + 8 + 4 * c.data.size


def test_nlos_cpp_round_trip_is_byte_identical(driver, tmp_path):
    from fasterbackprojection_gb300 import nlos_io

    _, c = _capture()
    a, b = tmp_path / "a.nlos", tmp_path / "b.nlos"
    nlos_io.write_nlos(a, c)
    out = subprocess.run([str(driver), "roundtrip", str(a), str(b)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert a.read_bytes() == b.read_bytes()


def test_nlos_corrupt_and_truncated_files_are_rejected(driver, tmp_path):
    from fasterbackprojection_gb300 import nlos_io

    _, c = _capture()
    a = tmp_path / "a.nlos"
    nlos_io.write_nlos(a, c)
    raw = a.read_bytes()
    (tmp_path / "t.nlos").write_bytes(raw[: len(raw) // 2])
    with pytest.raises(ValueError):
        nlos_io.read_nlos(tmp_path / "t.nlos")
    assert subprocess.run([str(driver), "roundtrip", str(tmp_path / "t.nlos"), str(tmp_path / "x")]).returncode != 0
    bad = bytearray(raw)
    bad[69:77] = (1 << 40).to_bytes(8, "little")  # absurd dimension count
    (tmp_path / "c.nlos").write_bytes(bytes(bad))
    with pytest.raises(ValueError):
        nlos_io.read_nlos(tmp_path / "c.nlos")
    assert subprocess.run([str(driver), "roundtrip", str(tmp_path / "c.nlos"), str(tmp_path / "y")]).returncode != 0


@pytest.mark.gpu
@pytest.mark.parametrize("filt,fourier", [(0, 0), (2, 1), (1, 0), (3, 1)])
def test_laser_reconstruct_shape_matches_c_abi(driver, ctx, tmp_path, filt, fourier):
    from fasterbackprojection_gb300 import make_info, nlos_io

    cap, c = _capture()
    nlos_io.write_nlos(tmp_path / "cap.nlos", c)
    V = 16
    out = subprocess.run([str(driver), "shape", str(tmp_path / "cap.nlos"), str(tmp_path), str(V), str(filt),
                          str(fourier), "1"], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    vol = nlos_io.read_cube(tmp_path / "aabb.cube", (V, V, V))
    # Same geometry through the C ABI (NLosData::toGpu: voxel size = size / res, bounces on).
    info = make_info(num_laser_targets=64, num_time_bins=256, time_step=cap.time_step, voxel_res=(V, V, V),
                     hidden_min=(-1.0, -2.0, -1.0), voxel_size=(2.0 / V, 2.0 / V, 2.0 / V),
                     discard_first_last_bounces=0, laser_position=(0.1, -0.2, 0.0),
                     sensor_position=(0.0, -0.2, 0.1))
    want = ctx.reconstruct_shape_host(info, cap.cube, cap.laser_xyz, use_fourier_filter=bool(fourier),
                                      postfilter=filt)
    np.testing.assert_array_equal(vol, want)


@pytest.mark.gpu
def test_laser_depth_mode_writes_activations(driver, ctx, tmp_path):
    from fasterbackprojection_gb300 import nlos_io

    _, c = _capture()
    nlos_io.write_nlos(tmp_path / "cap.nlos", c)
    out = subprocess.run([str(driver), "shape", str(tmp_path / "cap.nlos"), str(tmp_path), "8", "0", "0", "0"],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    act = np.fromfile(tmp_path / "depths.raw", dtype=np.float32).reshape(64, 20)
    assert act.min() >= 0.0 and act.max() == pytest.approx(1.0)
    # Laser.cu:409-424: one PNG per depth, an 8 x 8 scan enlarged to 256 x 256.
    from oracle import numpy_ref
    from tests.test_images_cpu import _decode_png

    for d in (0, 7, 19):
        img = _decode_png((tmp_path / f"transient_{d}.png").read_bytes())
        np.testing.assert_array_equal(img, numpy_ref.transient_image(act.ravel(), 8, 8, (256, 256), stride=20,
                                                                     offset=d))


@pytest.mark.gpu
def test_nlos_save_images_writes_normalised_slices(driver, ctx, tmp_path):
    """NLosData::saveImages (NLosData.cpp:161-180): one normalised [cols][T] image per scan row."""
    from fasterbackprojection_gb300 import nlos_io
    from oracle import numpy_ref
    from tests.test_images_cpu import _decode_png

    cap, c = _capture(n=6, T=64)
    nlos_io.write_nlos(tmp_path / "cap.nlos", c)
    out = subprocess.run([str(driver), "images", str(tmp_path / "cap.nlos"), str(tmp_path / "img")],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    data = cap.cube.reshape(6, 6 * 64)
    for r in range(6):
        img = _decode_png((tmp_path / "img" / f"transient_{r}.png").read_bytes())
        np.testing.assert_array_equal(img, numpy_ref.transient_image(data[r], 6, 64, (6, 64), normalize=True))


@pytest.mark.gpu
def test_lct_class_matches_c_abi(driver, ctx, cuda, tmp_path):
    import torch
    from fasterbackprojection_gb300 import FBP_LAYOUT_TIME_INNER, nlos_io

    cap, c = _capture(n=16, T=128, seed=5)
    nlos_io.write_nlos(tmp_path / "cap.nlos", c)
    out = subprocess.run([str(driver), "lct", str(tmp_path / "cap.nlos"), str(tmp_path / "lct.cube")],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    vol = nlos_io.read_cube(tmp_path / "lct.cube", (128, 16, 16))
    want = ctx.lct(torch.from_numpy(cap.cube.reshape(16, 16, 128)).to(cuda), 1.0, cap.time_step,
                   layout=FBP_LAYOUT_TIME_INNER).cpu().numpy()
    assert rel_l2(vol, want) < 1e-6


@pytest.mark.gpu
def test_transient_image_class_matches_the_reference_conversion(driver, ctx, tmp_path):
    """TransientImage::save, both overloads (TransientImage.cpp:31-64)."""
    from oracle import numpy_ref
    from tests.test_images_cpu import _decode_png

    out = subprocess.run([str(driver), "timage", str(tmp_path)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    f = np.array([((i * 37) % 101) / np.float32(97.0) for i in range(1 + 3 * 35)], np.float32)
    np.testing.assert_array_equal(_decode_png((tmp_path / "float.png").read_bytes()),
                                  numpy_ref.transient_image(f, 7, 5, (13, 9), stride=3, offset=1))
    u = np.array([(i * 40, 300 - i, i, 7) for i in range(12)], np.uint32).reshape(3, 4, 4)
    want = np.minimum(u, 255).astype(np.uint8)[::-1].copy()
    want[..., 3] = 255
    np.testing.assert_array_equal(_decode_png((tmp_path / "uvec4.png").read_bytes()), want)


@pytest.mark.gpu
def test_laser_mis_entry_point_runs_the_reference_mode(driver, ctx, cuda, tmp_path):
    """Laser::reconstructAABBConfocalMIS (Laser.cu:526-611) = FBP_MIS_REFERENCE
    with L/4 samples and the default noise buffer, on the capture's data."""
    import torch
    from fasterbackprojection_gb300 import FBP_MIS_REFERENCE, make_info, nlos_io

    cap, c = _capture()
    nlos_io.write_nlos(tmp_path / "cap.nlos", c)
    out = subprocess.run([str(driver), "mis", str(tmp_path / "cap.nlos"), str(tmp_path / "mis.raw")],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    got = np.fromfile(tmp_path / "mis.raw", dtype=np.float32).reshape(8, 8, 8)
    info = make_info(num_laser_targets=64, num_time_bins=256, time_step=cap.time_step, voxel_res=(8, 8, 8),
                     hidden_min=(-1.0, -2.0, -1.0), voxel_size=(0.25, 0.25, 0.25), discard_first_last_bounces=0,
                     laser_position=(0.1, -0.2, 0.0), sensor_position=(0.0, -0.2, 0.1))
    want = ctx.mis_backproject(info, torch.from_numpy(cap.cube).to(cuda), torch.from_numpy(cap.laser_xyz).to(cuda),
                               FBP_MIS_REFERENCE, 0).cpu().numpy()
    assert float(np.abs(want).max()) > 0
    np.testing.assert_array_equal(got, want)

