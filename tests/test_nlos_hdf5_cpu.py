"""nlos_io.from_datasets: the layout NLosData builds from an HDF5 capture
(NLosData.cpp:28-123, 186-308), against loop restatements of its setUp
functions, on synthetic datasets (h5py is not needed)."""
import numpy as np
import pytest

f32 = np.float32


def _loop_grid(raw):
    """NLosData.cpp:205-222: data[x * width + y] with width = raw[0].size()."""
    W, H = len(raw[0]), len(raw[0][0])
    out = np.zeros((W * H, 3), np.float32)
    for x in range(W):
        for y in range(H):
            out[x * W + y] = [f32(raw[0][x][y]), f32(raw[1][x][y]), f32(raw[2][x][y])]
    return out


def _loop_confocal(raw4):
    """NLosData.cpp:249-268: data[y*C*T + x*T + t] += float(raw[t][b][y][x])."""
    T, B, R, C = raw4.shape
    out = np.zeros(R * C * T, np.float32)
    for t in range(T):
        for x in range(C):
            for y in range(R):
                for b in range(B):
                    i = y * C * T + x * T + t
                    out[i] = f32(out[i] + f32(raw4[t, b, y, x]))
    return out, [R, C, T]


def _loop_exhaustive(raw7):
    """NLosData.cpp:270-308."""
    _, T, B, lR, lC, cR, cC = raw7.shape
    out = np.zeros(lR * lC * cR * cC * T, np.float32)
    for t in range(T):
        for b in range(B):
            for cx in range(cC):
                for cy in range(cR):
                    for lx in range(lC):
                        for ly in range(lR):
                            i = ly * lC * cR * cC * T + lx * cR * cC * T + cy * cC * T + cx * T + t
                            out[i] = f32(out[i] + f32(raw7[0, t, b, ly, lx, cy, cx]))
    return out, [lR, lC, cR, cC, T]


def _datasets(rng, data, confocal=True, size=(0.8, 0.6, 1.0), T=6):
    return {
        "cameraGridPositions": rng.normal(size=(3, 4, 4)), "cameraGridNormals": rng.normal(size=(3, 4, 4)),
        "cameraPosition": rng.normal(size=3), "cameraGridSize": np.array([2.0, 1.5]),
        "laserGridPositions": rng.normal(size=(3, 3, 3)), "laserGridNormals": rng.normal(size=(3, 3, 3)),
        "laserPosition": rng.normal(size=3), "laserGridSize": np.array([1.0, 1.0]),
        "t": np.array(T, dtype=np.uint32),  # its own dataset in the file
        "t0": np.array(-7.9), "deltaT": np.array(0.0012345678901),
        "hiddenVolumePosition": np.array([0.1, -0.7, 0.2]), "hiddenVolumeSize": np.asarray(size, dtype=np.float64),
        "isConfocal": np.array(1 if confocal else 0, dtype=np.uint32), "data": data,
    }


@pytest.mark.parametrize("five_d", [False, True])
def test_confocal_capture_matches_the_loader_loops(five_d):
    from fasterbackprojection_gb300 import nlos_io

    rng = np.random.default_rng(1)
    raw4 = rng.random((6, 3, 2, 5)) * 1e3  # [T][B][R][C], several bounces
    ds = _datasets(rng, raw4[None] if five_d else raw4)
    c = nlos_io.from_datasets(ds)
    want, dims = _loop_confocal(raw4)
    np.testing.assert_array_equal(c.data, want)
    assert c.dims == dims and c.is_confocal and c.temporal_resolution == 6
    np.testing.assert_array_equal(c.camera_grid_positions, _loop_grid(ds["cameraGridPositions"]))
    np.testing.assert_array_equal(c.laser_grid_normals, _loop_grid(ds["laserGridNormals"]))
    assert c.camera_position == tuple(float(f32(v)) for v in ds["cameraPosition"])
    assert c.camera_grid_size == (2.0, 1.5)
    assert c.t0 == -7.0  # read as an integer (truncated)
    assert c.delta_t == float(f32(0.0012345678901))
    pos, size = [f32(v) for v in (0.1, -0.7, 0.2)], [f32(v) for v in (0.8, 0.6, 1.0)]
    assert c.hidden_min == tuple(float(p - s / f32(2)) for p, s in zip(pos, size))
    assert c.hidden_max == tuple(float(p + s / f32(2)) for p, s in zip(pos, size))


def test_scalar_hidden_size_and_exhaustive_layout():
    from fasterbackprojection_gb300 import nlos_io

    rng = np.random.default_rng(2)
    raw7 = rng.random((1, 4, 2, 2, 3, 2, 2)) * 10
    c = nlos_io.from_datasets(_datasets(rng, raw7, confocal=False, size=0.5))
    want, dims = _loop_exhaustive(raw7)
    np.testing.assert_array_equal(c.data, want)
    assert c.dims == dims and not c.is_confocal
    # A scalar hiddenVolumeSize s means (s, 0.1, s) (NLosData.cpp:85-87).
    assert c.hidden_max[1] - c.hidden_min[1] == pytest.approx(0.1, rel=1e-6)
    assert c.hidden_max[0] - c.hidden_min[0] == pytest.approx(0.5, rel=1e-6)


def test_bad_datasets_are_refused(tmp_path):
    from fasterbackprojection_gb300 import nlos_io

    rng = np.random.default_rng(3)
    ds = _datasets(rng, rng.random((4, 1, 2, 2)))
    del ds["deltaT"]
    with pytest.raises(ValueError, match="deltaT"):
        nlos_io.from_datasets(ds)
    ds = _datasets(rng, rng.random((4, 2, 2)))
    with pytest.raises(ValueError, match="Invalid dimensions"):
        nlos_io.from_datasets(ds)
    ds = _datasets(rng, rng.random((4, 1, 2, 2)))
    ds["cameraGridPositions"] = rng.normal(size=(3, 4, 5))
    with pytest.raises(ValueError, match="non-square"):
        nlos_io.from_datasets(ds)
    # The result is an ordinary capture: it round-trips through the .nlos cache.
    c = nlos_io.from_datasets(_datasets(rng, rng.random((4, 1, 2, 2))))
    nlos_io.write_nlos(tmp_path / "a.nlos", c)
    r = nlos_io.read_nlos(tmp_path / "a.nlos")
    np.testing.assert_array_equal(r.data, c.data)
    assert r.dims == c.dims and r.t0 == c.t0


def test_read_hdf5_names_its_dependency(tmp_path):
    import importlib.util

    from fasterbackprojection_gb300 import nlos_io

    if importlib.util.find_spec("h5py") is not None:
        pytest.skip("h5py is installed here")
    with pytest.raises(ImportError, match="h5py"):
        nlos_io.read_hdf5(tmp_path / "capture.hdf5")
