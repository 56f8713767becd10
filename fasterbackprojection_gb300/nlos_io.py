"""Reader and writer of the reference's ".nlos" capture cache and the raw
".cube" volume.

.nlos (NLosData::saveBinaryFile / loadBinaryFile, FasterBackprojection/
NLosData.cpp:320-405) is a sequence of raw fields in the MSVC x64 layout,
little endian:

    cameraPosition      3 x f32
    laserPosition       3 x f32
    temporalResolution  u32
    deltaT              f32
    t0                  f32
    isConfocal          u8
    hiddenGeometry      32 bytes: AABB object = 8-byte vtable pointer
                        (meaningless on disk), max (3 x f32), min (3 x f32)
    numDims             u64, then numDims x u64
    numCamera           u64, positions numCamera x 3 x f32,
                        normals numCamera x 3 x f32, cameraGridSize 2 x f32
    numLaser            u64, positions, normals, laserGridSize 2 x f32
    numValues           u64, then numValues x f32 (the transient data)

.cube (Laser::saveReconstructedAABB, Laser.cu:518-524): raw f32 values of the
[Vz][Vy][Vx] volume, no header.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np


@dataclass
class NLosCapture:
    data: np.ndarray  # float32, flat, time innermost
    dims: list
    camera_grid_positions: np.ndarray  # [S][3]
    camera_grid_normals: np.ndarray
    camera_position: tuple = (0.0, 0.0, 0.0)
    camera_grid_size: tuple = (2.0, 2.0)
    laser_grid_positions: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    laser_grid_normals: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    laser_position: tuple = (0.0, 0.0, 0.0)
    laser_grid_size: tuple = (2.0, 2.0)
    hidden_min: tuple = (-1.0, -1.5, -1.0)
    hidden_max: tuple = (1.0, 0.0, 1.0)
    temporal_resolution: int = 0
    delta_t: float = 0.0
    t0: float = 0.0
    is_confocal: bool = True


def write_nlos(path, c: NLosCapture) -> None:
    out = bytearray()
    out += struct.pack("<3f", *c.camera_position)
    out += struct.pack("<3f", *c.laser_position)
    out += struct.pack("<I", int(c.temporal_resolution))
    out += struct.pack("<f", float(c.delta_t))
    out += struct.pack("<f", float(c.t0))
    out += struct.pack("<B", 1 if c.is_confocal else 0)
    out += b"\0" * 8 + struct.pack("<3f", *c.hidden_max) + struct.pack("<3f", *c.hidden_min) + b"\0" * 0
    out += struct.pack("<Q", len(c.dims))
    for d in c.dims:
        out += struct.pack("<Q", int(d))
    for pos, nrm, size in ((c.camera_grid_positions, c.camera_grid_normals, c.camera_grid_size),
                           (c.laser_grid_positions, c.laser_grid_normals, c.laser_grid_size)):
        pos = np.ascontiguousarray(pos, dtype="<f4").reshape(-1, 3)
        nrm = np.ascontiguousarray(nrm, dtype="<f4").reshape(-1, 3)
        if pos.shape != nrm.shape:
            raise ValueError("positions and normals differ in length")
        out += struct.pack("<Q", pos.shape[0]) + pos.tobytes() + nrm.tobytes() + struct.pack("<2f", *size)
    data = np.ascontiguousarray(c.data, dtype="<f4").ravel()
    out += struct.pack("<Q", data.size) + data.tobytes()
    Path(path).write_bytes(bytes(out))


def read_nlos(path) -> NLosCapture:
    b = Path(path).read_bytes()
    off = 0

    def take(fmt):
        nonlocal off
        n = struct.calcsize(fmt)
        if off + n > len(b):
            raise ValueError(f"truncated .nlos file: {path}")
        v = struct.unpack_from(fmt, b, off)
        off += n
        return v

    def take_array(count, comps):
        nonlocal off
        n = count * comps * 4
        if off + n > len(b):
            raise ValueError(f"truncated .nlos file: {path}")
        a = np.frombuffer(b, dtype="<f4", count=count * comps, offset=off).reshape(count, comps).copy()
        off += n
        return a

    cam_pos = take("<3f")
    las_pos = take("<3f")
    (tres,) = take("<I")
    (dt,) = take("<f")
    (t0,) = take("<f")
    (conf,) = take("<B")
    take("<8x")
    hmax = take("<3f")
    hmin = take("<3f")
    (nd,) = take("<Q")
    if nd > 16:
        raise ValueError("corrupt .nlos header (dimension count)")
    dims = list(take(f"<{nd}Q")) if nd else []
    grids = []
    for _ in range(2):
        (n,) = take("<Q")
        if n > (1 << 32):
            raise ValueError("corrupt .nlos header (grid size)")
        pos = take_array(n, 3)
        nrm = take_array(n, 3)
        size = take("<2f")
        grids.append((pos, nrm, size))
    (nv,) = take("<Q")
    if off + 4 * nv > len(b):
        raise ValueError(f"truncated .nlos file: {path}")
    data = np.frombuffer(b, dtype="<f4", count=nv, offset=off).copy()
    if dims and int(np.prod(dims)) != nv:
        raise ValueError(".nlos dims do not match the data size")
    return NLosCapture(data=data, dims=dims, camera_grid_positions=grids[0][0], camera_grid_normals=grids[0][1],
                       camera_position=cam_pos, camera_grid_size=grids[0][2], laser_grid_positions=grids[1][0],
                       laser_grid_normals=grids[1][1], laser_position=las_pos, laser_grid_size=grids[1][2],
                       hidden_min=hmin, hidden_max=hmax, temporal_resolution=tres, delta_t=dt, t0=t0,
                       is_confocal=bool(conf))


def write_cube(path, vol: np.ndarray) -> None:
    Path(path).write_bytes(np.ascontiguousarray(vol, dtype="<f4").tobytes())


def read_cube(path, shape) -> np.ndarray:
    return np.fromfile(path, dtype="<f4").reshape(shape)


# ------------------------------------------------------------ HDF5 captures

_HDF5_FIELDS = ("cameraGridPositions", "cameraGridNormals", "cameraPosition", "laserGridNormals",
                "laserGridPositions", "laserPosition", "t", "t0", "deltaT", "isConfocal", "data")


def _grid(raw) -> np.ndarray:
    """NLosData::setUp(vector<vec3>&, raw[3][W][H]) (NLosData.cpp:205-222):
    entry x * W + y holds (raw[0][x][y], raw[1][x][y], raw[2][x][y]).  The
    reference indexes with W for both axes, so only square grids are
    well-defined there; other shapes are refused."""
    a = np.asarray(raw, dtype=np.float64)
    if a.ndim != 3 or a.shape[0] != 3:
        raise ValueError(f"grid dataset must be 3 x W x H, got {a.shape}")
    if a.shape[1] != a.shape[2]:
        raise ValueError(f"non-square grid {a.shape[1]} x {a.shape[2]}: the reference's indexing is undefined")
    return np.ascontiguousarray(a.astype(np.float32).reshape(3, -1).T)


def _vec(raw, n: int, name: str) -> tuple:
    a = np.asarray(raw, dtype=np.float64).ravel()
    if a.size != n:
        raise ValueError(f"{name}: expected {n} values, got {a.size}")  # NLosData.cpp:191-203
    return tuple(float(np.float32(v)) for v in a)


def _sum_bounces(raw: np.ndarray, bounce_axis: int) -> np.ndarray:
    """data += float(raw) over the bounces in order, in float32
    (NLosData.cpp:233-242, 256-265, 289-305)."""
    acc = np.zeros(np.delete(raw.shape, bounce_axis), dtype=np.float32)
    for b in range(raw.shape[bounce_axis]):
        acc = (acc + np.take(raw, b, axis=bounce_axis).astype(np.float32)).astype(np.float32)
    return acc


def from_datasets(ds) -> NLosCapture:
    """The capture NLosData builds from an HDF5 file (NLosData.cpp:28-123,
    186-308), given its datasets as arrays (a dict, an h5py File, ...):
    grids flattened x * W + y, positions and sizes to float32, t0 read as an
    integer, the hidden box from hiddenVolumePosition +- hiddenVolumeSize / 2
    in float32 (a scalar size means (s, 0.1, s)), and the transient data with
    its bounces summed, time innermost: confocal [1][T][B][R][C] or
    [T][B][R][C] -> [R][C][T], exhaustive [1][T][B][lR][lC][cR][cC] ->
    [lR][lC][cR][cC][T]."""
    missing = [k for k in _HDF5_FIELDS if k not in ds]
    if missing:
        raise ValueError("NLosData: Missing required datasets in the file: " + ", ".join(missing))
    f32 = np.float32
    pos = np.asarray(ds["hiddenVolumePosition"], dtype=np.float64).ravel()
    size = np.asarray(ds["hiddenVolumeSize"], dtype=np.float64)
    size = np.array([size.item(), 0.1, size.item()]) if size.ndim == 0 or size.size == 1 else size.ravel()
    hmin = tuple(float(f32(pos[k]) - f32(size[k]) / f32(2.0)) for k in range(3))
    hmax = tuple(float(f32(pos[k]) + f32(size[k]) / f32(2.0)) for k in range(3))
    confocal = bool(int(np.asarray(ds["isConfocal"]).item()))
    raw = np.asarray(ds["data"])
    if confocal:
        if raw.ndim == 5:
            if raw.shape[0] != 1:
                raise ValueError("NLosData: one channel expected")
            raw = raw[0]
        if raw.ndim != 4:
            raise ValueError("NLosData: Invalid dimensions for confocal data.")
        T, _, R, C = raw.shape
        data = np.transpose(_sum_bounces(raw, 1), (1, 2, 0))  # [T][R][C] -> [R][C][T]
        dims = [R, C, T]
    else:
        if raw.ndim != 7 or raw.shape[0] != 1:
            raise ValueError("NLosData: exhaustive data must be [1][T][B][lR][lC][cR][cC]")
        _, T, _, lR, lC, cR, cC = raw.shape
        data = np.transpose(_sum_bounces(raw[0], 1), (1, 2, 3, 4, 0))
        dims = [lR, lC, cR, cC, T]
    return NLosCapture(
        data=np.ascontiguousarray(data, dtype=np.float32).ravel(), dims=dims,
        camera_grid_positions=_grid(ds["cameraGridPositions"]), camera_grid_normals=_grid(ds["cameraGridNormals"]),
        camera_position=_vec(ds["cameraPosition"], 3, "cameraPosition"),
        camera_grid_size=_vec(ds["cameraGridSize"], 2, "cameraGridSize"),
        laser_grid_positions=_grid(ds["laserGridPositions"]), laser_grid_normals=_grid(ds["laserGridNormals"]),
        laser_position=_vec(ds["laserPosition"], 3, "laserPosition"),
        laser_grid_size=_vec(ds["laserGridSize"], 2, "laserGridSize"),
        hidden_min=hmin, hidden_max=hmax, temporal_resolution=int(np.asarray(ds["t"]).item()),
        delta_t=float(f32(np.asarray(ds["deltaT"], dtype=np.float64).item())),
        t0=float(int(np.asarray(ds["t0"]).item())), is_confocal=confocal)


def read_hdf5(path) -> NLosCapture:
    """An HDF5 capture through h5py (when installed) and from_datasets."""
    try:
        import h5py
    except ImportError as e:  # pragma: no cover - depends on the environment
        raise ImportError("reading HDF5 captures needs h5py; convert once to .nlos elsewhere") from e
    with h5py.File(path, "r") as f:
        return from_datasets({k: f[k][()] for k in f.keys()})
