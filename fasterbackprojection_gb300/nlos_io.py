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
