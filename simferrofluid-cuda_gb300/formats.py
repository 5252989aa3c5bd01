"""Readers and writers of the reference's on-disk formats, so that a GPU pipeline can resume from a reference run's
checkpoint and its outputs can be compared with the reference's.  All are raw little-endian records written with
IO::Write (core/Common.h:70-91: a value's bytes, or a contiguous range's bytes with no length prefix).

* checkpoint ``<frame>.sav`` (demo/Driver.cpp:95-101, Simulation::Save core/Simulation.cpp:118-125):
  velocity face arrays x, y, z (float64, face-grid layout, SGridData::Save core/SGridData.h:35), level set (float64,
  cell layout, GridData::Save core/GridData.h:47), m_InitVolume, m_CumulVolError, m_VolError (float64),
  m_MaxMeshSize (int32), then the timing table of StopWatch::Save (core/StopWatch.cpp:18-26): size_t count, the
  names NUL-terminated, uint32 counts, float64 mean and max seconds.
* ``contour.out`` (SurfaceMesh::Export core/SurfaceMesh.cpp:10-20): uint32 vertex count, float32 xyz positions,
  float32 xyz normals, uint32 index count, uint32 triangle indices.
* ``curv.out`` / ``mag_pressure.out`` (core/Simulation.cpp:86-115): as contour.out with one float32 value per
  vertex (mean curvature / magnetic pressure) after the normals.
* ``collider.out`` (core/Simulation.cpp:67-84): uint32 count, float32 xyz positions, float32 xyz normals.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Checkpoint:
    velocity: list            # three float64 face arrays (grid.face_shape(a))
    level_set: np.ndarray     # float64 cell array (grid.shape)
    init_volume: float = 0.0
    cumul_vol_error: float = 0.0
    vol_error: float = 0.0
    max_mesh_size: int = 0
    timings: list = field(default_factory=list)  # (name, count, mean_s, max_s)


def write_checkpoint(path, grid, ck: Checkpoint):
    with open(path, "wb") as f:
        for a in range(3):
            v = np.ascontiguousarray(ck.velocity[a], dtype="<f8")
            if v.size != int(np.prod(grid.face_shape(a))):
                raise ValueError(f"velocity[{a}] has {v.size} values, the grid has {int(np.prod(grid.face_shape(a)))}")
            f.write(v.tobytes())
        phi = np.ascontiguousarray(ck.level_set, dtype="<f8")
        if phi.size != int(np.prod(grid.shape)):
            raise ValueError("level set size does not match the grid")
        f.write(phi.tobytes())
        f.write(struct.pack("<dddi", ck.init_volume, ck.cumul_vol_error, ck.vol_error, ck.max_mesh_size))
        f.write(struct.pack("<Q", len(ck.timings)))
        for name, *_ in ck.timings:
            f.write(name.encode() + b"\0")
        f.write(np.array([t[1] for t in ck.timings], dtype="<u4").tobytes())
        f.write(np.array([t[2] for t in ck.timings], dtype="<f8").tobytes())
        f.write(np.array([t[3] for t in ck.timings], dtype="<f8").tobytes())


def read_checkpoint(path, grid) -> Checkpoint:
    data = open(path, "rb").read()
    off = 0

    def take(n, dtype):
        nonlocal off
        size = np.dtype(dtype).itemsize * n
        if off + size > len(data):
            raise ValueError(f"{path}: truncated checkpoint")
        a = np.frombuffer(data, dtype=dtype, count=n, offset=off)
        off += size
        return a

    vel = [take(int(np.prod(grid.face_shape(a))), "<f8").reshape(grid.face_shape(a)).copy() for a in range(3)]
    phi = take(int(np.prod(grid.shape)), "<f8").reshape(grid.shape).copy()
    init_volume, cumul, vol_error = take(3, "<f8")
    max_mesh = int(take(1, "<i4")[0])
    timings = []
    if off < len(data):
        n = int(take(1, "<u8")[0])
        names = []
        for _ in range(n):
            end = data.index(b"\0", off)
            names.append(data[off:end].decode())
            off = end + 1
        counts, means, maxes = take(n, "<u4"), take(n, "<f8"), take(n, "<f8")
        timings = [(names[i], int(counts[i]), float(means[i]), float(maxes[i])) for i in range(n)]
    return Checkpoint(vel, phi, float(init_volume), float(cumul), float(vol_error), max_mesh, timings)


@dataclass
class MeshRecord:
    positions: np.ndarray           # (n, 3) float32
    normals: np.ndarray             # (n, 3) float32
    values: np.ndarray | None       # (n,) float32 (curvature or magnetic pressure) or None
    indices: np.ndarray             # (m,) uint32


def write_mesh(path, positions, normals, indices, values=None):
    """contour.out (values None), curv.out or mag_pressure.out (values per vertex)."""
    pos = np.ascontiguousarray(positions, dtype="<f4").reshape(-1, 3)
    nrm = np.ascontiguousarray(normals, dtype="<f4").reshape(-1, 3)
    idx = np.ascontiguousarray(indices, dtype="<u4").ravel()
    if nrm.shape != pos.shape:
        raise ValueError("positions and normals differ in length")
    with open(path, "wb") as f:
        f.write(struct.pack("<I", pos.shape[0]))
        f.write(pos.tobytes())
        f.write(nrm.tobytes())
        if values is not None:
            vals = np.ascontiguousarray(values, dtype="<f4").ravel()
            if vals.size != pos.shape[0]:
                raise ValueError("one value per vertex expected")
            f.write(vals.tobytes())
        f.write(struct.pack("<I", idx.size))
        f.write(idx.tobytes())


def read_mesh(path, with_values: bool) -> MeshRecord:
    data = open(path, "rb").read()
    n = struct.unpack_from("<I", data, 0)[0]
    off = 4
    pos = np.frombuffer(data, "<f4", 3 * n, off).reshape(n, 3).copy()
    off += 12 * n
    nrm = np.frombuffer(data, "<f4", 3 * n, off).reshape(n, 3).copy()
    off += 12 * n
    vals = None
    if with_values:
        vals = np.frombuffer(data, "<f4", n, off).copy()
        off += 4 * n
    m = struct.unpack_from("<I", data, off)[0]
    off += 4
    idx = np.frombuffer(data, "<u4", m, off).copy()
    if off + 4 * m != len(data):
        raise ValueError(f"{path}: {len(data) - off - 4 * m} trailing bytes")
    return MeshRecord(pos, nrm, vals, idx)


def write_collider(path, positions, normals):
    pos = np.ascontiguousarray(positions, dtype="<f4").reshape(-1, 3)
    nrm = np.ascontiguousarray(normals, dtype="<f4").reshape(-1, 3)
    with open(path, "wb") as f:
        f.write(struct.pack("<I", pos.shape[0]))
        f.write(pos.tobytes())
        f.write(nrm.tobytes())


def read_collider(path):
    data = open(path, "rb").read()
    n = struct.unpack_from("<I", data, 0)[0]
    pos = np.frombuffer(data, "<f4", 3 * n, 4).reshape(n, 3).copy()
    nrm = np.frombuffer(data, "<f4", 3 * n, 4 + 12 * n).reshape(n, 3).copy()
    return pos, nrm
