"""Triangle-mesh input and voxelisation (CreateVoxilizedModel with a mesh file).

read_ply() parses the ASCII .ply files the reference reads
(src/common/ReadTriangularPolygonMesh_plyFormat.m:3-21); voxelize() runs the
GPU voxeliser behind gmgs_voxelize_mesh (src/common/CreateVoxilizedModel.m:10-26).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .solver import GMGSError


def read_ply(path):
    """(vertices (nv, 3) float64, faces (nf, 3) int32 0-based) of an ASCII
    triangle .ply with 'element vertex' and 'element face' header lines."""
    with open(path, "r") as f:
        tokens = f.read().split()
    try:
        end = tokens.index("end_header")
        head = tokens[:end]
        nv = int(head[head.index("vertex") + 1])
        nf = int(head[head.index("face") + 1])
    except ValueError as e:
        raise GMGSError(L.ERR_INVALID_ARGUMENT, f"{path}: not an ASCII .ply with vertex and face counts") from e
    body = tokens[end + 1:]
    v = np.array(body[:3 * nv], dtype=np.float64).reshape(nv, 3)
    fl = np.array(body[3 * nv:3 * nv + 4 * nf], dtype=np.int64).reshape(nf, 4)
    if np.any(fl[:, 0] != 3):
        raise GMGSError(L.ERR_INVALID_ARGUMENT, f"{path}: only triangle faces are supported")
    return v, np.ascontiguousarray(fl[:, 1:], dtype=np.int32)


def voxelize(vertices, faces, finest_resolution: int):
    """(occupancy (ny, nx, nz) int32 Fortran order, ele_size (x, y, z)).

    ele_size is the bounding-box extent per axis divided by the voxel count
    (DiscretizeDesignDomain.m:53-65; padding does not change it)."""
    lib = L.load()
    v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
    f = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
    dims = (C.c_int32 * 3)()
    pv = v.ctypes.data_as(C.POINTER(C.c_double))
    pf = f.ctypes.data_as(C.POINTER(C.c_int32))
    st = lib.gmgs_voxelize_mesh(pv, len(v), pf, len(f), int(finest_resolution), dims, None)
    if st != L.OK:
        raise GMGSError(st, lib.gmgs_last_error(None).decode())
    ny, nx, nz = dims[0], dims[1], dims[2]
    occ = np.zeros(ny * nx * nz, dtype=np.int32)
    st = lib.gmgs_voxelize_mesh(pv, len(v), pf, len(f), int(finest_resolution), dims,
                                occ.ctypes.data_as(C.POINTER(C.c_int32)))
    if st != L.OK:
        raise GMGSError(st, lib.gmgs_last_error(None).decode())
    ext = v.max(axis=0) - v.min(axis=0)
    return occ.reshape((ny, nx, nz), order="F"), ext / np.array([nx, ny, nz], dtype=np.float64)
