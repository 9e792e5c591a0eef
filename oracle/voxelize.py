"""CPU restatement of the reference's mesh voxeliser (test infrastructure).

The oracle for the voxeliser row: reads a triangle mesh (.ply), sizes the
grid and voxelises it by ray parity exactly as the reference does, so the
occupancy (and from it the DOF counts the reference README publishes) can
be checked.  Nothing in the product imports this module.

Follows, in FP64 with the reference's evaluation order:
  src/common/ReadTriangularPolygonMesh_plyFormat.m:3-21  (ASCII .ply reader)
  src/common/AdaptData4Voxelize.m:3-18                    (grid size per axis)
  src/common/CreateVoxilizedModel.m:10-26                 (flip along y, int32)
  src/common/Voxelize.m:1-93                              (three ray directions, majority vote)
  src/common/Voxelize.m:95-331                            (ray casting along one axis)
The voxeliser in the reference is A. H. Aitkenhead's VOXELISE (2013, BSD),
vendored into Voxelize.m; its published algorithm is restated here.
"""
from __future__ import annotations

import numpy as np


class VoxelizeError(RuntimeError):
    pass


# ---------------------------------------------------------------- .ply input
def read_ply(path):
    """(nodeCoords (n,3) float64, faces (m,3) int 0-based) of an ASCII .ply
    whose header carries the element counts (ReadTriangularPolygonMesh_plyFormat.m:7-20)."""
    with open(path, "r") as f:
        tokens = f.read().split()
    i = tokens.index("end_header")
    header = tokens[:i]
    nv = int(header[header.index("vertex") + 1])
    nf = int(header[header.index("face") + 1])
    body = tokens[i + 1:]
    coords = np.array(body[:3 * nv], dtype=np.float64).reshape(nv, 3)
    fl = np.array(body[3 * nv:3 * nv + 4 * nf], dtype=np.int64).reshape(nf, 4)
    if np.any(fl[:, 0] != 3):
        raise VoxelizeError("only triangle faces are supported")
    return coords, fl[:, 1:]


def matlab_round(x):
    """MATLAB round: half away from zero."""
    x = np.asarray(x, dtype=np.float64)
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def adapt_for_voxelize(coords, faces, max_res):
    """(nx, ny, nz, meshXYZ (m,3,3)): AdaptData4Voxelize.m:5-18."""
    dims = coords.max(axis=0) - coords.min(axis=0)
    res = matlab_round(max_res * (dims / dims.max())).astype(np.int64)
    mesh = np.stack([coords[faces[:, 0]], coords[faces[:, 1]], coords[faces[:, 2]]], axis=2)
    return int(res[0]), int(res[1]), int(res[2]), mesh


def colon(a, d, b):
    """MATLAB's a:d:b for d > 0: n+1 points with the first half a + k d and the
    second half b' - (n-k) d, b' = a + n d, the symmetric evaluation MATLAB's
    colon operator uses, and a count that tolerates rounding in (b - a)/d."""
    q = (b - a) / d
    tol = 2.0 * np.finfo(float).eps * max(abs(a), abs(b)) / d
    n = int(np.floor(q + tol))
    if n < 0:
        return np.zeros(0)
    k = np.arange(n + 1, dtype=np.float64)
    c = a + n * d
    v = np.empty(n + 1)
    half = (n + 1) // 2
    v[:half] = a + k[:half] * d
    v[half:] = c - (n - k[half:]) * d
    return v


def _nearest_index(grid, value):
    idx = np.flatnonzero(np.abs(grid - value) == np.min(np.abs(grid - value)))
    return int(idx[0])


# ---------------------------------------------------------- one ray direction
def _voxelise_internal(gx, gy, gz, mesh):
    """Rays along the third axis through every (gx, gy) pixel (Voxelize.m:95-331).

    mesh: (m, 3, 3) facet vertex coordinates [facet, axis, vertex].
    Returns a bool array (len(gx), len(gy), len(gz)).
    """
    nx, ny, nz = len(gx), len(gy), len(gz)
    out = np.zeros((nx, ny, nz), dtype=bool)
    zmin = mesh[:, 2, :].min()
    zmax = mesh[:, 2, :].max()
    ixmin = _nearest_index(gx, mesh[:, 0, :].min())
    ixmax = _nearest_index(gx, mesh[:, 0, :].max())
    iymin = _nearest_index(gy, mesh[:, 1, :].min())
    iymax = _nearest_index(gy, mesh[:, 1, :].max())
    if ixmin > ixmax:
        ixmin, ixmax = ixmax, ixmin
    if iymin > iymax:
        iymin, iymax = iymax, iymin
    fmin = mesh.min(axis=2)
    fmax = mesh.max(axis=2)
    X1, X2, X3 = mesh[:, 0, 0], mesh[:, 0, 1], mesh[:, 0, 2]
    Y1, Y2, Y3 = mesh[:, 1, 0], mesh[:, 1, 1], mesh[:, 1, 2]
    Z1, Z2, Z3 = mesh[:, 2, 0], mesh[:, 2, 1], mesh[:, 2, 2]
    with np.errstate(divide="ignore", invalid="ignore"):
        # edge predictions that do not depend on the ray (Voxelize.m:222,228,234)
        Y1p = Y2 - ((Y2 - Y3) * (X2 - X1) / (X2 - X3))
        Y2p = Y3 - ((Y3 - Y1) * (X3 - X2) / (X3 - X1))
        Y3p = Y1 - ((Y1 - Y2) * (X1 - X3) / (X1 - X2))
        # plane coefficients (Voxelize.m:262-265)
        pA = Y1 * (Z2 - Z3) + Y2 * (Z3 - Z1) + Y3 * (Z1 - Z2)
        pB = Z1 * (X2 - X3) + Z2 * (X3 - X1) + Z3 * (X1 - X2)
        pC = X1 * (Y2 - Y3) + X2 * (Y3 - Y1) + X3 * (Y1 - Y2)
        pD = -X1 * (Y2 * Z3 - Y3 * Z2) - X2 * (Y3 * Z1 - Y1 * Z3) - X3 * (Y1 * Z2 - Y2 * Z1)
    pC = np.where(np.abs(pC) < 1e-14, 0.0, pC)
    corrections = []
    xs = np.arange(ixmin, ixmax + 1)
    for iy in range(iymin, iymax + 1):
        yv = gy[iy]
        cand_y = np.flatnonzero((fmin[:, 1] <= yv) & (fmax[:, 1] >= yv))
        if cand_y.size == 0:
            continue
        xv = gx[xs]                                              # rays of this row
        inx = (fmin[cand_y, 0][:, None] <= xv[None, :]) & (fmax[cand_y, 0][:, None] >= xv[None, :])
        if not inx.any():
            continue
        f = cand_y
        # rays through a facet vertex: the reference's vertex branch calls a
        # helper it does not define, so such a ray stops the voxelisation
        vhit = ((mesh[f, 0, 0][:, None] == xv) & (mesh[f, 1, 0][:, None] == yv)) | \
               ((mesh[f, 0, 1][:, None] == xv) & (mesh[f, 1, 1][:, None] == yv)) | \
               ((mesh[f, 0, 2][:, None] == xv) & (mesh[f, 1, 2][:, None] == yv))
        if np.any(vhit & inx):
            raise VoxelizeError("a ray crosses a mesh vertex exactly (Voxelize.m:176-203 is not executable)")
        with np.errstate(divide="ignore", invalid="ignore"):
            YR1 = Y2[f][:, None] - ((Y2[f] - Y3[f])[:, None] * (X2[f][:, None] - xv[None, :]) / (X2[f] - X3[f])[:, None])
            ok = ((Y1p[f][:, None] > Y1[f][:, None]) & (YR1 > yv)) | ((Y1p[f][:, None] < Y1[f][:, None]) & (YR1 < yv))
            YR2 = Y3[f][:, None] - ((Y3[f] - Y1[f])[:, None] * (X3[f][:, None] - xv[None, :]) / (X3[f] - X1[f])[:, None])
            ok &= ((Y2p[f][:, None] > Y2[f][:, None]) & (YR2 > yv)) | ((Y2p[f][:, None] < Y2[f][:, None]) & (YR2 < yv))
            YR3 = Y1[f][:, None] - ((Y1[f] - Y2[f])[:, None] * (X1[f][:, None] - xv[None, :]) / (X1[f] - X2[f])[:, None])
            ok &= ((Y3p[f][:, None] > Y3[f][:, None]) & (YR3 > yv)) | ((Y3p[f][:, None] < Y3[f][:, None]) & (YR3 < yv))
            ok &= inx
            zc = ((-pD[f])[:, None] - pA[f][:, None] * xv[None, :] - pB[f][:, None] * yv) / pC[f][:, None]
        for j in np.flatnonzero(ok.any(axis=0)):
            z = zc[ok[:, j], j]
            z = z[(z >= zmin - 1e-12) & (z <= zmax + 1e-12)]
            z = np.unique(matlab_round(z * 1e12) / 1e12)
            ix = int(xs[j])
            if z.size % 2 == 0:
                for k in range(z.size // 2):
                    out[ix, iy, (gz > z[2 * k]) & (gz < z[2 * k + 1])] = True
            elif z.size:
                corrections.append((ix, iy))
    # rays with an odd number of crossings: 8-neighbour vote, in the order found
    # (Voxelize.m:306-330); out-of-range neighbours count as empty
    for ix, iy in corrections:
        s = np.zeros(nz, dtype=np.int64)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                if dx == 0 and dy == 0:
                    continue
                jx, jy = ix + dx, iy + dy
                if 0 <= jx < nx and 0 <= jy < ny:
                    s += out[jx, jy, :]
        out[ix, iy, s >= 4] = True
    return out


def voxelize(nx, ny, nz, mesh):
    """Occupancy (len(gy), len(gx), len(gz)) bool of Voxelize.m:1-93 (before the
    flip of CreateVoxilizedModel.m)."""
    ax = []
    for d, n in enumerate((nx, ny, nz)):
        lo = mesh[:, d, :].min()
        hi = mesh[:, d, :].max()
        w = (hi - lo) / (n + 0.5)
        ax.append(colon(lo + w / 2, w, hi - w / 2))
    gx, gy, gz = ax
    vx = _voxelise_internal(gy, gz, gx, mesh[:, [1, 2, 0], :]).transpose(2, 0, 1)
    vy = _voxelise_internal(gz, gx, gy, mesh[:, [2, 0, 1], :]).transpose(1, 2, 0)
    vz = _voxelise_internal(gx, gy, gz, mesh)
    votes = vx.astype(np.int8) + vy + vz
    grid = votes >= 1.5
    return grid.transpose(1, 0, 2)


def create_voxelized_model(path, finest_resolution):
    """(voxelizedVolume int32 (ny, nx, nz), bounding box (2, 3), (nx, ny, nz)) of
    CreateVoxilizedModel(triFaceModelFile, finestResCtrl) (CreateVoxilizedModel.m:10-26)."""
    coords, faces = read_ply(path)
    return create_voxelized_model_from_arrays(coords, faces, finest_resolution)


def create_voxelized_model_from_arrays(coords, faces, finest_resolution):
    """create_voxelized_model for a mesh given as (vertices (n,3), faces (m,3) 0-based)."""
    coords = np.asarray(coords, dtype=np.float64)
    faces = np.asarray(faces)
    nx, ny, nz, mesh = adapt_for_voxelize(coords, faces, finest_resolution)
    vol = voxelize(nx, ny, nz, mesh)[::-1, :, :]
    bbox = np.stack([coords.min(axis=0), coords.max(axis=0)])
    return np.ascontiguousarray(vol.astype(np.int32)), bbox, (nx, ny, nz)
