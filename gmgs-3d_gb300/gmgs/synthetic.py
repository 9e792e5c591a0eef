"""Seeded synthetic voxel models and boundary conditions.

The reference's demos voxelise triangle meshes (src/common/CreateVoxilizedModel.m)
and load picked boundary nodes from data/demo_BC_*.dat (src/Demo.m:16-64).  The
workloads here stand in for them: a solid nelx x nely x nelz block with
spherical voids, all solid nodes of the z = 0 face fixed, and a total force of
-1 in z spread evenly over the solid nodes of the original top face.
Node ids are the reference's compact 1-based numbering
(src/common/DiscretizeDesignDomain.m:76-93), computed on the padded grid.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Workload:
    name: str
    nelx: int
    nely: int
    nelz: int
    voids: int
    seed: int
    num_levels: int = 0           # 0 -> the reference's level rule
    omega: float = 0.6
    tol: float = 1.0e-3
    rho_range: tuple | None = None
    penal: float = 3.0


# The five workloads of the benchmark description (resolution nelx x nely x nelz).
WORKLOADS = {
    "block42_fp64": Workload("block42_fp64", 42, 37, 64, 20, 1001, num_levels=4),
    "block169_fp64_vs_mixed": Workload("block169_fp64_vs_mixed", 169, 147, 256, 40, 1002),
    "block84_adjoint": Workload("block84_adjoint", 84, 73, 128, 0, 1003, rho_range=(0.2, 1.0)),
    "block337_mixed_L6": Workload("block337_mixed_L6", 337, 294, 512, 120, 1004, num_levels=6),
    "block428_mixed_adjoint_L7": Workload("block428_mixed_adjoint_L7", 428, 373, 650, 200, 1005,
                                          num_levels=7, rho_range=(0.3, 1.0)),
}


def _keep_anchored(solid: np.ndarray) -> np.ndarray:
    """Drop solid voxels that are not face-connected to the z = 0 layer.

    Pieces cut off by voids (or hinged on one node or edge) would make the
    stiffness matrix singular.
    """
    try:
        from scipy import ndimage
    except ImportError:       # pragma: no cover - scipy is present on both machines
        return solid
    lab, n = ndimage.label(solid)
    if n <= 1:
        return solid
    anchored = np.unique(lab[:, :, 0])
    anchored = anchored[anchored > 0]
    return np.isin(lab, anchored) & solid


def sphere_voids(nelx: int, nely: int, nelz: int, voids: int, seed: int) -> np.ndarray:
    """(nely, nelx, nelz) int32 occupancy, 1 = solid, MATLAB (y, x, z) layout.

    Sphere centres are uniform in [0,nelx)x[0,nely)x[0,nelz) (voxel units) and
    radii uniform in [3, 8]; a voxel is void when its centre lies inside a sphere.
    """
    rng = np.random.default_rng(seed)
    centres = rng.uniform([0.0, 0.0, 0.0], [nelx, nely, nelz], size=(voids, 3))
    radii = rng.uniform(3.0, 8.0, size=voids)
    solid = np.ones((nely, nelx, nelz), dtype=bool)
    for (cx, cy, cz), r in zip(centres, radii):
        x0, x1 = max(0, int(np.floor(cx - r))), min(nelx, int(np.ceil(cx + r)) + 1)
        y0, y1 = max(0, int(np.floor(cy - r))), min(nely, int(np.ceil(cy + r)) + 1)
        z0, z1 = max(0, int(np.floor(cz - r))), min(nelz, int(np.ceil(cz + r)) + 1)
        if x0 >= x1 or y0 >= y1 or z0 >= z1:
            continue
        ys = (np.arange(y0, y1) + 0.5 - cy) ** 2
        xs = (np.arange(x0, x1) + 0.5 - cx) ** 2
        zs = (np.arange(z0, z1) + 0.5 - cz) ** 2
        inside = ys[:, None, None] + xs[None, :, None] + zs[None, None, :] < r * r
        solid[y0:y1, x0:x1, z0:z1] &= ~inside
    solid = _keep_anchored(solid)
    return solid.astype(np.int32)


def padded_shape(nely: int, nelx: int, nelz: int, num_levels: int) -> tuple:
    f = 2 ** (num_levels - 1)
    return tuple(-(-n // f) * f for n in (nely, nelx, nelz))


def solid_node_mask(vox_padded: np.ndarray) -> np.ndarray:
    """(ny+1, nx+1, nz+1) bool: nodes touched by a solid element."""
    s = vox_padded == 1
    ny, nx, nz = s.shape
    m = np.zeros((ny + 1, nx + 1, nz + 1), dtype=bool)
    for dy in (0, 1):
        for dx in (0, 1):
            for dz in (0, 1):
                m[dy:dy + ny, dx:dx + nx, dz:dz + nz] |= s
    return m


def boundary_conditions(vox: np.ndarray, num_levels: int):
    """(fixed node ids, loads (n x 4: id fx fy fz)) in the compact 1-based numbering.

    Fixed: every solid node with z-index 0.  Load: -1 in z in total, split
    evenly over the solid nodes with z-index nelz (the unpadded top face).
    """
    nely, nelx, nelz = vox.shape
    ny, nx, nz = padded_shape(nely, nelx, nelz, num_levels)
    pad = np.zeros((ny, nx, nz), dtype=np.int32)
    pad[:nely, :nelx, :nelz] = vox
    mask = solid_node_mask(pad)
    flat = mask.ravel(order="F")
    compact = np.cumsum(flat)                      # 1-based compact id at solid nodes
    lin = np.arange(flat.size).reshape(mask.shape, order="F")
    fixed = compact[lin[:, :, 0][mask[:, :, 0]]]
    top = lin[:, :, nelz][mask[:, :, nelz]]
    top_ids = compact[top]
    loads = np.zeros((len(top_ids), 4))
    loads[:, 0] = top_ids
    loads[:, 3] = -1.0 / max(1, len(top_ids))
    return np.sort(fixed).astype(np.int32), loads


def level_count(nely: int, nelx: int, nelz: int, num_levels: int, ctrl: int = 10000) -> int:
    """numLevels by the reference's rule (DiscretizeDesignDomain.m:33-41) unless given."""
    if num_levels:
        return num_levels
    num = nelx * nely * nelz
    k = 0
    while num >= ctrl:
        k += 1
        num = nelx / 2 ** k * nely / 2 ** k * nelz / 2 ** k
    return k + 1


def density(n_solid: int, rho_range, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed + 7919)
    return rng.uniform(rho_range[0], rho_range[1], size=n_solid)


def make(workload: Workload | str, scale: float = 1.0):
    """(voxels, fixed ids, loads, num_levels, rho or None) for a workload.

    `scale` < 1 shrinks the resolution (test sizes); the voids keep their radii.
    """
    w = WORKLOADS[workload] if isinstance(workload, str) else workload
    nelx = max(2, int(round(w.nelx * scale)))
    nely = max(2, int(round(w.nely * scale)))
    nelz = max(2, int(round(w.nelz * scale)))
    vox = sphere_voids(nelx, nely, nelz, w.voids, w.seed)
    L = level_count(nely, nelx, nelz, w.num_levels)
    fixed, loads = boundary_conditions(vox, L)
    rho = None
    if w.rho_range is not None:
        rho = density(int(vox.sum()), w.rho_range, w.seed)
    # the reference's voxelizedVolume_ is a column-major (y, x, z) array
    return np.asfortranarray(vox), fixed, loads, L, rho


# ---------------------------------------------------------------------------
# closed triangle meshes for the voxeliser (synthetic stand-ins for the
# reference's kitten and parts models)
# ---------------------------------------------------------------------------
def blob_mesh(n_lat: int = 24, n_lon: int = 48, seed: int = 0, amp: float = 0.25):
    """(vertices, faces) of a closed genus-0 surface: a UV sphere whose radius
    varies with a few seeded low-order harmonics.  Outward-oriented faces."""
    rng = np.random.default_rng(seed)
    coef = rng.normal(size=(4, 4)) * amp / 4
    phase = rng.uniform(0, 2 * np.pi, size=(4, 4))
    th = np.linspace(0, np.pi, n_lat + 1)[1:-1]
    ph = np.linspace(0, 2 * np.pi, n_lon, endpoint=False)
    T, P = np.meshgrid(th, ph, indexing="ij")

    def radius(t, p):
        r = np.ones_like(t)
        for i in range(4):
            for j in range(4):
                r = r + coef[i, j] * np.cos((i + 1) * t) * np.cos(j * p + phase[i, j])
        return r

    R = radius(T, P)
    ring = np.stack([R * np.sin(T) * np.cos(P), R * np.sin(T) * np.sin(P), R * np.cos(T)], axis=-1).reshape(-1, 3)
    north = np.array([[0.0, 0.0, float(radius(np.zeros(1), np.zeros(1))[0])]])
    south = np.array([[0.0, 0.0, -float(radius(np.full(1, np.pi), np.zeros(1))[0])]])
    verts = np.concatenate([north, ring, south]) * np.array([1.3, 1.0, 1.6]) + 3.0
    nn, ns = 0, 1 + ring.shape[0]
    vid = lambda i, j: 1 + i * n_lon + (j % n_lon)
    faces = []
    for j in range(n_lon):
        faces.append((nn, vid(0, j), vid(0, j + 1)))
        faces.append((ns, vid(n_lat - 2, j + 1), vid(n_lat - 2, j)))
    for i in range(n_lat - 2):
        for j in range(n_lon):
            a, b, c, d = vid(i, j), vid(i, j + 1), vid(i + 1, j), vid(i + 1, j + 1)
            faces.append((a, c, b))
            faces.append((b, c, d))
    return verts, np.asarray(faces, dtype=np.int32)


def torus_mesh(R: float = 2.0, r: float = 0.7, nu: int = 48, nv: int = 24, seed: int = 0):
    """(vertices, faces) of a closed torus (genus 1) with seeded vertex jitter."""
    rng = np.random.default_rng(seed)
    u = np.linspace(0, 2 * np.pi, nu, endpoint=False)
    v = np.linspace(0, 2 * np.pi, nv, endpoint=False)
    U, V = np.meshgrid(u, v, indexing="ij")
    rr = r * (1 + 0.05 * rng.standard_normal(U.shape))
    verts = np.stack([(R + rr * np.cos(V)) * np.cos(U), (R + rr * np.cos(V)) * np.sin(U), rr * np.sin(V)],
                     axis=-1).reshape(-1, 3) + np.array([3.0, 3.0, 1.0])
    vid = lambda i, j: (i % nu) * nv + (j % nv)
    faces = []
    for i in range(nu):
        for j in range(nv):
            a, b, c, d = vid(i, j), vid(i + 1, j), vid(i, j + 1), vid(i + 1, j + 1)
            faces.append((a, b, d))
            faces.append((a, d, c))
    return verts, np.asarray(faces, dtype=np.int32)
