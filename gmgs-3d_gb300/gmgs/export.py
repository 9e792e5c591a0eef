"""Output formats of the reference (host-side text writers).

export_dataset_3dtsv: the ".carti" Cartesian-grid stress dataset of
    src/common/ExportDataset_3DTSV.m:11-41.
wrap_voxel_fea_model: the wrapped voxel FEA model text of
    src/common/WrapVoxelFEAmodel.m:7-25.
grid_maps: eleMapBack / nodMapBack, the reference's compact-to-grid maps
    (src/common/DiscretizeDesignDomain.m:68-86), 1-based linear indices into
    the padded element grid (ny, nx, nz) and node grid (ny+1, nx+1, nz+1),
    column-major.

Line formats follow the reference's fprintf calls, including its habit of
passing one string to a format with several %s: MATLAB prints the literal
text up to the first conversion that has no data left, so
fprintf(fid, '%s %s', 'DATASET CARTESIAN_GRID') writes "DATASET CARTESIAN_GRID ".
"""
from __future__ import annotations

import numpy as np


def grid_maps(occupancy):
    """(eleMapBack, nodMapBack) of a padded occupancy (ny, nx, nz); value 1 = solid."""
    vox = np.asarray(occupancy) == 1
    ny, nx, nz = vox.shape
    ele = np.flatnonzero(vox.ravel(order="F")) + 1
    node = np.zeros((ny + 1, nx + 1, nz + 1), dtype=bool)
    for dy in (0, 1):
        for dx in (0, 1):
            for dz in (0, 1):
                node[dy:dy + ny, dx:dx + nx, dz:dz + nz] |= vox
    nod = np.flatnonzero(node.ravel(order="F")) + 1
    return ele.astype(np.int64), nod.astype(np.int64)


def _loads_rows(loading, nod_map_back, offset):
    ld = np.asarray(loading, dtype=np.float64).reshape(-1, 4)
    ids = nod_map_back[ld[:, 0].astype(np.int64) - 1] - offset
    return "".join(f"{int(i)} {fx:.6f} {fy:.6f} {fz:.6f}\n" for i, (fx, fy, fz) in zip(ids, ld[:, 1:]))


def export_dataset_3dtsv(path, resolution, lower, upper, ele_map_back, nod_map_back, fixing, loading, stress):
    """Write the .carti dataset.  resolution = (resX, resY, resZ) of the padded
    finest grid; lower/upper = boundingBox_ rows; stress = nodal [xx yy zz yz zx xy]."""
    stress = np.asarray(stress, dtype=np.float64).reshape(-1, 6)
    fixing = np.asarray(fixing, dtype=np.int64).ravel()
    out = ["DATASET CARTESIAN_GRID \n",
           "Resolution:" + "".join(f" {int(r)}" for r in resolution) + "\n",
           "LowerBound:" + "".join(f" {v:.6f}" for v in lower) + "\n",
           "UpperBound:" + "".join(f" {v:.6f}" for v in upper) + "\n",
           f"ELEMENTS {len(ele_map_back)} int \n",
           "".join(f"{int(e) - 1}\n" for e in ele_map_back),
           "Number of Stress Fields: 1\n",
           f"Node Forces: {np.asarray(loading).reshape(-1, 4).shape[0]}\n",
           _loads_rows(loading, nod_map_back, 1),
           f"Fixed Nodes: {len(fixing)}\n",
           "".join(f"{int(nod_map_back[i - 1]) - 1}\n" for i in fixing),
           f"Cartesian Stress: {len(nod_map_back)}\n",
           "".join("{:.6e} {:.6e} {:.6e} {:.6e} {:.6e} {:.6e}\n".format(*row) for row in stress)]
    with open(path, "w") as f:
        f.write("".join(out))


def wrap_voxel_fea_model(path, resolution, ele_map_back, nod_map_back, fixing, loading):
    """Write the wrapped voxel FEA model (1-based grid indices)."""
    fixing = np.asarray(fixing, dtype=np.int64).ravel()
    out = ["domain type: 3D \n",
           "resolution: " + " ".join(str(int(r)) for r in resolution) + "\n",
           f"valid elements: {len(ele_map_back)}\n",
           "".join(f"{int(e)}\n" for e in ele_map_back),
           f"fixed position: {len(fixing)}\n",
           "".join(f"{int(nod_map_back[i - 1])} 1 1 1\n" for i in fixing),
           f"loading condition: {np.asarray(loading).reshape(-1, 4).shape[0]}\n",
           _loads_rows(loading, nod_map_back, 0)]
    with open(path, "w") as f:
        f.write("".join(out))
