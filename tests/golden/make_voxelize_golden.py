"""Generate tests/golden/voxelize_dofs.json and the 64-resolution occupancies.

    python tests/golden/make_voxelize_golden.py [REFERENCE_DIR]

REFERENCE_DIR is a GMGS-3D checkout; without the argument the script reads
it from $GMGS_REFERENCE_DIR and stops when neither is given.
For every model and resolution of the reference README's statistics table
(README.md:29-41) this voxelises data/<model>.ply with the oracle restatement
(oracle/voxelize.py), discretises it with the oracle (DiscretizeDesignDomain),
and records the grid, solid voxels and DOFs next to the README figure, plus
the number and the largest node id of the reference's demo boundary
conditions for that model and resolution (data/demo_BC_<model>_<res>_*.dat),
which index the reference's compact node numbering.  The 64-resolution
occupancies are stored bit-packed, with those demos' boundary conditions, so
the tests can run the reference's own 64-resolution demos without the
reference checkout.
"""
import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path[:0] = [str(ROOT / "oracle"), str(ROOT / "gmgs-3d_gb300")]
import gmgs_oracle as G          # noqa: E402
import voxelize as V             # noqa: E402

# README.md:29-41 (Intel i7-7700K, tol 1e-3): resolution -> DOFs
README = {
    "kitten": {64: 120198, 128: 929961, 256: 6732912, 512: 52499889, 650: 106873614},
    "parts": {64: 141744, 128: 999342, 256: 7570380, 512: 58608732, 650: 118761510},
}


def reference_dir():
    """The reference checkout named by $GMGS_REFERENCE_DIR, or None."""
    import os
    d = os.environ.get("GMGS_REFERENCE_DIR")
    return Path(d) if d else None


def main():
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else reference_dir()
    if ref is None:
        raise SystemExit("give the GMGS-3D checkout as an argument or in $GMGS_REFERENCE_DIR")
    out = {}
    for model, table in README.items():
        out[model] = {}
        for res, readme_dofs in table.items():
            t0 = time.time()
            vol, bbox, grid = V.create_voxelized_model(ref / "data" / f"{model}.ply", res)
            fine, _, _ = G.discretize(vol, G.Params())
            fixed = np.loadtxt(ref / "data" / f"demo_BC_{model}_{res}_fixedNodes.dat", ndmin=1)
            loads = np.loadtxt(ref / "data" / f"demo_BC_{model}_{res}_loadingVec.dat", ndmin=2)
            out[model][str(res)] = {
                "grid_nx_ny_nz": list(grid), "solid_voxels": int(vol.sum()),
                "nodes": int(fine.numNodes), "dofs": 3 * int(fine.numNodes), "readme_dofs": readme_dofs,
                "bc_fixed_count": int(fixed.size), "bc_fixed_max_id": int(fixed.max()),
                "bc_load_count": int(loads.shape[0]), "bc_load_max_id": int(loads[:, 0].max()),
                # DiscretizeDesignDomain.m:53-65: bounding box / voxel counts
                "ele_size": ((bbox[1] - bbox[0]) / np.array(grid, dtype=float)).tolist(),
            }
            print(model, res, out[model][str(res)], f"{time.time() - t0:.1f}s", flush=True)
            if res == 64:
                np.savez_compressed(HERE / f"{model}64_occupancy.npz", shape=np.array(vol.shape),
                                    bits=np.packbits(vol.astype(bool).ravel(order="F")))
                # the demo's boundary conditions (Demo.m:15-18): fixingCond_ and loadingCond_
                np.savez_compressed(HERE / f"{model}64_demo_bc.npz", fixed=fixed.astype(np.int32), loads=loads)
    (HERE / "voxelize_dofs.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
