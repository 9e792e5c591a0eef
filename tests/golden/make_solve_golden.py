"""Golden solve fixtures from the CPU oracle at benchmark-workload scale.

    python tests/golden/make_solve_golden.py WORKLOAD [--solid] [--levels L] [--omega W]
        [--no-density] [--scale S]

Runs the oracle (oracle/gmgs_oracle.py, the FP64 restatement of the
reference's SetupSolver / CG_solver / Vcycle / GetCartesianStress) to
relative residual 1e-3 on one of the seeded synthetic workloads of
gmgs.synthetic and writes tests/golden/solve_<name>.npz with:

* the workload's parameters (shape, levels, omega, tol, seed) and DOF count;
* the PCG iteration count, final relative residual and the residual history
  (iterationHist_, CG_solver.m:49);
* ||U||, the sum of each displacement component, and U at 20,000 seeded DOF
  indices;
* ||sigma|| of the nodal stress and the nodal stress at 5,000 seeded nodes.

The full displacement of these models (tens to hundreds of MB) is not stored;
the GPU tests compare their own solve with these figures.  `--solid` drops
the voids (a solid block of the workload's size), `--no-density` drops the
workload's density field, `--scale` shrinks the resolution the way
gmgs.synthetic.make does (the voids keep their number and radii).
"""
import argparse
import json
import resource
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path[:0] = [str(ROOT / "oracle"), str(ROOT / "gmgs-3d_gb300")]
from gmgs import synthetic          # noqa: E402
from gmgs_oracle import Oracle, Params   # noqa: E402

N_DOF_SAMPLES = 20_000
N_NODE_SAMPLES = 5_000


def fixture_name(workload: str, solid: bool, levels: int, density: bool, scale: float = 1.0) -> str:
    name = workload + ("_solid" if solid else "")
    if scale != 1.0:
        name += f"_s{scale:g}"
    if levels:
        name += f"_L{levels}"
    if not density:
        name += "_nodensity"
    return name


def build(workload: str, solid: bool, levels: int, density: bool, scale: float = 1.0):
    w = synthetic.WORKLOADS[workload]
    nelx, nely, nelz = (max(2, int(round(n * scale))) for n in (w.nelx, w.nely, w.nelz))
    if solid:
        vox = np.ones((nely, nelx, nelz), np.int32)
    else:
        vox = synthetic.sphere_voids(nelx, nely, nelz, w.voids, w.seed)
    L = synthetic.level_count(nely, nelx, nelz, levels or w.num_levels)
    fixed, loads = synthetic.boundary_conditions(vox, L)
    rho = None
    if density and w.rho_range is not None:
        rho = synthetic.density(int(vox.sum()), w.rho_range, w.seed)
    return vox, fixed, loads, L, rho, w


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=sorted(synthetic.WORKLOADS))
    ap.add_argument("--solid", action="store_true")
    ap.add_argument("--levels", type=int, default=0)
    ap.add_argument("--omega", type=float, default=0.4)
    ap.add_argument("--no-density", action="store_true")
    ap.add_argument("--scale", type=float, default=1.0)
    a = ap.parse_args()
    density = not a.no_density
    vox, fixed, loads, L, rho, w = build(a.workload, a.solid, a.levels, density, a.scale)
    t0 = time.perf_counter()
    o = Oracle(vox, Params(omega=a.omega, num_levels=L, tol=w.tol))
    o.apply_boundary_condition(fixed, loads)
    if rho is not None:
        o.set_density(rho, w.penal)
    o.setup()
    t1 = time.perf_counter()
    u = o.get_deformation()
    t2 = time.perf_counter()
    nodal, _ = o.get_cartesian_stress()
    rng = np.random.default_rng(20260)
    dof_idx = np.sort(rng.choice(u.size, size=min(N_DOF_SAMPLES, u.size), replace=False))
    node_idx = np.sort(rng.choice(nodal.shape[0], size=min(N_NODE_SAMPLES, nodal.shape[0]), replace=False))
    hist = np.array([h[2] for h in o.iterationHist])
    name = fixture_name(a.workload, a.solid, a.levels, density, a.scale)
    out = HERE / f"solve_{name}.npz"
    meta = {"workload": a.workload, "solid": a.solid, "scale": a.scale, "levels": L, "omega": a.omega, "tol": w.tol,
            "density": rho is not None, "penal": w.penal, "shape_y_x_z": list(vox.shape),
            "dofs": int(u.size), "iterations": int(o.iterations), "relres": float(o.relres),
            "oracle_setup_s": t1 - t0, "oracle_solve_s": t2 - t1,
            "peak_rss_gb": resource.getrusage(resource.RUSAGE_SELF).ru_maxrss / 1e6}
    np.savez_compressed(out, meta=json.dumps(meta), history=hist, u_norm=np.linalg.norm(u),
                        u_comp_sum=u.reshape(-1, 3).sum(axis=0), dof_idx=dof_idx, u_samples=u[dof_idx],
                        stress_norm=np.linalg.norm(nodal), node_idx=node_idx, stress_samples=nodal[node_idx])
    print(json.dumps(meta))
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
