"""GPU solves at benchmark-workload scale against the oracle's golden fixtures.

tests/golden/solve_*.npz hold what the CPU oracle (the FP64 restatement of
CG_solver.m / Vcycle.m / SetupSolver.m) computed on the full-size seeded
workloads: iteration count, residual history, ||U||, U at 20,000 seeded DOFs
and nodal stress at 5,000 seeded nodes (tests/golden/make_solve_golden.py
made them).  The CUDA path, called through the C ABI on the same inputs, must
give:

* FP64 path (the drop-in): the same iteration count, residual history and
  final relative residual within 1e-8, displacement within 1e-6 relative,
  nodal stress within 1e-6 relative;
* mixed path: the same iteration count (one more at most), displacement
  within 1e-5 relative, nodal stress within 1e-4 relative.
"""
import importlib.util
import json
from pathlib import Path

import numpy as np
import pytest

from gmgs import Solver

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = sorted(GOLDEN.glob("solve_*.npz"))


def _generator():
    spec = importlib.util.spec_from_file_location("make_solve_golden", GOLDEN / "make_solve_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module", params=FIXTURES, ids=lambda p: p.stem)
def case(request):
    g = np.load(request.param)
    meta = json.loads(str(g["meta"]))
    gen = _generator()
    vox, fixed, loads, L, rho, w = gen.build(meta["workload"], meta["solid"], meta["levels"], meta["density"],
                                                 meta.get("scale", 1.0))
    assert L == meta["levels"] and list(vox.shape) == meta["shape_y_x_z"]
    return meta, g, (vox, fixed, loads, L, rho, w)


def _solve(inputs, meta, precision):
    vox, fixed, loads, L, rho, w = inputs
    s = Solver(vox, omega=meta["omega"], num_levels=L, tol=meta["tol"], precision=precision)
    s.set_bc(fixed, loads)
    if rho is not None:
        s.set_density(rho, meta["penal"])
    u = s.solve(with_history=True)
    nodal = s.stress(per_voxel=False)
    return s, u, nodal


def test_fp64_matches_oracle_at_scale(case):
    meta, g, inputs = case
    s, u, nodal = _solve(inputs, meta, "fp64")
    assert 3 * s.num_nodes(1) == meta["dofs"]
    assert s.status == 0
    assert s.iterations == meta["iterations"]
    h_ref = g["history"]
    assert s.history.shape[0] == len(h_ref)
    if len(h_ref):
        assert np.max(np.abs(s.history[:, 2] - h_ref) / h_ref) < 1e-8
    assert abs(s.relres - meta["relres"]) / meta["relres"] < 1e-8
    assert abs(np.linalg.norm(u) - float(g["u_norm"])) / float(g["u_norm"]) < 1e-6
    assert _rel(u[g["dof_idx"]], g["u_samples"]) < 1e-6
    assert _rel(nodal[g["node_idx"]], g["stress_samples"]) < 1e-6
    s.close()


def test_mixed_matches_oracle_at_scale(case):
    meta, g, inputs = case
    s, u, nodal = _solve(inputs, meta, "mixed")
    assert s.status == 0
    assert meta["iterations"] <= s.iterations <= meta["iterations"] + 1
    assert s.relres < meta["tol"]
    assert abs(np.linalg.norm(u) - float(g["u_norm"])) / float(g["u_norm"]) < 1e-5
    assert _rel(u[g["dof_idx"]], g["u_samples"]) < 1e-5
    assert _rel(nodal[g["node_idx"]], g["stress_samples"]) < 1e-4
    s.close()
