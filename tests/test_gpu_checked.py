"""The checked build (gmgs-3d_gb300/build.py --debug, GMGS_CHECKED) against
the oracle: every instrumented gather, scatter and shared-memory access of the
solver kernels tests its index, and an out-of-range one fails the C-ABI call
with GMGS_ERR_CUDA naming the kernel and index.  This stands in for
compute-sanitizer's memcheck, which is not available on these GPUs.

A child process loads libgmgs_checked.so (GMGS_LIB) and runs the FP64 and
mixed solves (the CUDA-core and the tensor-core down-sweep), the operator and
preconditioner calls, stress and the adjoint gradient on small models with
voids, a density field and a five-level hierarchy, each checked against the
oracle."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import sys
sys.path[:0] = [sys.argv[1] + '/gmgs-3d_gb300', sys.argv[1] + '/oracle']
import os
import numpy as np
from gmgs import Solver, synthetic
from gmgs_oracle import Oracle, Params
assert os.environ["GMGS_LIB"].endswith("libgmgs_checked.so")

def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)

cases = [("ragged_L3", synthetic.sphere_voids(21, 13, 18, 6, 7), 3, None),
         ("block42_L5", synthetic.make("block42_fp64")[0], 5, None),
         ("density_L3", synthetic.sphere_voids(28, 24, 32, 2, 5), 3, (0.3, 1.0))]
for name, vox, L, rr in cases:
    fixed, loads = synthetic.boundary_conditions(vox, L)
    rho = synthetic.density(int(vox.sum()), rr, 5) if rr else None
    o = Oracle(vox, Params(omega=0.4, num_levels=L))
    o.apply_boundary_condition(fixed, loads)
    if rho is not None:
        o.set_density(rho, 3.0)
    u_ref = o.get_deformation()
    nodal_ref, _ = o.get_cartesian_stress()
    for prec, tc in (("fp64", "0"), ("mixed", "0"), ("mixed", "1")):
        os.environ["GMGS_TC"] = tc
        s = Solver(vox, omega=0.4, num_levels=L, precision=prec)
        s.set_bc(fixed, loads)
        if rho is not None:
            s.set_density(rho, 3.0)
        u = s.solve()
        assert abs(s.iterations - o.iterations) <= 1, (name, prec, tc, s.iterations, o.iterations)
        assert rel(u, u_ref) < (1e-6 if prec == "fp64" else 1e-5), (name, prec, tc, rel(u, u_ref))
        nodal, vox6 = s.stress()
        assert rel(nodal, nodal_ref) < 1e-4, (name, prec, rel(nodal, nodal_ref))
        r = np.random.default_rng(1).standard_normal(u.size)
        for lvl in range(1, L + 1):
            try:
                s.apply_operator(np.random.default_rng(lvl).standard_normal(3 * s.num_nodes(lvl)), lvl)
            except Exception as e:
                if "level 2 keeps only FP32" not in str(e):
                    raise
        s.apply_preconditioner(r)
        if rho is not None:
            g = s.grad()
            assert np.all(np.isfinite(g))
        s.close()
    print("checked", name, "ok")
print("CHECKED BUILD OK")
"""


def test_checked_build_matches_oracle_without_violations():
    sys.path.insert(0, str(ROOT / "gmgs-3d_gb300"))
    import build as B   # gmgs-3d_gb300/build.py
    lib = B.build(debug=True)
    env = dict(os.environ, GMGS_LIB=str(lib))
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], env=env, capture_output=True, text=True,
                       timeout=1200)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    assert "CHECKED BUILD OK" in r.stdout
    assert "checked build:" not in r.stdout + r.stderr
