"""The V-cycle down-sweep on the tensor cores (tc.cu, tcgen05 kind::tf32,
element form) against the FP32 CUDA-core kernels it replaces (GMGS_TC=0)
and against the oracle.

The tensor cores read the down-sweep's element differences as TF32 (10-bit
mantissa).  That only changes the preconditioner: the preconditioned residual
agrees with the FP32 kernels' and the oracle's to TF32 accuracy, and the
mixed solve reaches the same tolerance within one iteration of the oracle's
count, with the displacement within 1e-5 of the FP64 oracle.
"""
import numpy as np
import pytest

from gmgs import Solver, synthetic
from gmgs_oracle import Oracle, Params

pytestmark = pytest.mark.gpu

CASES = {
    "ragged_L3": (lambda: synthetic.sphere_voids(21, 13, 18, 6, 7), 3, None),
    "block42_L4": (lambda: synthetic.make("block42_fp64")[0], 4, None),
    # levels 3-4 store one Galerkin matrix per element: their nodes go to the per-element kernel
    "block42_L5": (lambda: synthetic.make("block42_fp64")[0], 5, None),
    # finest-level element scales: every level below holds per-element matrices
    "density_L3": (lambda: synthetic.sphere_voids(28, 24, 32, 2, 5), 3, (0.3, 1.0)),
}


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _inputs(name):
    build, L, rho_range = CASES[name]
    vox = build()
    fixed, loads = synthetic.boundary_conditions(vox, L)
    rho = synthetic.density(int(vox.sum()), rho_range, 5) if rho_range else None
    return vox, fixed, loads, L, rho


def _solver(vox, fixed, loads, L, rho):
    s = Solver(vox, omega=0.4, num_levels=L, precision="mixed")
    s.set_bc(fixed, loads)
    if rho is not None:
        s.set_density(rho, 3.0)
    return s


@pytest.mark.parametrize("name", list(CASES))
def test_tc_preconditioner_matches_fp32_kernels_and_oracle(name, monkeypatch):
    vox, fixed, loads, L, rho = _inputs(name)
    s = _solver(vox, fixed, loads, L, rho)
    s.solve()                                   # builds the coarse operators and work buffers
    o = Oracle(vox, Params(omega=0.4, num_levels=L))
    o.apply_boundary_condition(fixed, loads)
    if rho is not None:
        o.set_density(rho, 3.0)
    o.setup()
    rng = np.random.default_rng(3)
    r = rng.standard_normal(3 * s.num_nodes(1))
    r[o.levels[0].fixedDOFs] = 0
    monkeypatch.setenv("GMGS_TC", "1")
    z_tc = s.apply_preconditioner(r)
    z_tc2 = s.apply_preconditioner(r)
    monkeypatch.setenv("GMGS_TC", "0")
    z_cc = s.apply_preconditioner(r)
    z_ref = o.vcycle(r)
    assert np.array_equal(z_tc, z_tc2)          # deterministic
    assert rel(z_cc, z_ref) < 1e-5              # FP32 CUDA-core V-cycle
    assert rel(z_tc, z_cc) < 3e-3               # TF32 down-sweep operands
    assert rel(z_tc, z_ref) < 3e-3
    s.close()


@pytest.mark.parametrize("name", list(CASES))
def test_tc_mixed_solve_matches_oracle(name, monkeypatch):
    vox, fixed, loads, L, rho = _inputs(name)
    o = Oracle(vox, Params(omega=0.4, num_levels=L))
    o.apply_boundary_condition(fixed, loads)
    if rho is not None:
        o.set_density(rho, 3.0)
    u_ref = o.get_deformation()
    monkeypatch.setenv("GMGS_TC", "1")
    s = _solver(vox, fixed, loads, L, rho)
    u = s.solve()
    assert s.status == 0 and s.relres < 1e-3
    assert abs(s.iterations - o.iterations) <= 1
    assert rel(u, u_ref) < 1e-5
    s.close()
