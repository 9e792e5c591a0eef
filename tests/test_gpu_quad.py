"""The four-nodes-per-thread stencil kernels (quad.cu, f32x2 arithmetic)
against the one-node-per-thread kernels they replace (fine.cu) and the oracle.

Both compute the same FP32 operations in the same order per node, so the
V-cycle (down-sweeps on every level that uses the streaming kernel, the
per-element levels included) is bit-identical.  In a solve the CG direction
kernel's dot product p.q sums the same products in a different order per
thread, so the mixed solve agrees with the one-node kernels to rounding of
that sum (same iteration count, displacement within 1e-9) and with the
oracle to the mixed path's tolerance.
"""
import numpy as np
import pytest

from gmgs import Solver, synthetic
from gmgs_oracle import Oracle, Params

pytestmark = pytest.mark.gpu

CASES = {
    "ragged_L3": (lambda: synthetic.sphere_voids(21, 13, 18, 6, 7), 3, None),
    "block42_L4": (lambda: synthetic.make("block42_fp64")[0], 4, None),
    # levels 3-4 hold per-element Galerkin matrices: those nodes go to the per-element kernel
    "block42_L5": (lambda: synthetic.make("block42_fp64")[0], 5, None),
    "density_L3": (lambda: synthetic.sphere_voids(28, 24, 32, 2, 5), 3, (0.3, 1.0)),
    # several 32 x 16 tiles and z-chunks, ragged in y and x
    "wide_L4": (lambda: synthetic.sphere_voids(75, 70, 40, 12, 11), 4, None),
}
VARIANTS = ["1", "3"]     # the kernel at 4 and 3 resident CTAs per SM


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


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("name", list(CASES))
def test_quad_vcycle_bit_identical(name, variant, monkeypatch):
    vox, fixed, loads, L, rho = _inputs(name)
    s = _solver(vox, fixed, loads, L, rho)
    s.solve()
    rng = np.random.default_rng(4)
    r = rng.standard_normal(3 * s.num_nodes(1))
    monkeypatch.setenv("GMGS_QUAD", "0")
    z_ref = s.apply_preconditioner(r)
    monkeypatch.setenv("GMGS_QUAD", variant)
    z_q = s.apply_preconditioner(r)
    assert np.array_equal(z_q, z_ref)
    s.close()


@pytest.mark.parametrize("name", list(CASES))
def test_quad_mixed_solve(name, monkeypatch):
    vox, fixed, loads, L, rho = _inputs(name)
    monkeypatch.setenv("GMGS_QUAD", "0")
    s0 = _solver(vox, fixed, loads, L, rho)
    u0 = s0.solve()
    monkeypatch.setenv("GMGS_QUAD", "1")
    s1 = _solver(vox, fixed, loads, L, rho)
    u1 = s1.solve()
    assert s1.status == 0 and s1.iterations == s0.iterations
    assert rel(u1, u0) < 1e-9
    o = Oracle(vox, Params(omega=0.4, num_levels=L))
    o.apply_boundary_condition(fixed, loads)
    if rho is not None:
        o.set_density(rho, 3.0)
    u_ref = o.get_deformation()
    assert abs(s1.iterations - o.iterations) <= 1
    assert rel(u1, u_ref) < 1e-5
    s0.close()
    s1.close()
