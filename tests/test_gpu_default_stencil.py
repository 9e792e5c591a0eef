"""The streaming kernels with the default material's coefficients compiled in
as instruction immediates (fine.cu, k_fine<MODE, true>; the table is
generated at build time from the library's own element code) against the
same kernels reading the coefficients from their parameter
(GMGS_DEFAULT_STENCIL=0).

Both compute the same FP32 operations with the same values, so the mixed
solve is bit-identical.  A model with another material takes the parameter
path and still matches the oracle.
"""
import numpy as np
import pytest

from gmgs import Solver, synthetic
from gmgs_oracle import Oracle, Params

pytestmark = pytest.mark.gpu

CASES = {
    "ragged_L3": (lambda: synthetic.sphere_voids(21, 13, 18, 6, 7), 3, None),
    "block42_L5": (lambda: synthetic.make("block42_fp64")[0], 5, None),
    "density_L3": (lambda: synthetic.sphere_voids(28, 24, 32, 2, 5), 3, (0.3, 1.0)),
}


def _solve(vox, L, rho, **kw):
    fixed, loads = synthetic.boundary_conditions(vox, L)
    s = Solver(vox, omega=0.4, num_levels=L, precision="mixed", **kw)
    s.set_bc(fixed, loads)
    if rho is not None:
        s.set_density(rho, 3.0)
    u = s.solve()
    its = s.iterations
    nodal, _ = s.stress()
    s.close()
    return u, its, nodal


@pytest.mark.parametrize("name", list(CASES))
def test_immediate_coefficients_bit_identical(name, monkeypatch):
    build, L, rr = CASES[name]
    vox = build()
    rho = synthetic.density(int(vox.sum()), rr, 5) if rr else None
    monkeypatch.setenv("GMGS_DEFAULT_STENCIL", "0")
    u0, it0, s0 = _solve(vox, L, rho)
    monkeypatch.delenv("GMGS_DEFAULT_STENCIL")
    u1, it1, s1 = _solve(vox, L, rho)
    assert it1 == it0
    assert np.array_equal(u1, u0)
    assert np.array_equal(s1, s0)


def test_other_material_takes_the_parameter_path():
    vox = synthetic.sphere_voids(21, 13, 18, 6, 7)
    L = 3
    fixed, loads = synthetic.boundary_conditions(vox, L)
    u, its, _ = _solve(vox, L, None, poisson_ratio=0.25, youngs_modulus=2.0, ele_size=(1.25, 1.25, 1.25))
    o = Oracle(vox, Params(omega=0.4, num_levels=L, poisson_ratio=0.25, youngs_modulus=2.0), ele_size=(1.25, 1.25, 1.25))
    o.apply_boundary_condition(fixed, loads)
    u_ref = o.get_deformation()
    assert abs(its - o.iterations) <= 1
    assert np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref) < 1e-5
