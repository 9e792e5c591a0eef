"""The oracle's adjoint gradient (extension beyond the reference) against
central finite differences.  The solves are exact (sparse direct): at the
reference's tolerance 1e-3 the finite-difference quotient would be noise,
and the reference's PCG can stagnate long before machine precision (its
post-smoother reuses the pre-smoothing residual, so the preconditioner is
not symmetric)."""
import numpy as np
import pytest

from gmgs import synthetic
import gmgs_oracle as G


def _model(seed=5):
    vox = synthetic.sphere_voids(7, 6, 8, 1, seed)
    fixed, loads = synthetic.boundary_conditions(vox, 2)
    rho = synthetic.density(int(vox.sum()), (0.2, 1.0), seed)
    return vox, fixed, loads, rho


def _solve(vox, fixed, loads, rho, penal=3.0):
    o = G.Oracle(vox, G.Params(omega=0.4, num_levels=2))
    o.apply_boundary_condition(fixed, loads)
    o.set_density(rho, penal)
    u = o.direct_solve()
    return o, u


@pytest.mark.parametrize("functional", ["compliance", "tip"])
def test_gradient_matches_central_differences(functional):
    vox, fixed, loads, rho = _model()
    o, u = _solve(vox, fixed, loads, rho)
    ell = None
    if functional == "tip":
        ell = np.zeros_like(u)
        ell[3 * (int(loads[0, 0]) - 1) + 2] = 1.0      # z displacement of one loaded node
        J = lambda uu: ell @ uu
    else:
        J = lambda uu: o.F @ uu
    lam = None if ell is None else o.direct_solve(ell)
    g = o.gradient(u, ell, lam=lam)
    rng = np.random.default_rng(0)
    idx = rng.choice(len(rho), size=8, replace=False)
    h = 1e-4
    for e in idx:
        rp, rm = rho.copy(), rho.copy()
        rp[e] += h
        rm[e] -= h
        _, up = _solve(vox, fixed, loads, rp)
        _, um = _solve(vox, fixed, loads, rm)
        fd = (J(up) - J(um)) / (2 * h)
        assert abs(fd - g[e]) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(g).max()), (e, fd, g[e])


def test_compliance_gradient_is_negative():
    """Adding stiffness never increases compliance."""
    vox, fixed, loads, rho = _model(10)
    o, u = _solve(vox, fixed, loads, rho)
    g = o.gradient(u)
    assert np.all(g <= 1e-15)


def test_stress_scales_with_uniform_density():
    """Stress of a fixed displacement scales with a uniform rho^penal."""
    vox, fixed, loads, rho = _model()
    o, u = _solve(vox, fixed, loads, np.ones_like(rho))
    o.U = u
    n1, v1 = o.get_cartesian_stress()
    o.set_density(np.full_like(rho, 0.5), 3.0)
    o.setup()
    o.U = u
    n2, v2 = o.get_cartesian_stress()
    assert np.allclose(n2, 0.125 * n1, rtol=1e-12, atol=1e-15)
    assert np.allclose(v2, 0.125 * v1, rtol=1e-12, atol=1e-15)
