"""Adjoint gradient on the GPU (extension beyond the reference): against the
oracle's gradient from exact solves, against central finite differences of
GPU solves (step 1e-4, tolerance 1e-4 as the benchmark description asks), and
through the torch.autograd.Function binding.

The reference's PCG converges slowly near omega = 0.4 on graded densities
(lambda_max(D^-1 K) = 4.31 against 2/omega = 5 on this model), so these tight
solves use omega = 0.3; the gradient does not depend on omega."""
import numpy as np
import pytest

from gmgs import Solver, synthetic
import gmgs_oracle as G

pytestmark = pytest.mark.gpu

TOL = 1e-11


def _model():
    vox = synthetic.sphere_voids(12, 10, 14, 1, 10)
    fixed, loads = synthetic.boundary_conditions(vox, 2)
    rho = synthetic.density(int(vox.sum()), (0.2, 1.0), 10)
    return vox, fixed, loads, rho


def _gpu(vox, fixed, loads, precision="fp64", tol=TOL):
    s = Solver(vox, num_levels=2, omega=0.3, tol=tol, max_it=5000, precision=precision)
    s.set_bc(fixed, loads)
    return s


def _oracle(vox, fixed, loads, rho):
    o = G.Oracle(vox, G.Params(omega=0.3, num_levels=2))
    o.apply_boundary_condition(fixed, loads)
    o.set_density(rho, 3.0)
    return o


def _tip(s, loads):
    ell = np.zeros(3 * s.num_nodes(1))
    ell[3 * (int(loads[0, 0]) - 1) + 2] = 1.0
    return ell


def test_gradient_matches_oracle_exact_solves():
    vox, fixed, loads, rho = _model()
    s = _gpu(vox, fixed, loads)
    s.set_density(rho, 3.0)
    u = s.solve()
    assert s.status == 0
    o = _oracle(vox, fixed, loads, rho)
    u_ref = o.direct_solve()
    assert np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref) < 1e-8
    g = s.grad()
    g_ref = o.gradient(u_ref)
    assert np.max(np.abs(g - g_ref)) <= 1e-7 * np.abs(g_ref).max()
    ell = _tip(s, loads)
    g2 = s.grad(ell)
    g2_ref = o.gradient(u_ref, ell, lam=o.direct_solve(ell))
    assert np.max(np.abs(g2 - g2_ref)) <= 1e-7 * np.abs(g2_ref).max()


@pytest.mark.parametrize("functional", ["compliance", "tip"])
def test_gradient_matches_central_differences(functional):
    vox, fixed, loads, rho = _model()
    s = _gpu(vox, fixed, loads)
    ell = _tip(s, loads) if functional == "tip" else None
    s.set_density(rho, 3.0)
    s.solve()
    g = s.grad(ell)
    w = s.load_vector() if ell is None else ell

    def J(r):
        s.set_density(r, 3.0)
        return float(w @ s.solve())

    rng = np.random.default_rng(3)
    h = 1e-4
    for e in rng.choice(len(rho), size=8, replace=False):
        rp, rm = rho.copy(), rho.copy()
        rp[e] += h
        rm[e] -= h
        fd = (J(rp) - J(rm)) / (2 * h)
        assert abs(fd - g[e]) <= 1e-4 * max(abs(fd), 1e-2 * np.abs(g).max()), (e, fd, g[e])


def test_autograd_function():
    torch = pytest.importorskip("torch")
    from gmgs.autograd import compliance, displacement_functional
    vox, fixed, loads, rho = _model()
    s = _gpu(vox, fixed, loads)
    r = torch.tensor(rho, dtype=torch.float64, requires_grad=True)
    c = compliance(r, s)
    c.backward()
    s.set_density(rho, 3.0)
    u = s.solve()
    assert abs(c.item() - s.load_vector() @ u) <= 1e-12 * abs(c.item())
    assert np.allclose(r.grad.numpy(), s.grad(), rtol=1e-10, atol=0)
    ell = _tip(s, loads)
    r2 = torch.tensor(rho, dtype=torch.float64, requires_grad=True)
    j = displacement_functional(r2, s, ell)
    j.backward()
    assert np.all(np.isfinite(r2.grad.numpy()))
    assert np.allclose(r2.grad.numpy(), s.grad(ell), rtol=1e-10, atol=0)


def test_mixed_precision_gradient_close_to_fp64():
    vox, fixed, loads, rho = _model()
    out = {}
    for prec in ("fp64", "mixed"):
        s = _gpu(vox, fixed, loads, precision=prec, tol=1e-3)
        s.set_density(rho, 3.0)
        s.solve()
        out[prec] = s.grad()
    assert np.linalg.norm(out["mixed"] - out["fp64"]) <= 1e-4 * np.linalg.norm(out["fp64"])


def test_stress_with_density_same_displacement():
    """Stress kernels against the oracle's OTP*D*B / Gauss-mean matrices on the
    GPU's own displacement, with per-voxel stiffness scales."""
    vox, fixed, loads, rho = _model()
    s = _gpu(vox, fixed, loads, tol=1e-8)
    s.set_density(rho, 3.0)
    u = s.solve()
    o = _oracle(vox, fixed, loads, rho)
    o.setup()
    o.U = u
    nodal_ref, vox_ref = o.get_cartesian_stress()
    nodal, v6 = s.stress()
    assert np.max(np.abs(nodal - nodal_ref)) <= 1e-12 * np.abs(nodal_ref).max()
    assert np.max(np.abs(v6 - vox_ref)) <= 1e-6 * np.abs(vox_ref).max()


def test_block84_adjoint_central_differences_64_voxels():
    """The 84x73x128 adjoint workload (930K voxels, rho ~ U[0.2, 1], penal 3):
    compliance and tip-displacement gradients against central differences with
    step 1e-4 on 64 seeded random voxels, within 1e-4 relative.  FP64 solves to
    relres 1e-10 (omega 0.3, which converges in fewer iterations than 0.4 on
    graded densities)."""
    vox, fixed, loads, L, rho = synthetic.make("block84_adjoint")
    s = Solver(vox, omega=0.3, num_levels=L, tol=1e-10, max_it=5000, precision="fp64")
    s.set_bc(fixed, loads)
    s.set_density(rho, 3.0)
    s.solve()
    assert s.status == 0
    F = s.load_vector()
    ell = _tip(s, loads)
    g_c = s.grad()
    g_t = s.grad(ell)
    rng = np.random.default_rng(84)
    h = 1e-4
    worst = 0.0
    for e in rng.choice(len(rho), size=64, replace=False):
        rp, rm = rho.copy(), rho.copy()
        rp[e] += h
        rm[e] -= h
        s.set_density(rp, 3.0)
        up = s.solve()
        s.set_density(rm, 3.0)
        um = s.solve()
        for w, g in ((F, g_c), (ell, g_t)):
            fd = (w @ up - w @ um) / (2 * h)
            err = abs(fd - g[e]) / max(abs(fd), 1e-3 * np.abs(g).max())
            worst = max(worst, err)
            assert err <= 1e-4, (int(e), fd, g[e])
    print(f"worst relative FD error {worst:.2e}")


def test_mixed_density_three_levels_fp32_only_level2():
    """Mixed precision with a density field keeps the level-2 Galerkin matrices
    in FP32 only and builds level 3 from the 64 finest descendants; the solve
    and the gradient still match the FP64 path, and the FP64 operator of
    level 2 is reported as unavailable."""
    from gmgs.solver import GMGSError
    import gmgs._lib as L
    vox = synthetic.sphere_voids(24, 20, 28, 3, 17)
    fixed, loads = synthetic.boundary_conditions(vox, 3)
    rho = synthetic.density(int(vox.sum()), (0.3, 1.0), 17)
    out = {}
    for prec in ("fp64", "mixed"):
        s = Solver(vox, num_levels=3, omega=0.4, tol=1e-6, max_it=2000, precision=prec)
        s.set_bc(fixed, loads)
        s.set_density(rho, 3.0)
        u = s.solve()
        assert s.status == 0
        out[prec] = (u, s.iterations, s.grad(), s)
    (u64, it64, g64, s64), (u32, it32, g32, s32) = out["fp64"], out["mixed"]
    assert abs(it32 - it64) <= 1
    assert np.linalg.norm(u32 - u64) / np.linalg.norm(u64) < 1e-5
    assert np.linalg.norm(g32 - g64) / np.linalg.norm(g64) < 1e-4
    x = np.random.default_rng(0).standard_normal(3 * s64.num_nodes(2))
    s64.apply_operator(x, level=2)                     # FP64 handle: available
    with pytest.raises(GMGSError) as e:
        s32.apply_operator(x, level=2)
    assert e.value.status == L.ERR_STATE
