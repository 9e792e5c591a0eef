"""Device-buffer entry points (gmgs_apply_operator_dev, gmgs_apply_preconditioner_dev,
gmgs_dot_dev) against their host-buffer twins and NumPy.  torch only holds
device memory here; every computation runs in libgmgs."""
import numpy as np
import pytest

from gmgs import Solver, synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def solver():
    vox = synthetic.sphere_voids(19, 14, 22, 5, 21)
    fixed, loads = synthetic.boundary_conditions(vox, 3)
    s = Solver(vox, omega=0.4, num_levels=3)
    s.set_bc(fixed, loads)
    s.solve()
    return s


def test_operator_dev_matches_host(solver):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    for level in range(1, solver.num_levels + 1):
        x = rng.standard_normal(3 * solver.num_nodes(level))
        xd = torch.tensor(x, device="cuda")
        yd = torch.empty_like(xd)
        solver.apply_operator_dev(xd.data_ptr(), yd.data_ptr(), level)
        assert np.array_equal(yd.cpu().numpy(), solver.apply_operator(x, level))


def test_preconditioner_dev_matches_host(solver):
    torch = pytest.importorskip("torch")
    r = np.random.default_rng(4).standard_normal(3 * solver.num_nodes(1))
    rd = torch.tensor(r, device="cuda")
    zd = torch.empty_like(rd)
    solver.apply_preconditioner_dev(rd.data_ptr(), zd.data_ptr())
    assert np.array_equal(zd.cpu().numpy(), solver.apply_preconditioner(r))


@pytest.mark.parametrize("n", [1, 1000, 3_000_001])
def test_dot_dev(solver, n):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n)
    a, b = rng.standard_normal(n), rng.standard_normal(n)
    ad, bd = torch.tensor(a, device="cuda"), torch.tensor(b, device="cuda")
    v1 = solver.dot_dev(ad.data_ptr(), bd.data_ptr(), n)
    v2 = solver.dot_dev(ad.data_ptr(), bd.data_ptr(), n)
    assert v1 == v2                               # deterministic
    ref = float(np.dot(a, b))
    assert abs(v1 - ref) <= 1e-12 * np.sum(np.abs(a * b))


def test_two_handles_with_different_materials_solve_independently():
    """Element matrices and stencils are per handle (kernel parameters), so two
    live handles with different voxel sizes and moduli do not interfere."""
    import gmgs_oracle as G
    from gmgs import Solver, synthetic
    vox = synthetic.sphere_voids(12, 10, 16, 1, 21)
    fixed, loads = synthetic.boundary_conditions(vox, 2)
    cfg = [dict(ele_size=(1.0, 1.0, 1.0), youngs_modulus=1.0), dict(ele_size=(0.5, 1.5, 2.0), youngs_modulus=7.0)]
    solvers, refs = [], []
    for c in cfg:
        s = Solver(vox, num_levels=2, omega=0.4, **c)
        s.set_bc(fixed, loads)
        solvers.append(s)
        o = G.Oracle(vox, G.Params(num_levels=2, omega=0.4, youngs_modulus=c["youngs_modulus"]),
                     ele_size=c["ele_size"])
        o.apply_boundary_condition(fixed, loads)
        refs.append(o.get_deformation())
    for _ in range(2):                       # alternate: each solve must use its own handle's coefficients
        for s, u_ref in zip(solvers, refs):
            u = s.solve()
            assert np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref) < 1e-6
