"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

FP64 path: operators and V-cycle to 1e-11 relative, PCG iteration counts
identical, residual histories to 1e-8 relative, displacement to 1e-6
relative (the displacement bar of the drop-in), stress to 1e-8 relative.
Mixed path: same iteration count, displacement within 1e-5 relative of the
FP64 oracle solve at tolerance 1e-3.
"""
import numpy as np
import pytest

from gmgs import Solver, synthetic
from gmgs_oracle import Oracle, Params

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


CASES = {
    # name: (voxels builder, num_levels, omega)
    "cube12_L3": (lambda: np.ones((12, 12, 12), np.int32), 3, 0.4),
    "block42_L4": (lambda: synthetic.make("block42_fp64")[0], 4, 0.4),
    "ragged_L3": (lambda: synthetic.sphere_voids(21, 13, 18, 6, 7), 3, 0.4),
    # five levels: level 4 stores one Galerkin matrix per element and is smoothed
    "block42_L5": (lambda: synthetic.make("block42_fp64")[0], 5, 0.4),
    # a long column: the coarsest level (3 x 3 x 50 elements, 2376 free DOFs)
    # splits into 19 diagonal blocks of order 128, so both sweeps of the
    # two-ended block LDL^T run long chains
    "column_L3": (lambda: synthetic.sphere_voids(9, 10, 200, 6, 5), 3, 0.4),
}

# V-cycle agreement bar.  The column's coarsest matrix has condition number
# 2e7, so last-bit differences in the restricted residual (summation order of
# the smoother and the restriction) come out of the coarsest solve amplified
# to about cond * eps = 2e-9 relative; a dense inverse Cholesky factor of the
# whole coarsest matrix gives 2.45e-9 here as well.
VCYCLE_TOL = {"column_L3": 1e-8}


def _pair(name, precision="fp64", tol=1e-3):
    build, L, omega = CASES[name]
    vox = build()
    fixed, loads = synthetic.boundary_conditions(vox, L)
    o = Oracle(vox, Params(omega=omega, num_levels=L, tol=tol))
    o.apply_boundary_condition(fixed, loads)
    s = Solver(vox, omega=omega, num_levels=L, tol=tol, precision=precision)
    s.set_bc(fixed, loads)
    return o, s


@pytest.fixture(scope="module", params=list(CASES))
def solved_pair(request):
    o, s = _pair(request.param)
    u_ref = o.get_deformation()
    u = s.solve(with_history=True)
    return request.param, o, s, u_ref, u


def test_sizes_match(solved_pair):
    _, o, s, _, _ = solved_pair
    assert s.num_levels == o.numLevels
    for l, lv in enumerate(o.levels):
        assert s.num_nodes(l + 1) == lv.numNodes
        assert s.num_elements(l + 1) == lv.numElements


def test_operator_each_level(solved_pair):
    _, o, s, _, _ = solved_pair
    rng = np.random.default_rng(0)
    for l, lv in enumerate(o.levels):
        x = rng.standard_normal(lv.numDOFs)
        y_ref = o.atx(x, l)
        y = s.apply_operator(x, l + 1)
        assert rel(y, y_ref) < 1e-11, f"level {l + 1}"


def test_vcycle(solved_pair):
    name, o, s, _, _ = solved_pair
    rng = np.random.default_rng(1)
    r = rng.standard_normal(o.levels[0].numDOFs)
    r[o.levels[0].fixedDOFs] = 0
    assert rel(s.apply_preconditioner(r), o.vcycle(r)) < VCYCLE_TOL.get(name, 1e-10)


def test_pcg_history_and_displacement(solved_pair):
    _, o, s, u_ref, u = solved_pair
    assert s.status == 0
    assert s.iterations == o.iterations
    h_ref = np.array([h[2] for h in o.iterationHist])
    assert s.history.shape[0] == len(h_ref)
    if len(h_ref):
        assert np.max(np.abs(s.history[:, 2] - h_ref) / h_ref) < 1e-8
    assert abs(s.relres - o.relres) / o.relres < 1e-8
    assert rel(u, u_ref) < 1e-6


def test_stress(solved_pair):
    _, o, s, u_ref, u = solved_pair
    nodal_ref, vox_ref = o.get_cartesian_stress()
    nodal, vox = s.stress()
    assert rel(nodal, nodal_ref) < 1e-6
    assert rel(vox, vox_ref) < 1e-5   # FP32 output


@pytest.mark.parametrize("name", ["block42_L4", "ragged_L3", "block42_L5"])
def test_mixed_precision_error(name):
    o, s = _pair(name, precision="mixed")
    u_ref = o.get_deformation()
    u = s.solve(with_history=True)
    assert s.status == 0
    assert s.iterations == o.iterations
    assert rel(u, u_ref) < 1e-5
    h_ref = np.array([h[2] for h in o.iterationHist])
    assert np.max(np.abs(s.history[:, 2] - h_ref) / h_ref) < 1e-4


def test_divergent_omega_matches_oracle():
    """omega = 0.6 diverges on void models in the reference algorithm as well:
    both residual histories grow identically until the solve gives up."""
    vox = synthetic.make("block42_fp64")[0]
    fixed, loads = synthetic.boundary_conditions(vox, 4)
    o = Oracle(vox, Params(omega=0.6, num_levels=4, max_it=12))
    o.apply_boundary_condition(fixed, loads)
    with np.errstate(all="ignore"):
        o.get_deformation()
    s = Solver(vox, omega=0.6, num_levels=4, max_it=12)
    s.set_bc(fixed, loads)
    s.solve(with_history=True)
    assert s.status == 7       # GMGS_ERR_MAX_ITERATIONS
    h_ref = np.array([h[2] for h in o.iterationHist])
    assert len(h_ref) == 13 and s.history.shape[0] == 13
    assert h_ref[-1] > h_ref[0]
    assert np.max(np.abs(s.history[:, 2] - h_ref) / h_ref) < 1e-6


def test_repeat_solve_is_bitwise_identical():
    _, s = _pair("ragged_L3")
    u1 = s.solve()
    u2 = s.solve()
    assert np.array_equal(u1, u2)


def test_second_boundary_condition_changes_level_one_only():
    """GetDeformation.m:12-16 runs SetupSolver() once: new fixings given to a
    solved model change the finest level, while the coarse fixed DOFs and the
    coarsest factorisation keep the first ones.  The GPU and the oracle
    follow the same call sequence to the same iterations and displacement."""
    vox = synthetic.sphere_voids(21, 13, 18, 6, 7)
    fixed_a, loads = synthetic.boundary_conditions(vox, 3)
    fixed_b = fixed_a[: len(fixed_a) // 2]          # half of the base plane
    o = Oracle(vox, Params(omega=0.4, num_levels=3))
    o.apply_boundary_condition(fixed_a, loads)
    o.get_deformation()
    o.apply_boundary_condition(fixed_b, loads)
    u_ref = o.get_deformation()
    s = Solver(vox, omega=0.4, num_levels=3)
    s.set_bc(fixed_a, loads)
    s.solve()
    s.set_bc(fixed_b, loads)
    u = s.solve()
    assert s.iterations == o.iterations
    assert rel(u, u_ref) < 1e-6


def test_graph_replay_matches_eager_launches(monkeypatch):
    """The mixed PCG iterations replayed from CUDA graphs (GMGS_GRAPH=1) give
    bitwise the same solution as eager launches."""
    vox = synthetic.make("block42_fp64")[0]
    fixed, loads = synthetic.boundary_conditions(vox, 4)
    s = Solver(vox, omega=0.4, num_levels=4, precision="mixed")
    s.set_bc(fixed, loads)
    monkeypatch.setenv("GMGS_GRAPH", "1")
    u_graph = s.solve()
    u_graph2 = s.solve()                            # cached graphs
    monkeypatch.delenv("GMGS_GRAPH")
    u_eager = s.solve()
    assert s.iterations > 2
    assert np.array_equal(u_graph, u_eager)
    assert np.array_equal(u_graph2, u_eager)


def test_duplicate_load_rows_last_one_wins():
    """ApplyBoundaryCondition.m:9: a node listed twice in the loading
    condition takes its later row (the device picks the largest row index)."""
    vox = synthetic.sphere_voids(21, 13, 18, 6, 7)
    fixed, loads = synthetic.boundary_conditions(vox, 3)
    loads = np.asarray(loads, dtype=np.float64).reshape(-1, 4)
    early = loads[:5].copy()
    early[:, 1:] = 7.0                                   # overridden by the rows that follow
    late = loads[-3:].copy()
    late[:, 1:] *= 2.0                                   # overrides the rows before
    dup = np.vstack([early, loads, late])
    expect = loads.copy()
    expect[-3:, 1:] *= 2.0
    a = Solver(vox, omega=0.4, num_levels=3)
    a.set_bc(fixed, dup)
    b = Solver(vox, omega=0.4, num_levels=3)
    b.set_bc(fixed, expect)
    assert np.array_equal(a.solve(), b.solve())


def test_solve_into_caller_buffer():
    """Solver.solve(out=...) writes U into the caller's array (the bench keeps
    it in pinned host memory) with the same values as a fresh output."""
    o, s = _pair("ragged_L3")
    u = s.solve()
    buf = np.full_like(u, np.nan)
    u2 = s.solve(out=buf)
    assert u2 is buf
    assert np.array_equal(buf, u)
    with pytest.raises(ValueError):
        s.solve(out=np.zeros(u.size, dtype=np.float32))
    with pytest.raises(ValueError):
        s.solve(out=np.zeros(u.size + 3))



@pytest.mark.parametrize("density", [False, True])
def test_mixed_stress_matches_oracle_on_same_displacement(density):
    """The mixed path recovers stress in FP32 arithmetic on a double-float
    split of U (hi + lo); on the same displacement the oracle's FP64 maps
    (GetCartesianStress.m:11-41 and the per-voxel centre stress) agree to
    FP32 accuracy."""
    vox = synthetic.sphere_voids(28, 24, 32, 2, 5)
    fixed, loads = synthetic.boundary_conditions(vox, 3)
    rho = synthetic.density(int(vox.sum()), (0.3, 1.0), 5) if density else None
    s = Solver(vox, omega=0.4, num_levels=3, precision="mixed")
    s.set_bc(fixed, loads)
    o = Oracle(vox, Params(omega=0.4, num_levels=3))
    o.apply_boundary_condition(fixed, loads)
    if density:
        s.set_density(rho, 3.0)
        o.set_density(rho, 3.0)
    u = s.solve()
    o.setup()
    o.U = u
    nodal_ref, vox_ref = o.get_cartesian_stress()
    nodal, vox6 = s.stress()
    assert rel(nodal, nodal_ref) < 2e-6
    assert rel(vox6, vox_ref) < 2e-6
