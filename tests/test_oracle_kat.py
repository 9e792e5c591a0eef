"""Known-answer checks that pin the CPU oracle.

The reference is MATLAB and ships no tests or golden outputs, so the oracle
is pinned by mathematics it must satisfy: an exact symbolic element matrix,
rigid-body modes, the trilinear transfer rules, the Galerkin identities the
reference relies on, adjointness of restriction and prolongation, and
equilibrium of the solved field.
"""
import numpy as np
import pytest

from gmgs import synthetic
import gmgs_oracle as G


def _exact_ke(E, nu, size):
    """Ke = int B^T D B over a box, by exact polynomial integration (sympy)."""
    sp = pytest.importorskip("sympy")
    s, t, p = sp.symbols("s t p")
    a, b, c = (sp.Rational(v).limit_denominator(1000) / 2 for v in size)   # half edge lengths
    signs = G._NODE_SIGNS.astype(int)
    N = [sp.Rational(1, 8) * (1 + i * s) * (1 + j * t) * (1 + k * p) for i, j, k in signs]
    dx = [sp.diff(n, s) / a for n in N]
    dy = [sp.diff(n, t) / b for n in N]
    dz = [sp.diff(n, p) / c for n in N]
    B = sp.zeros(6, 24)
    for k in range(8):
        B[0, 3 * k] = dx[k]; B[1, 3 * k + 1] = dy[k]; B[2, 3 * k + 2] = dz[k]
        B[3, 3 * k + 1] = dz[k]; B[3, 3 * k + 2] = dy[k]
        B[4, 3 * k] = dz[k]; B[4, 3 * k + 2] = dx[k]
        B[5, 3 * k] = dy[k]; B[5, 3 * k + 1] = dx[k]
    Er, nur = sp.Rational(E).limit_denominator(1000), sp.Rational(nu).limit_denominator(1000)
    c1 = (1 + nur) * (1 - 2 * nur)
    D = sp.zeros(6, 6)
    for i in range(3):
        for j in range(3):
            D[i, j] = Er * (nur if i != j else 1 - nur) / c1
    for i in range(3, 6):
        D[i, i] = Er / (2 * (1 + nur))
    integrand = (B.T * D * B) * (a * b * c)
    K = np.zeros((24, 24))
    for i in range(24):
        for j in range(i, 24):
            poly = sp.Poly(sp.expand(integrand[i, j]), s, t, p)
            val = 0
            for (es, et, ep), coef in poly.terms():
                m = 1
                for e in (es, et, ep):
                    m *= 0 if e % 2 else sp.Rational(2, e + 1)
                val += coef * m
            K[i, j] = K[j, i] = float(val)
    return K


@pytest.mark.parametrize("size", [(1.0, 1.0, 1.0), (1.0, 2.0, 0.5)])
def test_element_stiffness_exact(size):
    K = G.element_stiffness(1.0, 0.3, size)
    Kx = _exact_ke(1.0, 0.3, size)
    # 2x2x2 Gauss integrates this integrand exactly; the only error is the
    # reference's 15-digit Gauss abscissa (GaussianIntegral.m:11)
    assert np.max(np.abs(K - Kx)) / np.max(np.abs(Kx)) < 1e-14


def test_element_stiffness_rigid_modes():
    K = G.element_stiffness(1.0, 0.3)
    assert np.max(np.abs(K - K.T)) < 1e-15
    w = np.linalg.eigvalsh(0.5 * (K + K.T))
    assert np.all(np.abs(w[:6]) < 1e-14) and w[6] > 1e-2
    X = G.element_node_coords((1, 1, 1))
    modes = []
    for d in range(3):
        m = np.zeros((8, 3)); m[:, d] = 1; modes.append(m.ravel())
    for (i, j) in ((0, 1), (1, 2), (2, 0)):
        m = np.zeros((8, 3)); m[:, i] = -X[:, j]; m[:, j] = X[:, i]; modes.append(m.ravel())
    for m in modes:
        assert np.max(np.abs(K @ m)) < 1e-14


def test_trilinear_table_rules():
    RI = G.trilinear_node_table()
    assert RI.shape == (27, 8)
    assert np.allclose(RI.sum(axis=1), 1.0)                       # partition of unity
    assert set(np.unique(RI)) <= {0.0, 0.125, 0.25, 0.5, 1.0}
    # reproduces linear fields: fine-node coordinates from corner coordinates
    corners = 2 * G.LOCAL_CORNERS
    m = np.arange(27)
    fine = np.stack([m % 3, (m // 3) % 3, m // 9], axis=1)
    assert np.allclose(RI @ corners, fine)
    # every child's local nodes are its block corners (SubEleNodMat.m:3-11)
    sub = G.sub_element_nodes()
    assert sorted(np.unique(sub)) == list(range(27))
    assert sub[0].tolist() == [1, 4, 3, 0, 10, 13, 12, 9]           # 0-based ids of child (0,0,0)


def test_galerkin_of_full_children_is_scaled_ke():
    """The reference's universal shortcut Ke_l = Ke0 * 2^(l-1) (SetupSolver.m:37,47)."""
    Ke = G.element_stiffness(1.0, 0.3)
    kids = np.broadcast_to(Ke, (1, 8, 24, 24)).copy()
    Kc = G.Oracle._galerkin(kids)[0]
    assert np.max(np.abs(Kc - 2 * Ke)) < 1e-13


def _small(L=3, shape=(9, 11, 10), voids=4, seed=3, omega=0.4):
    nelx, nely, nelz = shape[1], shape[0], shape[2]
    vox = synthetic.sphere_voids(nelx, nely, nelz, voids, seed)
    fixed, loads = synthetic.boundary_conditions(vox, L)
    o = G.Oracle(vox, G.Params(omega=omega, num_levels=L))
    o.apply_boundary_condition(fixed, loads)
    o.setup()
    return o


def test_restriction_is_adjoint_of_prolongation():
    o = _small()
    rng = np.random.default_rng(0)
    for ii in range(1, o.numLevels):
        r = rng.standard_normal(o.levels[ii - 1].numDOFs)
        e = rng.standard_normal(o.levels[ii].numDOFs)
        lhs = o.restrict(r, ii) @ e
        rhs = r @ o.interpolate(e, ii)
        assert abs(lhs - rhs) < 1e-11 * (abs(lhs) + 1)


def test_matrix_free_equals_assembled():
    """AtX against the explicitly assembled K (DirectlyAssembleStifnessMatrix.m:7-23)."""
    o = _small()
    rng = np.random.default_rng(1)
    for ii in range(o.numLevels):
        K = o.assemble_level(ii)
        x = rng.standard_normal(K.shape[0])
        y = K @ x
        y[o.levels[ii].fixedDOFs] = 0
        assert np.allclose(o.atx(x, ii), y, rtol=0, atol=1e-11 * np.abs(y).max())


def test_galerkin_identity_state1():
    """With two levels every coarse element is Galerkin: K_c = P^T K_f P."""
    o = _small(L=2, shape=(8, 6, 10), voids=0)
    Kf = o.assemble_level(0)
    Kc = o.assemble_level(1)
    nc = o.levels[1].numDOFs
    P = np.stack([o.interpolate(np.eye(nc)[:, j], 1) for j in range(nc)], axis=1)
    assert np.max(np.abs(P.T @ Kf @ P - Kc)) < 1e-12 * np.abs(Kc).max()


def test_oracle_solution_equilibrium():
    o = _small(L=3, shape=(12, 10, 14), voids=3)
    u = o.get_deformation()
    K = o.assemble_level(0)
    lv = o.levels[0]
    r = o.F - K @ u
    r[lv.fixedDOFs] = 0
    assert np.linalg.norm(r) / np.linalg.norm(o.F) < 1e-3 * 1.0001
    assert np.all(u[lv.fixedDOFs] == 0)
    # rigid translations are in the null space of K, so the nodal forces K u
    # at the fixed DOFs (the support reactions) cancel the applied load
    react = (K @ u)[lv.fixedDOFs].reshape(-1, 3).sum(axis=0)
    total = o.F.reshape(-1, 3).sum(axis=0)
    assert np.allclose(react, -total, atol=2e-3 * np.abs(total).max())


def test_stress_patch_uniform_strain():
    """A linear displacement field gives the constant Hooke stress at every node."""
    o = _small(L=2, shape=(4, 6, 4), voids=0)
    lv = o.levels[0]
    ny, nx = lv.resY, lv.resX
    lin = lv.nodMapBack
    iy = lin % (ny + 1); ix = (lin // (ny + 1)) % (nx + 1); iz = lin // ((ny + 1) * (nx + 1))
    x, y, z = ix * 1.0, (ny - iy) * 1.0, iz * 1.0          # physical y decreases with iy
    eps = np.array([1e-3, -2e-3, 5e-4, 3e-4, -1e-4, 2e-4])  # exx eyy ezz gyz gzx gxy
    u = np.stack([eps[0] * x + eps[5] * y + eps[4] * z,
                  eps[1] * y + eps[3] * z,
                  eps[2] * z], axis=1)
    o.U = u.ravel()
    nodal, vox = o.get_cartesian_stress()
    sig = G.hooke(1.0, 0.3) @ eps
    assert np.allclose(nodal, sig[None, :], atol=1e-12)
    assert np.allclose(vox, sig[None, :], atol=1e-12)


@pytest.mark.parametrize("dims,ctrl,levels,expect_L,expect_pad", [
    ((37, 42, 64), 10000, 0, 3, (40, 44, 64)),
    ((37, 42, 64), 10000, 4, 4, (40, 48, 64)),
    ((294, 337, 512), 10000, 0, 6, (320, 352, 512)),
    ((373, 428, 650), 10000, 0, 6, (384, 448, 672)),
    ((373, 428, 650), 10000, 7, 7, (384, 448, 704)),
])
def test_level_rule_and_padding(dims, ctrl, levels, expect_L, expect_pad):
    """DiscretizeDesignDomain.m:29-50 on the benchmark resolutions."""
    k = G.level_count(*dims, G.Params(coarsest_resolution_control=ctrl, num_levels=levels))
    assert k + 1 == expect_L
    f = 2 ** k
    assert tuple(-(-n // f) * f for n in dims) == expect_pad


def test_resolution_errors():
    with pytest.raises(G.GMGSError):
        G.level_count(4, 4, 4, G.Params())                 # 64 voxels < 10000
    with pytest.raises(G.GMGSError):
        G.Oracle(np.ones((4, 4, 4), np.int32), G.Params(num_levels=1))
    o = G.Oracle(np.ones((4, 4, 4), np.int32), G.Params(num_levels=2))
    with pytest.raises(G.GMGSError):
        o.apply_boundary_condition([1, 2], np.zeros((0, 4)))
    with pytest.raises(G.GMGSError):
        o.apply_boundary_condition([], [[1, 0, 0, -1]])


def test_load_duplicate_last_wins():
    o = G.Oracle(np.ones((4, 4, 4), np.int32), G.Params(num_levels=2))
    o.apply_boundary_condition([1], [[5, 1, 2, 3], [5, 4, 5, 6]])
    assert o.F[12:15].tolist() == [4.0, 5.0, 6.0]


def test_only_value_one_is_solid():
    vox = np.ones((4, 4, 4), np.int32)
    vox[0, 0, 0] = 2
    lv, L, _ = G.discretize(vox, G.Params(num_levels=2))
    assert lv.numElements == 63


def test_level2_galerkin_matrix_is_fixed_by_the_child_pattern():
    """SetupSolver.m:39-68 with a uniform finest material: a unique level-2
    element's Galerkin matrix depends only on which of its 8 children are
    solid.  The device keeps one matrix per pattern present on that basis."""
    from gmgs import synthetic
    vox = synthetic.sphere_voids(21, 13, 18, 6, 7)
    o = G.Oracle(vox, G.Params(num_levels=3))
    o.setup()
    lv = o.levels[1]
    assert lv.storingState == 2 and len(lv.uniqueElements) > 20
    masks = (lv.elementUpwardMap[lv.uniqueElements] != 0) @ (1 << np.arange(8))
    by_mask = {}
    for k, m in enumerate(masks):
        by_mask.setdefault(int(m), []).append(lv.Ks[1 + k])
    assert len(by_mask) < len(masks)
    for mats in by_mask.values():
        for K in mats[1:]:
            assert np.array_equal(K, mats[0])
    firsts = [m[0] for m in by_mask.values()]
    for i in range(len(firsts)):
        for j in range(i + 1, len(firsts)):
            assert not np.allclose(firsts[i], firsts[j])
