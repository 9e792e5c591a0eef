"""Voxeliser: the oracle restatement pinned by the reference README's DOF
counts (README.md:29-41) and the reference's own demo boundary-condition
files, and the GPU voxeliser (gmgs_voxelize_mesh) bit-identical to the
oracle on synthetic closed meshes."""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

from gmgs import synthetic
import gmgs_oracle as G
import voxelize as V

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import make_voxelize_golden as MK   # noqa: E402

REFERENCE = MK.reference_dir()      # $GMGS_REFERENCE_DIR: a checkout with the reference's meshes, or None


def _golden():
    return json.loads((GOLDEN / "voxelize_dofs.json").read_text())


def _occupancy(name):
    z = np.load(GOLDEN / f"{name}64_occupancy.npz")
    shape = tuple(int(s) for s in z["shape"])
    bits = np.unpackbits(z["bits"])[: int(np.prod(shape))]
    return bits.reshape(shape, order="F").astype(np.int32)


def test_readme_dof_counts():
    """9 of the 10 README DOF counts are reproduced exactly.  The tenth
    (kitten 84x73x128, 929,961) contradicts the reference's own demo fixture
    for that model: its largest loaded node id, 289,654, sits at the top of
    the part, next to the 289,656 nodes found here, while 929,961 DOFs would
    mean 309,987 nodes (the other rows are 3x the node count)."""
    g = _golden()
    for model, rows in g.items():
        for res, r in rows.items():
            assert r["dofs"] == 3 * r["nodes"]
            assert r["bc_fixed_max_id"] <= r["nodes"] and r["bc_load_max_id"] <= r["nodes"]
            if (model, res) == ("kitten", "128"):
                assert r["dofs"] != r["readme_dofs"]
                assert r["nodes"] - r["bc_load_max_id"] <= 2
            else:
                assert r["dofs"] == r["readme_dofs"], (model, res)
    # the top-most node is loaded in the kitten demos: the numbering is the reference's
    for res in ("256", "512", "650"):
        assert g["kitten"][res]["bc_load_max_id"] == g["kitten"][res]["nodes"]


@pytest.mark.parametrize("name,dofs", [("kitten", 120198), ("parts", 141744)])
def test_golden_occupancy_discretizes_to_readme_dofs(name, dofs):
    vol = _occupancy(name)
    fine, _, _ = G.discretize(vol, G.Params())
    assert 3 * fine.numNodes == dofs


@pytest.mark.skipif(REFERENCE is None or not (REFERENCE / "data" / "kitten.ply").exists(),
                    reason="reference meshes not present (set GMGS_REFERENCE_DIR)")
@pytest.mark.parametrize("name", ["kitten", "parts"])
def test_oracle_reproduces_golden_from_the_reference_mesh(name):
    vol, _, grid = V.create_voxelized_model(REFERENCE / "data" / f"{name}.ply", 64)
    assert np.array_equal(vol, _occupancy(name))
    assert list(grid) == _golden()[name]["64"]["grid_nx_ny_nz"]


def test_colon_semantics():
    assert len(V.colon(0.0, 0.1, 1.0)) == 11          # 0:0.1:1 has 11 elements in MATLAB
    v = V.colon(0.5, 1.0, 9.5)
    assert np.array_equal(v, np.arange(0.5, 10.0, 1.0))
    assert len(V.colon(1.0, 1.0, 0.5)) == 0


def _inside_box(pts, lo, hi):
    return np.all((pts > lo) & (pts < hi), axis=-1)


def test_oracle_box_mesh():
    """An axis-aligned box (12 facets): every voxel centre strictly inside is
    solid and every one outside is void."""
    lo, hi = np.array([0.3, 0.2, 0.1]), np.array([2.3, 1.45, 3.6])
    c = np.array([[x, y, z] for z in (lo[2], hi[2]) for y in (lo[1], hi[1]) for x in (lo[0], hi[0])])
    f = np.array([[0, 2, 1], [1, 2, 3], [4, 5, 6], [5, 7, 6], [0, 1, 4], [1, 5, 4],
                  [2, 6, 3], [3, 6, 7], [0, 4, 2], [2, 4, 6], [1, 3, 5], [3, 7, 5]])
    nx, ny, nz, mesh = V.adapt_for_voxelize(c, f, 32)
    vol = V.voxelize(nx, ny, nz, mesh)                 # (y, x, z), before the flip
    assert vol.all()                                   # voxel centres sit inside by construction


def test_oracle_blob_matches_analytic_interior():
    """Voxel centres well inside / outside a closed blob are classified as such."""
    v, f = synthetic.blob_mesh(seed=3)
    nx, ny, nz, mesh = V.adapt_for_voxelize(v, f, 40)
    vol = V.voxelize(nx, ny, nz, mesh)
    assert 0 < vol.sum() < vol.size
    # the blob is star-shaped about its centre: a centre far inside the hull is solid
    assert vol[vol.shape[0] // 2, vol.shape[1] // 2, vol.shape[2] // 2]
    assert not vol[0, 0, 0] and not vol[-1, -1, -1]


MESHES = {
    "blob_s1": lambda: synthetic.blob_mesh(seed=1),
    "blob_s7_fine": lambda: synthetic.blob_mesh(n_lat=40, n_lon=80, seed=7, amp=0.35),
    "torus": lambda: synthetic.torus_mesh(seed=2),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MESHES))
@pytest.mark.parametrize("res", [24, 64, 97])
def test_gpu_voxelizer_bit_identical_to_oracle(name, res):
    from gmgs import mesh as M
    v, f = MESHES[name]()
    ref, _, grid = V.create_voxelized_model_from_arrays(v, f, res)
    occ, ele = M.voxelize(v, f, res)
    assert occ.shape == ref.shape
    assert np.array_equal(occ, ref)
    ext = v.max(axis=0) - v.min(axis=0)
    assert np.allclose(ele, ext / np.array(grid, dtype=float))


@pytest.mark.gpu
def test_gpu_voxelizer_rejects_bad_input():
    from gmgs import mesh as M
    from gmgs.solver import GMGSError
    v, f = synthetic.blob_mesh(seed=1)
    with pytest.raises(GMGSError):
        M.voxelize(v, f + len(v), 32)
    with pytest.raises(GMGSError):
        M.voxelize(v, f, 0)


def _demo(name):
    vol = _occupancy(name)
    bc = np.load(GOLDEN / f"{name}64_demo_bc.npz")
    ele = np.array(_golden()[name]["64"]["ele_size"])
    return vol, bc["fixed"], bc["loads"], ele


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["kitten", "parts"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_reference_demo_64_matches_oracle(name, precision):
    """The reference's own demo inputs (Demo.m:15-18 and the parts variant):
    the 64-resolution voxelisation of data/<name>.ply with its demo boundary
    conditions, default controls (omega 0.4, tol 1e-3, the level rule)."""
    from gmgs import Solver
    vol, fixed, loads, ele = _demo(name)
    o = G.Oracle(vol, G.Params(), ele_size=ele)
    o.apply_boundary_condition(fixed, loads)
    u_ref = o.get_deformation()
    s = Solver(vol, ele_size=ele, precision=precision)
    s.set_bc(fixed, loads)
    u = s.solve(with_history=True)
    assert s.status == 0
    assert s.iterations == o.iterations
    tol = 1e-6 if precision == "fp64" else 1e-5
    assert np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref) < tol
    h_ref = np.array([h[2] for h in o.iterationHist])
    htol = 1e-8 if precision == "fp64" else 1e-4
    assert np.max(np.abs(s.history[:, 2] - h_ref) / h_ref) < htol
    if precision == "fp64":
        nodal_ref, _ = o.get_cartesian_stress()
        nodal, _ = s.stress()
        assert np.linalg.norm(nodal - nodal_ref) / np.linalg.norm(nodal_ref) < 1e-6


@pytest.mark.gpu
def test_session_mesh_overload(tmp_path):
    """Session.CreateVoxilizedModel(file, res) voxelises a .ply like the reference."""
    from gmgs import Session
    v, f = synthetic.blob_mesh(seed=5)
    p = tmp_path / "blob.ply"
    with open(p, "w") as fh:
        fh.write(f"ply\nformat ascii 1.0\nelement vertex {len(v)}\nproperty float x\nproperty float y\n"
                 f"property float z\nelement face {len(f)}\nproperty list uchar int vertex_indices\nend_header\n")
        for x in v:
            fh.write(f"{float(x[0])!r} {float(x[1])!r} {float(x[2])!r}\n")
        for t in f:
            fh.write(f"3 {t[0]} {t[1]} {t[2]}\n")
    s = Session()
    vol = s.CreateVoxilizedModel(str(p), 40)
    ref, _, grid = V.create_voxelized_model(p, 40)
    assert np.array_equal(vol, ref)
    assert np.allclose(s.eleSize_, (v.max(0) - v.min(0)) / np.array(grid, dtype=float))
