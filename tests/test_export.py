"""Output formats (ExportDataset_3DTSV.m, WrapVoxelFEAmodel.m) and the
compact-to-grid maps they write (DiscretizeDesignDomain.m:68-86)."""
import numpy as np
import pytest

from gmgs import export, synthetic
import gmgs_oracle as G


def test_grid_maps_match_the_oracle_discretisation():
    vox = synthetic.sphere_voids(9, 7, 11, 2, 4)
    fine, _, _ = G.discretize(vox, G.Params(num_levels=2))
    # the oracle pads; map the padded grid
    ele, nod = export.grid_maps(_padded(vox, fine))
    assert np.array_equal(ele - 1, np.asarray(fine.eleMapBack).ravel())     # the oracle keeps 0-based maps
    assert np.array_equal(nod - 1, np.asarray(fine.nodMapBack).ravel())
    assert len(nod) == fine.numNodes


def _padded(vox, fine):
    out = np.zeros((fine.resY, fine.resX, fine.resZ), dtype=np.int32)
    out[:vox.shape[0], :vox.shape[1], :vox.shape[2]] = vox
    return out


def test_carti_format(tmp_path):
    vox = np.zeros((2, 2, 2), dtype=np.int32)
    vox[0, 0, 0] = 1
    vox[1, 1, 1] = 1
    ele, nod = export.grid_maps(vox)
    assert list(ele) == [1, 8]
    assert len(nod) == 15                                 # two corner-sharing cubes
    p = tmp_path / "d.carti"
    stress = np.arange(6 * len(nod), dtype=float).reshape(-1, 6) * 1.5e-3
    export.export_dataset_3dtsv(p, (2, 2, 2), [0, 0, 0], [2.0, 2.5, 3.0], ele, nod, [1, 2],
                                np.array([[15, 0.0, 0.0, -1.0]]), stress)
    lines = p.read_text().splitlines()
    assert lines[0] == "DATASET CARTESIAN_GRID "
    assert lines[1] == "Resolution: 2 2 2"
    assert lines[2] == "LowerBound: 0.000000 0.000000 0.000000"
    assert lines[3] == "UpperBound: 2.000000 2.500000 3.000000"
    assert lines[4] == "ELEMENTS 2 int "
    assert lines[5:7] == ["0", "7"]
    assert lines[7] == "Number of Stress Fields: 1"
    assert lines[8] == "Node Forces: 1"
    assert lines[9] == f"{nod[14] - 1} 0.000000 0.000000 -1.000000"
    assert lines[10] == "Fixed Nodes: 2"
    assert lines[11:13] == [str(nod[0] - 1), str(nod[1] - 1)]
    assert lines[13] == f"Cartesian Stress: {len(nod)}"
    assert lines[14] == "0.000000e+00 1.500000e-03 3.000000e-03 4.500000e-03 6.000000e-03 7.500000e-03"
    assert len(lines) == 14 + len(nod)


def test_wrapped_model_format(tmp_path):
    vox = np.ones((1, 1, 2), dtype=np.int32)
    ele, nod = export.grid_maps(vox)
    p = tmp_path / "w.txt"
    export.wrap_voxel_fea_model(p, (1, 1, 2), ele, nod, [1, 2], np.array([[12, 0.25, 0, -1]]))
    assert p.read_text() == ("domain type: 3D \nresolution: 1 1 2\nvalid elements: 2\n1\n2\n"
                             "fixed position: 2\n1 1 1 1\n2 1 1 1\n"
                             "loading condition: 1\n12 0.250000 0.000000 -1.000000\n")


@pytest.mark.gpu
def test_session_exports(tmp_path):
    from gmgs import Session
    vox = synthetic.sphere_voids(12, 10, 16, 1, 3)
    fixed, loads = synthetic.boundary_conditions(vox, 2)
    s = Session()
    s.voxelizedVolume_ = vox
    s.numLevels_ = 2
    s.fixingCond_, s.loadingCond_ = fixed, loads
    s.GetDeformation()
    s.GetCartesianStress()
    p = s.ExportDataset_3DTSV(str(tmp_path / "d.carti"))
    lines = open(p).read().splitlines()
    assert lines[0] == "DATASET CARTESIAN_GRID "
    n = int(lines[-len(s.cartesianStressField_) - 1].split()[-1])
    assert n == len(s.cartesianStressField_)
    q = s.WrapVoxelFEAmodel(str(tmp_path / "w.txt"))
    assert open(q).read().startswith("domain type: 3D \nresolution: ")
