"""Every failure status of the C ABI, made on the host (bad inputs), with the
message the reference prints where it has one, and the handle still usable
or destroyable afterwards.

Reference cases: ApplyBoundaryCondition.m:12 (no loads) and :22 (no
fixings) abort with error(); SetupSolver.m:19-21 aborts on too few levels;
SetupSolver.m:259 ignores chol's failure flag, which the library reports as
GMGS_ERR_NOT_SPD instead of iterating on a broken factor.  No GPU fault is
involved: every failure comes from the inputs.
"""
import ctypes as C

import numpy as np
import pytest

from gmgs import GMGSError, Solver, _lib, synthetic

pytestmark = pytest.mark.gpu


def _model():
    vox = synthetic.sphere_voids(14, 12, 16, 3, 21)
    fixed, loads = synthetic.boundary_conditions(vox, 3)
    return vox, fixed, loads


def _last_error(s):
    return s._lib.gmgs_last_error(s.handle).decode()


def _solves_after(s, fixed, loads):
    s.set_bc(fixed, loads)
    u = s.solve()
    assert s.status == _lib.OK and np.all(np.isfinite(u)) and np.abs(u).max() > 0


def test_no_loads_then_usable():
    vox, fixed, loads = _model()
    s = Solver(vox, num_levels=3)
    with pytest.raises(GMGSError) as e:
        s.set_bc(fixed, np.zeros((0, 4)))
    assert e.value.status == _lib.ERR_NO_LOADS
    assert "No Loads! Unable to Perform Static FEA!" in _last_error(s)
    # nothing was applied: a solve now is a call-order error, not a crash
    assert s._lib.gmgs_solve(s.handle, None, None, None, None) == _lib.ERR_STATE
    _solves_after(s, fixed, loads)
    s.close()


def test_no_fixings_then_usable():
    vox, fixed, loads = _model()
    s = Solver(vox, num_levels=3)
    with pytest.raises(GMGSError) as e:
        s.set_bc(np.zeros(0, np.int32), loads)
    assert e.value.status == _lib.ERR_NO_FIXINGS
    assert "No Constraints! Unable to Perform Static FEA!" in _last_error(s)
    _solves_after(s, fixed, loads)
    s.close()


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_nonfinite_load_then_usable(bad):
    vox, fixed, loads = _model()
    s = Solver(vox, num_levels=3)
    broken = np.array(loads, dtype=np.float64).reshape(-1, 4).copy()
    broken[len(broken) // 2, 3] = bad
    with pytest.raises(GMGSError) as e:
        s.set_bc(fixed, broken)
    assert e.value.status == _lib.ERR_NONFINITE
    assert "non-finite load" in _last_error(s)
    _solves_after(s, fixed, loads)
    s.close()


def test_out_of_range_node_ids():
    vox, fixed, loads = _model()
    s = Solver(vox, num_levels=3)
    nn = s.num_nodes(1)
    bad_fixed = np.array(fixed, np.int32).copy()
    bad_fixed[0] = nn + 1
    with pytest.raises(GMGSError) as e:
        s.set_bc(bad_fixed, loads)
    assert e.value.status == _lib.ERR_INVALID_ARGUMENT
    bad_loads = np.array(loads, dtype=np.float64).reshape(-1, 4).copy()
    bad_loads[0, 0] = 0            # ids are 1-based
    with pytest.raises(GMGSError) as e:
        s.set_bc(fixed, bad_loads)
    assert e.value.status == _lib.ERR_INVALID_ARGUMENT
    _solves_after(s, fixed, loads)
    s.close()


def test_all_void_occupancy():
    vox = np.zeros((16, 16, 16), np.int32)
    with pytest.raises(GMGSError) as e:
        Solver(vox, num_levels=3)
    assert e.value.status == _lib.ERR_NO_SOLID
    assert b"no solid voxel" in _lib.load().gmgs_last_error(None)


def test_every_node_fixed_is_not_spd_then_usable():
    """Fixing every node leaves the coarsest level without a free DOF: the
    coarsest factorisation (SetupSolver.m:257-259) has nothing to factor.
    The failed setup is retried by the next solve."""
    vox, fixed, loads = _model()
    s = Solver(vox, num_levels=3)
    every = np.arange(1, s.num_nodes(1) + 1, dtype=np.int32)
    s.set_bc(every, loads)
    st = s._lib.gmgs_solve(s.handle, None, None, None, None)
    assert st == _lib.ERR_NOT_SPD
    assert "no free DOFs on the coarsest level" in _last_error(s)
    # a stress call has no solution to work on
    nodal = np.zeros((s.num_nodes(1), 6))
    assert s._lib.gmgs_stress(s.handle, nodal.ctypes.data_as(C.POINTER(C.c_double)), None) == _lib.ERR_NO_SOLUTION
    _solves_after(s, fixed, loads)
    s.close()


def test_floating_piece_never_reports_success():
    """A second solid piece with no fixed node makes K singular.  The
    reference factors it anyway (SetupSolver.m:259 ignores chol's flag); the
    library either refuses the factorisation (GMGS_ERR_NOT_SPD) or stops
    without convergence, but never returns GMGS_OK, and the handle is still
    destroyable."""
    vox = np.zeros((12, 12, 40), np.int32)
    vox[:, :, :12] = 1              # anchored on z = 0
    vox[:, :, 28:] = 1              # floats: a 16-voxel gap on every level
    L = 3
    fixed, _ = synthetic.boundary_conditions(vox[:, :, :12], L)
    # load the floating piece's top face
    _, loads = synthetic.boundary_conditions(vox, L)
    s = Solver(vox, num_levels=L, max_it=40)
    s.set_bc(fixed, loads)
    st = s._lib.gmgs_solve(s.handle, None, None, None, None)
    assert st in (_lib.ERR_NOT_SPD, _lib.ERR_MAX_ITERATIONS, _lib.ERR_NONFINITE), st
    s.close()


def test_too_few_levels():
    with pytest.raises(GMGSError) as e:
        Solver(np.ones((8, 8, 8), np.int32), num_levels=1)
    assert e.value.status == _lib.ERR_RESOLUTION


def test_gradient_needs_density_and_solution():
    vox, fixed, loads = _model()
    s = Solver(vox, num_levels=3)
    s.set_bc(fixed, loads)
    g = np.zeros(s.num_elements(1))
    gp = g.ctypes.data_as(C.POINTER(C.c_double))
    assert s._lib.gmgs_grad(s.handle, None, gp) == _lib.ERR_STATE
    s.set_density(np.full(s.num_elements(1), 0.5), 3.0)
    assert s._lib.gmgs_grad(s.handle, None, gp) == _lib.ERR_NO_SOLUTION
    s.solve()
    assert s._lib.gmgs_grad(s.handle, None, gp) == _lib.OK
    assert np.all(g <= 0)
    s.close()
