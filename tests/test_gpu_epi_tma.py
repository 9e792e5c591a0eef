"""The streaming kernels of the mixed path with their inputs staged into
shared memory by TMA (fine.cu, k_fine<MODE, DEF, STG>) against the same
kernels loading them per thread into registers:

* the CG update's per-node operands (r and x, high and low parts, q, p; one
  32 x 8 x 3 box per array and plane, 128-byte swizzle), off with
  GMGS_EPI_TMA=0;
* every mode's field inputs with the one-node halo (r and omega/diag, q, z,
  p; one 40 x 10 x 3 box per array and plane, unswizzled), off with
  GMGS_FIELD_TMA=0.

Both read the same values and round the same operations in the same order,
so the mixed solve is bit-identical; the models have ragged extents (boxes
that reach past the grid's edge read zeros), tile planes without a node to
update inside a CTA's z-chunk, coarse levels with per-element matrices and a
density field.
"""
import numpy as np
import pytest

from gmgs import Solver, synthetic

pytestmark = pytest.mark.gpu

def _stepped():
    """A block whose upper half keeps only a slab x < 9: the column tiles over
    x >= 9 have solid nodes in their lower planes and none above, so a CTA's
    z-chunk holds planes where no thread has a node to update."""
    vox = np.ones((20, 30, 40), dtype=np.int32)     # (y, x, z)
    vox[:, 9:, 20:] = 0
    return np.asfortranarray(vox)


CASES = {
    "stepped_L3": (_stepped, 3, None),
    "ragged_L3": (lambda: synthetic.sphere_voids(21, 13, 18, 6, 7), 3, None),
    "block42_L5": (lambda: synthetic.make("block42_fp64")[0], 5, None),
    "density_L3": (lambda: synthetic.sphere_voids(28, 24, 32, 2, 5), 3, (0.3, 1.0)),
    "block84_L4": (lambda: synthetic.make("block84_adjoint")[0], 4, (0.2, 1.0)),
}


def _solve(vox, L, rho):
    fixed, loads = synthetic.boundary_conditions(vox, L)
    s = Solver(vox, omega=0.4, num_levels=L, precision="mixed")
    s.set_bc(fixed, loads)
    if rho is not None:
        s.set_density(rho, 3.0)
    u = s.solve()
    its, rr = s.iterations, s.relres
    s.close()
    return u, its, rr


@pytest.mark.parametrize("name", list(CASES))
def test_tma_staged_inputs_bit_identical(name, monkeypatch):
    build, L, rr = CASES[name]
    vox = build()
    rho = synthetic.density(int(vox.sum()), rr, 5) if rr else None
    switches = ("GMGS_EPI_TMA", "GMGS_FIELD_TMA")
    for k in switches:
        monkeypatch.setenv(k, "0")
    u0, it0, r0 = _solve(vox, L, rho)
    for k in switches:
        monkeypatch.delenv(k)
    u1, it1, r1 = _solve(vox, L, rho)
    assert it1 == it0
    assert r1 == r0
    assert np.array_equal(u1, u0)
