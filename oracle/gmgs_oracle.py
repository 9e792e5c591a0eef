"""CPU oracle for the GMGS-3D multigrid-preconditioned CG elasticity solve.

TEST INFRASTRUCTURE ONLY.  This module is the checker that the CUDA library
(`libgmgs.so`) is compared against, and the timed CPU baseline of the bench.
Nothing in the product path imports it.

It restates, in NumPy/SciPy FP64, the MATLAB code of GMGS-3D step by step:

* element math:     src/common/SetupStiffnessMatrix.m:1-23,
                    src/common/ElementElasticityMatrix.m:11-24,
                    src/common/ElementStrainMatrix.m:3-94,
                    src/common/GaussianIntegral.m:11-17,
                    src/common/ShapeFunction.m:16-23,
                    src/common/DeShapeFunction.m:3-22
* discretisation:   src/common/DiscretizeDesignDomain.m:29-116
* hierarchy:        src/kernel/BuildingMeshHierarchy.m:8-142
* solver setup:     src/kernel/SetupSolver.m:9-259,
                    src/kernel/DirectlyAssembleStifnessMatrix.m:24-34
* transfer tables:  src/kernel/Operator4MultiGridRestrictionAndInterpolation.m:4-115,
                    src/kernel/SubEleNodMat.m:3-11 (generated from the trilinear
                    rule instead of being transcribed)
* operators:        src/kernel/AtX.m, JacobiSmoother.m, RestrictResidual.m,
                    InterpolationDeviation.m, Vcycle.m, CG_solver.m
* boundary:         src/common/ApplyBoundaryCondition.m:7-23
* stress:           src/kernel/GetCartesianStress.m:11-73

Indices follow the MATLAB layout (column-major (y, x, z) grids, node-major
interleaved DOFs) and are 0-based inside this module; only the boundary
condition input uses the reference's 1-based node ids.

Parity unpinned: the reference is MATLAB, which cannot run in this
environment, and the reference ships no tests, golden vectors or fixtures for
this path.  The restatement is pinned instead by known-answer checks in
tests/: the element matrix against an exact symbolic integration, the
Galerkin identity P^T K P against explicit assembly
(DirectlyAssembleStifnessMatrix.m:7-23), rigid-body modes, and the trilinear
transfer tables' defining properties.

Extension beyond the reference (marked where used): per-voxel stiffness
scaling rho^p on the finest level and the adjoint gradient of compliance or
of a linear displacement functional.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla

# GaussianIntegral.m:11-16 writes the Gauss abscissa with 15 digits; keep it.
GAUSS_ABSCISSA = 0.577350269189626


class GMGSError(RuntimeError):
    """Raised where the reference calls error() or warns and returns."""


@dataclass
class Params:
    """Solver controls; defaults are GlobalVariables.m:3-23."""
    tol: float = 1.0e-3
    max_it: int = 20000
    omega: float = 0.4
    youngs_modulus: float = 1.0
    poisson_ratio: float = 0.3
    coarsest_resolution_control: int = 10000
    num_levels: int = 0          # 0 -> the reference's rule (DiscretizeDesignDomain.m:33-41)


# --------------------------------------------------------------------------
# element math
# --------------------------------------------------------------------------
def hooke(E: float, nu: float) -> np.ndarray:
    """Isotropic 6x6 elasticity matrix, ElementElasticityMatrix.m:11-24."""
    c1 = (1.0 + nu) * (1.0 - 2.0 * nu)
    c2 = 2.0 * (1.0 + nu)
    S = np.zeros((6, 6))
    S[0, 0] = E * (1.0 - nu) / c1
    S[0, 1] = E * nu / c1
    S[0, 2] = S[0, 1]
    S[1, 0] = S[0, 1]; S[1, 1] = S[0, 0]; S[1, 2] = S[1, 0]
    S[2, 0] = S[0, 2]; S[2, 1] = S[1, 2]; S[2, 2] = S[1, 1]
    S[3, 3] = E / c2
    S[4, 4] = S[3, 3]
    S[5, 5] = S[4, 4]
    return S


# parametric node signs of the 8-node hex (ShapeFunction.m:16-23)
_NODE_SIGNS = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                        [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=float)


def gauss_points():
    """2x2x2 Gauss rule in the reference's point order, GaussianIntegral.m:11-17."""
    g = GAUSS_ABSCISSA
    s = g * _NODE_SIGNS[:, 0]
    t = g * _NODE_SIGNS[:, 1]
    p = g * _NODE_SIGNS[:, 2]
    w = np.ones(8)
    return s, t, p, w


def shape_functions(s, t, p) -> np.ndarray:
    """N (npts x 8), ShapeFunction.m:15-23."""
    s = np.asarray(s, float).ravel(); t = np.asarray(t, float).ravel(); p = np.asarray(p, float).ravel()
    sg = _NODE_SIGNS
    return 0.125 * (1 + s[:, None] * sg[None, :, 0]) * (1 + t[:, None] * sg[None, :, 1]) \
        * (1 + p[:, None] * sg[None, :, 2])


def shape_derivatives(s, t, p) -> np.ndarray:
    """dShape (3*npts x 8): rows 3g..3g+2 are d/ds, d/dt, d/dp; DeShapeFunction.m:3-22."""
    s = np.asarray(s, float).ravel(); t = np.asarray(t, float).ravel(); p = np.asarray(p, float).ravel()
    sg = _NODE_SIGNS
    fs = 1 + s[:, None] * sg[None, :, 0]
    ft = 1 + t[:, None] * sg[None, :, 1]
    fp = 1 + p[:, None] * sg[None, :, 2]
    out = np.zeros((3 * len(s), 8))
    out[0::3] = 0.125 * sg[None, :, 0] * ft * fp
    out[1::3] = 0.125 * sg[None, :, 1] * fs * fp
    out[2::3] = 0.125 * sg[None, :, 2] * fs * ft
    return out


def strain_matrix(dshape: np.ndarray, invJ: np.ndarray) -> np.ndarray:
    """B (48 x 24); rows [exx eyy ezz gyz gzx gxy] per Gauss point, ElementStrainMatrix.m:3-94."""
    der = invJ @ dshape
    B = np.zeros((48, 24))
    for g in range(8):
        dx, dy, dz = der[3 * g], der[3 * g + 1], der[3 * g + 2]
        for k in range(8):
            r, c = 6 * g, 3 * k
            B[r + 0, c + 0] = dx[k]
            B[r + 1, c + 1] = dy[k]
            B[r + 2, c + 2] = dz[k]
            B[r + 3, c + 1] = dz[k]; B[r + 3, c + 2] = dy[k]
            B[r + 4, c + 0] = dz[k]; B[r + 4, c + 2] = dx[k]
            B[r + 5, c + 0] = dy[k]; B[r + 5, c + 1] = dx[k]
    return B


def element_node_coords(ele_size) -> np.ndarray:
    """Coordinates of the 8 nodes of one element relative to node 1.

    The reference evaluates the Jacobian on the first solid element
    (SetupStiffnessMatrix.m:11-13).  Its local node 1 sits at (-x,-y,-z) since
    node y-indices grow towards smaller physical y (DiscretizeDesignDomain.m:96).
    """
    dx, dy, dz = (float(v) for v in ele_size)
    return (_NODE_SIGNS + 1.0) * 0.5 * np.array([dx, dy, dz])


def _jacobians(ele_size):
    s, t, p, w = gauss_points()
    dshape = shape_derivatives(s, t, p)
    X = element_node_coords(ele_size)
    detJ = np.zeros(8)
    invJ = np.zeros((24, 24))
    for g in range(8):
        J = dshape[3 * g:3 * g + 3] @ X
        detJ[g] = np.linalg.det(J)
        invJ[3 * g:3 * g + 3, 3 * g:3 * g + 3] = np.linalg.inv(J)
    return dshape, detJ, invJ, w


def element_stiffness(E: float, nu: float, ele_size=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Ke0 = B^T (D w) B, SetupStiffnessMatrix.m:4-22."""
    dshape, detJ, invJ, w = _jacobians(ele_size)
    B = strain_matrix(dshape, invJ)
    D = np.kron(np.eye(8), hooke(E, nu))
    wgt = np.repeat(w * detJ, 6)
    return B.T @ (D * wgt[None, :]) @ B


def outer_interpolation() -> np.ndarray:
    """OTP = inv(sFM) (48x48), GetCartesianStress.m:44-73: Gauss point -> node extrapolation."""
    s, t, p, _ = gauss_points()
    N = shape_functions(s, t, p)
    return np.linalg.inv(np.kron(N, np.eye(6)))


def stress_matrices(E: float, nu: float, ele_size=(1.0, 1.0, 1.0)):
    """(M_nodal 48x24, M_gauss 48x24): nodal = OTP D B, Gauss-point = D B (GetCartesianStress.m:19-36)."""
    dshape, _, invJ, _ = _jacobians(ele_size)
    B = strain_matrix(dshape, invJ)
    D = np.kron(np.eye(8), hooke(E, nu))
    DB = D @ B
    return outer_interpolation() @ DB, DB


# --------------------------------------------------------------------------
# transfer tables, generated from the trilinear rule
# --------------------------------------------------------------------------
# Local corner of element node k (0-based) as (y-offset, x-offset, z-offset) in
# node-index units: node 1 = (iy+1, ix, iz), 2 = (iy+1, ix+1, iz), 3 = (iy, ix+1, iz),
# 4 = (iy, ix, iz), 5..8 the same at iz+1 (DiscretizeDesignDomain.m:80).
LOCAL_CORNERS = np.array([[1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 0],
                          [1, 0, 1], [1, 1, 1], [0, 1, 1], [0, 0, 1]])


def trilinear_node_table() -> np.ndarray:
    """RI (27 x 8): weight of coarse corner k at fine node m of a span-2 block.

    Fine node m = a + 3b + 9c enumerates the 3x3x3 block column-major over
    (y, x, z) like BuildingMeshHierarchy.m:49-50; the values are those of
    Operator4MultiGridRestrictionAndInterpolation.m:4-31 ('inNODE', span 2).
    """
    RI = np.zeros((27, 8))
    for m in range(27):
        a, b, c = m % 3, (m // 3) % 3, m // 9
        for k in range(8):
            cy, cx, cz = 2 * LOCAL_CORNERS[k]
            RI[m, k] = (max(0.0, 1 - abs(a - cy) / 2) * max(0.0, 1 - abs(b - cx) / 2)
                        * max(0.0, 1 - abs(c - cz) / 2))
    return RI


def sub_element_nodes() -> np.ndarray:
    """(8 x 8) block-node ids (0-based) of the 8 local nodes of each child; SubEleNodMat.m:3-11.

    Child j = dy + 2 dx + 4 dz follows the column-major child order of
    BuildingMeshHierarchy.m:45-46.
    """
    out = np.zeros((8, 8), dtype=np.int64)
    for j in range(8):
        dy, dx, dz = j % 2, (j // 2) % 2, j // 4
        for k in range(8):
            a = dy + LOCAL_CORNERS[k, 0]
            b = dx + LOCAL_CORNERS[k, 1]
            c = dz + LOCAL_CORNERS[k, 2]
            out[j, k] = a + 3 * b + 9 * c
    return out


def node_dofs(nodes: np.ndarray) -> np.ndarray:
    """(..., 8) node ids -> (..., 24) interleaved DOF ids [n1x n1y n1z n2x ...] (SetupSolver.m:13-15)."""
    nodes = np.asarray(nodes, dtype=np.int64)
    return (3 * nodes[..., :, None] + np.arange(3)).reshape(*nodes.shape[:-1], 24)


# --------------------------------------------------------------------------
# mesh hierarchy
# --------------------------------------------------------------------------
@dataclass
class Level:
    resY: int
    resX: int
    resZ: int
    eleSize: np.ndarray
    eleMapBack: np.ndarray = None          # 0-based linear (y,x,z) indices of solid elements
    eleMapForward: np.ndarray = None       # length ny*nx*nz, 1-based compact id, 0 = void
    nodMapBack: np.ndarray = None          # 0-based linear node indices of solid nodes (own grid)
    eNodMat: np.ndarray = None             # (ne, 8) compact node ids
    eDofMat: np.ndarray = None             # (ne, 24)
    numElements: int = 0
    numNodes: int = 0
    # coarse levels only
    elementUpwardMap: np.ndarray = None    # (ne, 8) finer compact ids, 1-based, 0 = void
    transferMat: np.ndarray = None         # (27, ne) intermediate node ids
    transferMatCoeffi: np.ndarray = None   # (nInter,)
    solidNodeMapCoarser2Finer: np.ndarray = None
    intermediateNumNodes: int = 0
    # solver data
    storingState: int = 0
    Ke: np.ndarray = None
    Ks: np.ndarray = None                  # state 0: (24,24); 1: (ne,24,24); 2: (1+nu,24,24)
    uniqueElements: np.ndarray = None      # state 2, 0-based compact
    universalElements: np.ndarray = None
    diagK: np.ndarray = None
    fixedDOFs: np.ndarray = None
    freeDOFs: np.ndarray = None
    eleScale: np.ndarray = None            # extension: per-element rho^p on the finest level

    @property
    def numDOFs(self) -> int:
        return 3 * self.numNodes


def _element_nodes_global(lin: np.ndarray, ny: int, nx: int) -> np.ndarray:
    """Global node ids (own grid) of the 8 nodes of elements with linear index `lin`."""
    ey = lin % ny
    ex = (lin // ny) % nx
    ez = lin // (ny * nx)
    base = (ey + 1) + (ny + 1) * (ex + (nx + 1) * ez)
    s = (ny + 1) * (nx + 1)
    offs = np.array([0, ny + 1, ny, -1, s, s + ny + 1, s + ny, s - 1], dtype=np.int64)
    return base[:, None].astype(np.int64) + offs[None, :]


def _finish_level(lv: Level) -> None:
    ny, nx = lv.resY, lv.resX
    glob = _element_nodes_global(lv.eleMapBack, ny, nx)
    lv.nodMapBack = np.unique(glob)
    lv.numNodes = len(lv.nodMapBack)
    lv.eNodMat = np.searchsorted(lv.nodMapBack, glob)
    lv.eDofMat = node_dofs(lv.eNodMat)


def level_count(nely: int, nelx: int, nelz: int, params: Params) -> int:
    """Number of 2x coarsenings k (numLevels = k + 1), DiscretizeDesignDomain.m:29-41."""
    if params.num_levels:
        if params.num_levels < 2:
            raise GMGSError("There is no sufficient resolution to invoke GMGS!")
        return params.num_levels - 1
    ctrl = params.coarsest_resolution_control
    num = nelx * nely * nelz
    if num < ctrl:
        raise GMGSError("There is no Sufficient Resolution to Build Mesh Hierarchy!")
    k = 0
    while num >= ctrl:
        k += 1
        num = nelx / 2 ** k * nely / 2 ** k * nelz / 2 ** k
    return k


def discretize(voxels: np.ndarray, params: Params, ele_size=(1.0, 1.0, 1.0)):
    """Finest level + level count, DiscretizeDesignDomain.m:29-116.

    `voxels` is the (ny, nx, nz) int array (MATLAB's voxelizedVolume_);
    only the value 1 is solid (DiscretizeDesignDomain.m:68).
    Returns (finest Level, numLevels, numNod2Eles).
    """
    voxels = np.asarray(voxels)
    nely, nelx, nelz = voxels.shape
    k = level_count(nely, nelx, nelz, params)
    f = 2 ** k
    ny, nx, nz = (-(-nely // f)) * f, (-(-nelx // f)) * f, (-(-nelz // f)) * f
    padded = np.zeros((ny, nx, nz), dtype=np.int32)
    padded[:nely, :nelx, :nelz] = voxels
    lv = Level(ny, nx, nz, np.asarray(ele_size, float))
    lv.eleMapBack = np.flatnonzero(padded.ravel(order="F") == 1).astype(np.int64)
    lv.numElements = len(lv.eleMapBack)
    if lv.numElements == 0:
        raise GMGSError("no solid voxels")
    lv.eleMapForward = np.zeros(nx * ny * nz, dtype=np.int64)
    lv.eleMapForward[lv.eleMapBack] = np.arange(1, lv.numElements + 1)
    _finish_level(lv)
    numNod2Eles = np.bincount(lv.eNodMat.ravel(), minlength=lv.numNodes).astype(float)
    return lv, k + 1, numNod2Eles


def build_coarse_level(fine: Level) -> Level:
    """One step of BuildingMeshHierarchy.m:11-141 (span 2)."""
    ny, nx, nz = fine.resY // 2, fine.resX // 2, fine.resZ // 2
    lv = Level(ny, nx, nz, fine.eleSize * 2)
    # 3.1 children of every coarse element, column-major child order (dy, dx, dz)
    F = fine.eleMapForward.reshape((2 * ny, 2 * nx, 2 * nz), order="F")
    up = F.reshape((2, ny, 2, nx, 2, nz), order="F").transpose(5, 3, 1, 4, 2, 0).reshape(-1, 8)
    unempty = np.flatnonzero(up.sum(axis=1) > 0)
    # 3.2 intermediate fine nodes: 3x3x3 blocks of non-empty coarse elements
    gy = unempty % ny
    gx = (unempty // ny) % nx
    gz = unempty // (ny * nx)
    m = np.arange(27)
    a, b, c = m % 3, (m // 3) % 3, m // 9
    fny, fnx = 2 * ny + 1, 2 * nx + 1
    blk = ((2 * gy[None, :] + a[:, None]) + fny * ((2 * gx[None, :] + b[:, None])
                                                   + fnx * (2 * gz[None, :] + c[:, None])))
    inter = np.unique(blk)
    lv.intermediateNumNodes = len(inter)
    lv.transferMat = np.searchsorted(inter, blk)
    lv.transferMatCoeffi = np.bincount(lv.transferMat.ravel(), minlength=len(inter)).astype(float)
    pos = np.searchsorted(inter, fine.nodMapBack)
    assert np.all(inter[pos] == fine.nodMapBack)
    lv.solidNodeMapCoarser2Finer = pos
    # 3.3 solid (non-empty) coarse elements
    lv.eleMapBack = unempty.astype(np.int64)
    lv.numElements = len(unempty)
    lv.eleMapForward = np.zeros(nx * ny * nz, dtype=np.int64)
    lv.eleMapForward[unempty] = np.arange(1, lv.numElements + 1)
    lv.elementUpwardMap = up[unempty]
    _finish_level(lv)
    return lv


# --------------------------------------------------------------------------
# the solver
# --------------------------------------------------------------------------
class Oracle:
    """One GMGS-3D session: model, boundary conditions, setup, solve, stress."""

    def __init__(self, voxels, params: Params | None = None, ele_size=(1.0, 1.0, 1.0)):
        self.params = params or Params()
        fine, self.numLevels, self.numNod2Eles = discretize(voxels, self.params, ele_size)
        self.levels = [fine]
        self.F = None
        self.U = None
        self.iterationHist = []
        self.rho = None
        self.penal = 3.0
        self._setup_done = False

    # ---------------- boundary conditions (ApplyBoundaryCondition.m:7-23)
    def apply_boundary_condition(self, fixing_nodes, loading):
        lv = self.levels[0]
        loading = np.asarray(loading, float).reshape(-1, 4)
        fixing_nodes = np.asarray(fixing_nodes).ravel()
        if loading.shape[0] == 0:
            raise GMGSError("No Loads! Unable to Perform Static FEA!")
        if fixing_nodes.size == 0:
            raise GMGSError("No Constraints! Unable to Perform Static FEA!")
        F = np.zeros((lv.numNodes, 3))
        ids = loading[:, 0].astype(np.int64) - 1
        F[ids] = loading[:, 1:4]        # assignment: a later duplicate wins
        self.F = F.reshape(-1)
        fixed = 3 * (fixing_nodes.astype(np.int64) - 1)
        fixed = (fixed[:, None] + np.arange(3)).reshape(-1)
        lv.fixedDOFs = fixed
        lv.freeDOFs = np.setdiff1d(np.arange(lv.numDOFs), fixed)

    # ---------------- extension: per-voxel stiffness scaling
    def set_density(self, rho, penal: float = 3.0):
        """Finest-level element stiffness rho_e^penal * Ke0 (not in the reference)."""
        rho = np.asarray(rho, float).ravel()
        if rho.size != self.levels[0].numElements:
            raise GMGSError("density length must equal the number of solid elements")
        self.rho = rho
        self.penal = float(penal)
        self._setup_done = False
        if len(self.levels) > 1:
            self.levels = self.levels[:1]

    # ---------------- SetupSolver.m
    def setup(self):
        p = self.params
        fine = self.levels[0]
        self.Ke0 = element_stiffness(p.youngs_modulus, p.poisson_ratio, fine.eleSize)
        fine.Ke = self.Ke0
        if self.rho is None:
            fine.storingState = 0
            fine.Ks = self.Ke0
        else:   # extension: scaled finest elements
            fine.storingState = 0
            fine.Ks = self.Ke0
            fine.eleScale = self.rho ** self.penal
        if self.numLevels < 2:
            raise GMGSError("There is no sufficient resolution to invoke GMGS!")
        while len(self.levels) < self.numLevels:
            self.levels.append(build_coarse_level(self.levels[-1]))
        self._galerkin_levels()
        self._diagonals()
        self._coarse_fixed_dofs()
        self._factorize_coarsest()
        self._setup_done = True

    @staticmethod
    def _galerkin(child_mats: np.ndarray) -> np.ndarray:
        """Ks = P^T (sum_j scatter(K_j)) P for a batch; child_mats (B, 8, 24, 24), void = 0.

        SetupSolver.m:57-58 assembles the 81x81 block with sparse() and forms
        interpolatingKe' * K * interpolatingKe.
        """
        P81 = np.kron(trilinear_node_table(), np.eye(3))          # 81 x 24
        sub = node_dofs(sub_element_nodes())                     # 8 x 24
        out = np.zeros((child_mats.shape[0], 24, 24))
        for j in range(8):
            Pj = P81[sub[j]]                                     # 24 x 24
            out += np.einsum("ia,bik,kc->bac", Pj, child_mats[:, j], Pj, optimize=True)
        return out

    def _child_matrices(self, level_idx: int, elems: np.ndarray, finer_mat) -> np.ndarray:
        """(B, 8, 24, 24) children stiffness for coarse elements `elems` of level `level_idx`."""
        lv = self.levels[level_idx]
        up = lv.elementUpwardMap[elems]                          # 1-based finer ids
        mats = np.zeros((len(elems), 8, 24, 24))
        for j in range(8):
            solid = up[:, j] > 0
            if np.any(solid):
                mats[solid, j] = finer_mat(up[solid, j] - 1)
        return mats

    def _galerkin_levels(self):
        """Per-level coarse stiffness storage, SetupSolver.m:36-196."""
        L = self.numLevels
        fine = self.levels[0]
        ratio = lambda ii: self.levels[ii].eleSize[0] / fine.eleSize[0]
        scaled = fine.eleScale is not None
        if scaled:
            # extension: every coarse element gets its own Galerkin matrix
            finer = lambda ids: fine.eleScale[ids, None, None] * self.Ke0[None]
            for ii in range(1, L):
                lv = self.levels[ii]
                lv.Ke = self.Ke0 * ratio(ii)
                lv.storingState = 1
                lv.Ks = self._batched(ii, np.arange(lv.numElements), finer)
                Ks = lv.Ks
                finer = (lambda K: (lambda ids: K[ids]))(Ks)
            return
        state_prev = None   # eleStiffnessMatStateOnFinerLevel (0-based index into Ks, 0 = universal)
        for ii in range(1, L):
            lv = self.levels[ii]
            prev = self.levels[ii - 1]
            lv.Ke = self.Ke0 * ratio(ii)
            ne = lv.numElements
            if ii == 1:
                finer = lambda ids: np.broadcast_to(prev.Ke, (len(ids), 24, 24))
            elif ii in (2, 3):
                Kp, sp = prev.Ks, state_prev
                finer = (lambda Kp, sp: (lambda ids: Kp[sp[ids]]))(Kp, sp)
            else:
                Kp = prev.Ks
                finer = (lambda Kp: (lambda ids: Kp[ids]))(Kp)
            if ii == 1 and L > 2:
                lv.storingState = 2
                uniq = np.flatnonzero(np.any(lv.elementUpwardMap == 0, axis=1))
            elif ii == 2 and L > 3:
                lv.storingState = 2
                upP = prev.elementUpwardMap
                uniq = []
                # SetupSolver.m:96-101: only the non-void children are inspected
                for jj in range(ne):
                    kids = lv.elementUpwardMap[jj]
                    kids = kids[kids != 0] - 1
                    if np.any(upP[kids] == 0):
                        uniq.append(jj)
                uniq = np.asarray(uniq, dtype=np.int64)
            else:
                lv.storingState = 1
                lv.Ks = self._batched(ii, np.arange(ne), finer)
                continue
            univ = np.setdiff1d(np.arange(ne), uniq)
            Ks = np.empty((1 + len(uniq), 24, 24))
            Ks[0] = lv.Ke
            if len(uniq):
                Ks[1:] = self._batched(ii, uniq, finer)
            lv.Ks = Ks
            lv.uniqueElements = uniq
            lv.universalElements = univ
            state = np.zeros(ne, dtype=np.int64)
            state[uniq] = np.arange(1, 1 + len(uniq))
            state_prev = state

    def _batched(self, ii, elems, finer, batch=4096):
        out = np.empty((len(elems), 24, 24))
        for s in range(0, len(elems), batch):
            e = elems[s:s + batch]
            out[s:s + batch] = self._galerkin(self._child_matrices(ii, e, finer))
        return out

    def _diagonals(self):
        """diagK on levels 1..L-1, SetupSolver.m:204-244."""
        for ii in range(self.numLevels - 1):
            lv = self.levels[ii]
            d = np.zeros(lv.numDOFs)
            if lv.storingState == 0:
                if lv.eleScale is None:
                    contrib = np.broadcast_to(np.diag(lv.Ks), (lv.numElements, 24))
                else:
                    contrib = lv.eleScale[:, None] * np.diag(lv.Ks)[None, :]
            elif lv.storingState == 1:
                contrib = np.einsum("eii->ei", lv.Ks)
            else:
                contrib = np.empty((lv.numElements, 24))
                contrib[lv.universalElements] = np.diag(lv.Ks[0])
                if len(lv.uniqueElements):
                    contrib[lv.uniqueElements] = np.einsum("eii->ei", lv.Ks[1:])
            for c in range(24):
                d[lv.eDofMat[:, c]] += contrib[:, c]
            lv.diagK = d

    def _coarse_fixed_dofs(self):
        """Restricted fixed indicator, SetupSolver.m:247-254."""
        ind = np.zeros(self.levels[0].numDOFs)
        ind[self.levels[0].fixedDOFs] = 1.0
        for ii in range(1, self.numLevels):
            ind = self.restrict(ind, ii)
            lv = self.levels[ii]
            lv.freeDOFs = np.flatnonzero(ind == 0)
            lv.fixedDOFs = np.setdiff1d(np.arange(lv.numDOFs), lv.freeDOFs)

    def assemble_level(self, ii: int) -> np.ndarray:
        """Dense K of one level from its element storage (DirectlyAssembleStifnessMatrix.m)."""
        lv = self.levels[ii]
        mats = self.element_matrices(ii)
        K = np.zeros((lv.numDOFs, lv.numDOFs))
        rows = np.repeat(lv.eDofMat, 24, axis=1)
        cols = np.tile(lv.eDofMat, (1, 24))
        np.add.at(K, (rows.ravel(), cols.ravel()), mats.reshape(len(mats), -1).ravel())
        return K

    def element_matrices(self, ii: int) -> np.ndarray:
        lv = self.levels[ii]
        if lv.storingState == 0:
            if lv.eleScale is None:
                return np.broadcast_to(lv.Ks, (lv.numElements, 24, 24))
            return lv.eleScale[:, None, None] * lv.Ks[None]
        if lv.storingState == 1:
            return lv.Ks
        out = np.empty((lv.numElements, 24, 24))
        out[lv.universalElements] = lv.Ks[0]
        if len(lv.uniqueElements):
            out[lv.uniqueElements] = lv.Ks[1:]
        return out

    def _factorize_coarsest(self):
        """Assemble + Cholesky on the coarsest free DOFs, SetupSolver.m:257-259."""
        lv = self.levels[-1]
        K = self.assemble_level(self.numLevels - 1)
        Kf = K[np.ix_(lv.freeDOFs, lv.freeDOFs)]
        try:
            self.cholFac = sla.cho_factor(Kf, lower=True)
        except np.linalg.LinAlgError as exc:
            raise GMGSError("coarsest-level matrix is not positive definite") from exc

    # ---------------- operators
    def atx(self, x: np.ndarray, ii: int = 0) -> np.ndarray:
        """y = K_ii x element by element, fixed rows zeroed; AtX.m:1-58."""
        lv = self.levels[ii]
        v = np.zeros(lv.numDOFs)
        U = x[lv.eDofMat]
        if lv.storingState == 0:
            V = U @ lv.Ks
            if lv.eleScale is not None:
                V *= lv.eleScale[:, None]
        elif lv.storingState == 1:
            V = np.einsum("ei,eij->ej", U, lv.Ks)
        else:
            V = np.empty_like(U)
            if len(lv.uniqueElements):
                V[lv.uniqueElements] = np.einsum("ei,eij->ej", U[lv.uniqueElements], lv.Ks[1:])
            V[lv.universalElements] = U[lv.universalElements] @ lv.Ks[0]
        for c in range(24):
            v[lv.eDofMat[:, c]] += V[:, c]
        v[lv.fixedDOFs] = 0.0
        return v

    def jacobi(self, x, r, ii=0, want_residual=True):
        """JacobiSmoother.m:1-10."""
        dx = self.params.omega * r / self.levels[ii].diagK
        xn = x + dx
        if want_residual:
            return xn, r - self.atx(dx, ii)
        return xn

    def restrict(self, r_fine: np.ndarray, ii: int) -> np.ndarray:
        """RestrictResidual.m:1-18 (coarse level index ii, 0-based)."""
        fine, lv = self.levels[ii - 1], self.levels[ii]
        rF = r_fine.reshape(fine.numNodes, 3)
        r1 = np.zeros((lv.intermediateNumNodes, 3))
        r1[lv.solidNodeMapCoarser2Finer] = rF
        r1 /= lv.transferMatCoeffi[:, None]
        RI = trilinear_node_table()
        rc = np.zeros((lv.numNodes, 3))
        for comp in range(3):
            tmp = r1[lv.transferMat, comp].T @ RI          # (ne, 8)
            for k in range(8):
                rc[lv.eNodMat[:, k], comp] += tmp[:, k]
        return rc.reshape(-1)

    def interpolate(self, x_coarse: np.ndarray, ii: int) -> np.ndarray:
        """InterpolationDeviation.m:1-18 (coarse level index ii, 0-based)."""
        fine, lv = self.levels[ii - 1], self.levels[ii]
        xc = x_coarse.reshape(lv.numNodes, 3)
        xf = np.zeros((lv.intermediateNumNodes, 3))
        RI = trilinear_node_table()
        for comp in range(3):
            tmp1 = RI @ xc[lv.eNodMat, comp].T             # (27, ne)
            for k in range(27):
                xf[lv.transferMat[k], comp] += tmp1[k]
        xf /= lv.transferMatCoeffi[:, None]
        return xf[lv.solidNodeMapCoarser2Finer].reshape(-1)

    def coarsest_solve(self, r: np.ndarray) -> np.ndarray:
        lv = self.levels[-1]
        x = np.zeros(lv.numDOFs)
        x[lv.freeDOFs] = sla.cho_solve(self.cholFac, r[lv.freeDOFs])
        return x

    def vcycle(self, r: np.ndarray) -> np.ndarray:
        """Vcycle.m:1-36: V(1,1) with the post-smoother reusing the pre-smoothing residual."""
        L = self.numLevels
        xs = [None] * L
        rs = [None] * L
        rs[0] = r
        for ii in range(1, L):
            xs[ii - 1], rs[ii - 1] = self.jacobi(0.0, rs[ii - 1], ii - 1)
            rs[ii] = self.restrict(rs[ii - 1], ii)
        xs[L - 1] = self.coarsest_solve(rs[L - 1])
        for ii in range(L - 1, 0, -1):
            xs[ii - 1] = xs[ii - 1] + self.interpolate(xs[ii], ii)
            xs[ii - 1] = self.jacobi(xs[ii - 1], rs[ii - 1], ii - 1, want_residual=False)
        d = xs[0].copy()
        d[self.levels[0].fixedDOFs] = 0.0
        return d

    def cg(self, b: np.ndarray, tol=None, max_it=None, verbose=False, x0=None):
        """CG_solver.m:1-56, including the Jacobi step before each preconditioner call."""
        tol = self.params.tol if tol is None else tol
        max_it = self.params.max_it if max_it is None else max_it
        normB = np.linalg.norm(b)
        its = 0
        x = np.zeros_like(b) if x0 is None else np.array(x0, float)
        r1 = b - self.atx(x)
        hist = []
        t0 = time.perf_counter()
        rz_old = None
        p1 = None
        resnorm = np.inf
        self.converged = False
        while its <= max_it:
            x, r1 = self.jacobi(x, r1)
            z2 = self.vcycle(r1)
            its += 1
            rz = r1 @ z2
            if its == 1:
                p2 = z2
            else:
                p2 = z2 + (rz / rz_old) * p1
            q = self.atx(p2)
            alpha = rz / (p2 @ q)
            x = x + alpha * p2
            r2 = r1 - alpha * q
            resnorm = np.linalg.norm(r2) / normB
            if verbose:
                print(f" It.: {its:4d} Res.: {resnorm:16.6e}")
            if resnorm < tol:
                self.converged = True
                break
            rz_old = rz
            p1 = p2
            r1 = r2
            hist.append((its, time.perf_counter() - t0, resnorm))
        self.iterations = its
        self.relres = resnorm
        self.iterationHist = hist
        return x

    # ---------------- GetDeformation.m
    def get_deformation(self, verbose=False, x0=None):
        if self.F is None:
            raise GMGSError("no boundary conditions")
        if not self._setup_done:
            self.setup()
        self.U = self.cg(self.F, verbose=verbose, x0=x0)
        return self.U

    # ---------------- GetCartesianStress.m
    def get_cartesian_stress(self):
        """Nodal stress [xx yy zz yz zx xy] (GetCartesianStress.m:11-41) and the
        per-voxel mean of the 8 Gauss-point stresses (extension, FP64 here)."""
        if self.U is None:
            raise GMGSError("No Deformation Field Available")
        p = self.params
        lv = self.levels[0]
        Mn, Mg = stress_matrices(p.youngs_modulus, p.poisson_ratio, lv.eleSize)
        ue = self.U[lv.eDofMat]
        nodal_e = (ue @ Mn.T).reshape(-1, 8, 6)
        per_voxel = (ue @ Mg.T).reshape(-1, 8, 6).mean(axis=1)
        if self.rho is not None:          # extension: element stiffness rho^penal * Ke0
            sc = self.rho ** self.penal
            nodal_e = nodal_e * sc[:, None, None]
            per_voxel = per_voxel * sc[:, None]
        out = np.zeros((lv.numNodes, 6))
        for k in range(8):
            out[lv.eNodMat[:, k]] += nodal_e[:, k]
        out /= self.numNod2Eles[:, None]
        return out, per_voxel

    # ---------------- direct solve (test helper for gradient checks)
    def direct_solve(self, b=None):
        """Exact solution of the finest-level system on its free DOFs (sparse LU).

        The reference's PCG targets tol 1e-3 and can stagnate far above
        machine precision, so finite-difference checks use this instead.
        """
        import scipy.sparse as sp
        import scipy.sparse.linalg as spl
        if not self._setup_done:
            self.setup()
        lv = self.levels[0]
        b = self.F if b is None else np.asarray(b, float)
        mats = self.element_matrices(0)
        rows = np.repeat(lv.eDofMat, 24, axis=1).ravel()
        cols = np.tile(lv.eDofMat, (1, 24)).ravel()
        K = sp.csr_matrix((mats.reshape(len(mats), -1).ravel(), (rows, cols)), shape=(lv.numDOFs,) * 2)
        f = lv.freeDOFs
        x = np.zeros(lv.numDOFs)
        x[f] = spl.spsolve(K[f][:, f].tocsc(), b[f])
        return x

    # ---------------- extension: adjoint
    def gradient(self, u=None, ell=None, lam=None):
        """dJ/drho_e for J = f^T u (ell None) or J = ell^T u; needs set_density.

        dJ/drho_e = -penal * rho_e^(penal-1) * lam_e^T Ke0 u_e with K lam = ell
        (lam = u for the self-adjoint compliance case).
        """
        if self.rho is None:
            raise GMGSError("gradient needs a density field")
        u = self.U if u is None else u
        lv = self.levels[0]
        if lam is None:
            lam = u if ell is None else self.cg(np.asarray(ell, float))
        ue = u[lv.eDofMat]
        le = lam[lv.eDofMat]
        energy = np.einsum("ei,ij,ej->e", le, self.Ke0, ue)
        return -self.penal * self.rho ** (self.penal - 1.0) * energy
