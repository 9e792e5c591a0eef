"""Python host side of libgmgs: a handle wrapper and a session object that
mirrors the reference's call surface.

The reference drives its solve through MATLAB globals and two functions
(src/GMGS3D.m:11-34, src/Demo.m:67-81):

    voxelizedVolume_ = CreateVoxilizedModel(...); DiscretizeDesignDomain();
    fixingCond_ = ...; loadingCond_ = ...;
    GetDeformation();       % -> U_
    GetCartesianStress();   % -> cartesianStressField_

`Session` keeps the same names (tol_, maxIT_, weightFactorJacobi_, moduls_,
poissonRatio_, coarsestResolutionControl_, voxelizedVolume_, fixingCond_,
loadingCond_, U_, cartesianStressField_, iterationHist_) and methods
(DiscretizeDesignDomain, GetDeformation, GetCartesianStress).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class GMGSError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Solver:
    """One gmgs_handle: model + hierarchy on the current CUDA device."""

    def __init__(self, voxels, *, ele_size=(1.0, 1.0, 1.0), tol=1e-3, max_it=20000, omega=0.4,
                 youngs_modulus=1.0, poisson_ratio=0.3, coarsest_resolution_control=10000,
                 num_levels=0, precision="fp64", verbose=False):
        self._lib = L.load()
        vox = np.asfortranarray(np.asarray(voxels, dtype=np.int32))
        if vox.ndim != 3:
            raise ValueError("voxels must be a (ny, nx, nz) array")
        self.shape = vox.shape
        p = L.Params()
        self._lib.gmgs_default_params(C.byref(p))
        p.tol = tol
        p.max_it = max_it
        p.omega = omega
        p.youngs_modulus = youngs_modulus
        p.poisson_ratio = poisson_ratio
        p.coarsest_resolution_control = coarsest_resolution_control
        p.num_levels = num_levels
        p.precision = {"fp64": L.FP64, "mixed": L.MIXED}[precision] if isinstance(precision, str) else int(precision)
        p.verbose = int(bool(verbose))
        self.params = p
        flat = np.ascontiguousarray(vox.ravel(order="F"))
        es = np.asarray(ele_size, dtype=np.float64)
        h = C.c_void_p()
        st = self._lib.gmgs_create(_iptr(flat), vox.shape[0], vox.shape[1], vox.shape[2], _dptr(es),
                                   C.byref(p), C.byref(h))
        if st != L.OK:
            raise GMGSError(st, self._lib.gmgs_last_error(None).decode())
        self._h = h
        self.iterations = 0
        self.relres = float("nan")
        self.status = L.OK

    # ------------------------------------------------------------------ utils
    def _check(self, st, allow=()):
        if st != L.OK and st not in allow:
            raise GMGSError(st, self._lib.gmgs_last_error(self._h).decode())
        return st

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gmgs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    @property
    def num_levels(self) -> int:
        v = C.c_int32()
        self._check(self._lib.gmgs_num_levels(self._h, C.byref(v)))
        return v.value

    def num_nodes(self, level: int = 1) -> int:
        v = C.c_int64()
        self._check(self._lib.gmgs_num_nodes(self._h, level, C.byref(v)))
        return v.value

    def num_elements(self, level: int = 1) -> int:
        v = C.c_int64()
        self._check(self._lib.gmgs_num_elements(self._h, level, C.byref(v)))
        return v.value

    @property
    def padded_dims(self):
        d = (C.c_int32 * 3)()
        self._check(self._lib.gmgs_padded_dims(self._h, d))
        return tuple(d)

    @staticmethod
    def memory_stats(reset_peak: bool = False):
        """(bytes held now, high-water mark) over every handle in the process."""
        cur, peak = C.c_int64(), C.c_int64()
        L.load().gmgs_memory_stats(C.byref(cur), C.byref(peak), int(reset_peak))
        return cur.value, peak.value

    @property
    def device_bytes(self) -> int:
        v = C.c_int64()
        self._check(self._lib.gmgs_device_bytes(self._h, C.byref(v)))
        return v.value

    @property
    def launch_count(self) -> int:
        v = C.c_int64()
        self._check(self._lib.gmgs_launch_count(self._h, C.byref(v)))
        return v.value

    @property
    def phase_times_ms(self):
        d = (C.c_double * 4)()
        self._check(self._lib.gmgs_phase_times(self._h, d))
        return {"create": d[0], "bc_setup": d[1], "solve": d[2], "stress": d[3]}

    def set_profiling(self, enable: bool = True):
        self._check(self._lib.gmgs_set_profiling(self._h, int(bool(enable))))

    def kernel_time(self, kernel: int = 0):
        """(launches, total ms, algorithmic bytes) recorded since set_profiling(True)."""
        n = C.c_int64()
        ms = C.c_double()
        by = C.c_double()
        self._check(self._lib.gmgs_kernel_time(self._h, kernel, C.byref(n), C.byref(ms), C.byref(by)))
        return n.value, ms.value, by.value

    def set_stream(self, stream_ptr: int | None):
        self._check(self._lib.gmgs_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def set_tolerance(self, tol: float, max_it: int):
        self._check(self._lib.gmgs_set_tolerance(self._h, tol, max_it))

    # ---------------------------------------------------------------- the path
    def set_bc(self, fixed_nodes, loads):
        fixed = np.ascontiguousarray(np.asarray(fixed_nodes).ravel(), dtype=np.int32)
        ld = np.ascontiguousarray(np.asarray(loads, dtype=np.float64).reshape(-1, 4))
        self._loads = ld
        self._check(self._lib.gmgs_set_bc(self._h, _iptr(fixed) if fixed.size else None, fixed.size,
                                          _dptr(ld) if ld.size else None, ld.shape[0]))

    def load_vector(self):
        """F (3*num_nodes, interleaved) as ApplyBoundaryCondition.m:7-10 builds it."""
        F = np.zeros(3 * self.num_nodes(1))
        for row in self._loads:               # a later duplicate id wins
            i = 3 * (int(row[0]) - 1)
            F[i:i + 3] = row[1:4]
        return F

    def set_density(self, rho, penal: float = 3.0):
        r = np.ascontiguousarray(np.asarray(rho, dtype=np.float64).ravel())
        if r.size != self.num_elements(1):
            raise ValueError("rho must have one entry per solid voxel")
        self._check(self._lib.gmgs_set_density(self._h, _dptr(r), penal))

    def solve(self, with_history=False, out=None):
        """Return U (3*num_nodes, interleaved); raise on divergence.

        out: optional float64 C-contiguous array of 3*num_nodes to write U into
        (e.g. a pinned host buffer reused across solves); returned as U."""
        nn = self.num_nodes(1)
        if out is None:
            U = np.empty(3 * nn)
        else:
            U = out
            if U.dtype != np.float64 or U.size != 3 * nn or not U.flags.c_contiguous or not U.flags.writeable:
                raise ValueError("out must be a writeable C-contiguous float64 array of 3 * num_nodes")
        it = C.c_int32()
        rr = C.c_double()
        hist = np.zeros(3 * (self.params.max_it + 2)) if with_history else None
        st = self._check(self._lib.gmgs_solve(self._h, _dptr(U), C.byref(it), C.byref(rr), _dptr(hist)),
                         allow=(L.ERR_MAX_ITERATIONS,))
        self.status, self.iterations, self.relres = st, it.value, rr.value
        if with_history:
            nrows = self.iterations - 1 if st == L.OK else self.iterations
            self.history = hist[:3 * max(nrows, 0)].reshape(-1, 3)
        return U

    def solve_dev(self, U_dev_ptr: int | None):
        it = C.c_int32()
        rr = C.c_double()
        st = self._check(self._lib.gmgs_solve_dev(self._h, C.c_void_p(U_dev_ptr or 0), C.byref(it), C.byref(rr), None),
                         allow=(L.ERR_MAX_ITERATIONS,))
        self.status, self.iterations, self.relres = st, it.value, rr.value
        return st

    def stress(self, per_voxel=True):
        nodal = np.empty((self.num_nodes(1), 6))
        vox = np.empty((self.num_elements(1), 6), dtype=np.float32) if per_voxel else None
        self._check(self._lib.gmgs_stress(self._h, _dptr(nodal), _fptr(vox)))
        return (nodal, vox) if per_voxel else nodal

    def stress_dev(self, nodal_ptr: int | None, voxel_ptr: int | None):
        """Stress into device buffers: nodal (num_nodes x 6 f64) and/or per voxel (num_elements x 6 f32)."""
        self._check(self._lib.gmgs_stress_dev(self._h, C.c_void_p(nodal_ptr or 0), C.c_void_p(voxel_ptr or 0)))

    def grad_dev(self, ell_ptr: int | None, out_ptr: int):
        """dJ/drho into a device buffer (num_elements f64); ell_ptr None means compliance."""
        self._check(self._lib.gmgs_grad_dev(self._h, C.c_void_p(ell_ptr or 0), C.c_void_p(out_ptr)))

    def grad(self, ell=None):
        out = np.empty(self.num_elements(1))
        e = None if ell is None else np.ascontiguousarray(np.asarray(ell, dtype=np.float64).ravel())
        self._check(self._lib.gmgs_grad(self._h, _dptr(e), _dptr(out)))
        return out

    def apply_operator(self, x, level: int = 1):
        """AtX(x, level) on compact interleaved vectors."""
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
        y = np.empty_like(x)
        self._check(self._lib.gmgs_apply_operator(self._h, level, _dptr(x), _dptr(y)))
        return y

    def apply_operator_dev(self, x_ptr: int, y_ptr: int, level: int = 1):
        """AtX on device buffers (compact interleaved float64 of the level's DOFs)."""
        self._check(self._lib.gmgs_apply_operator_dev(self._h, level, C.c_void_p(x_ptr), C.c_void_p(y_ptr)))

    def apply_preconditioner_dev(self, r_ptr: int, z_ptr: int):
        self._check(self._lib.gmgs_apply_preconditioner_dev(self._h, C.c_void_p(r_ptr), C.c_void_p(z_ptr)))

    def dot_dev(self, x_ptr: int, y_ptr: int, n: int) -> float:
        """Deterministic FP64 inner product of two device vectors of n doubles."""
        out = C.c_double()
        self._check(self._lib.gmgs_dot_dev(self._h, C.c_void_p(x_ptr), C.c_void_p(y_ptr), n, C.byref(out)))
        return out.value

    def apply_preconditioner(self, r):
        """Vcycle(r) on a compact interleaved finest-level vector."""
        r = np.ascontiguousarray(np.asarray(r, dtype=np.float64))
        z = np.empty_like(r)
        self._check(self._lib.gmgs_apply_preconditioner(self._h, _dptr(r), _dptr(z)))
        return z


class Session:
    """The reference's global workspace and entry points (src/GlobalVariables.m:3-38)."""

    def __init__(self):
        self.tol_ = 1.0e-3
        self.maxIT_ = 20000
        self.weightFactorJacobi_ = 0.4
        self.moduls_ = 1.0
        self.poissonRatio_ = 0.3
        self.coarsestResolutionControl_ = 10000
        self.numLevels_ = 0            # 0 = the reference's rule
        self.eleSize_ = (1.0, 1.0, 1.0)
        self.precision_ = "fp64"
        self.voxelizedVolume_ = None
        self.fixingCond_ = None
        self.loadingCond_ = None
        self.F_ = None
        self.U_ = None
        self.cartesianStressField_ = None
        self.iterationHist_ = np.zeros((0, 3))
        self.boundingBox_ = None
        self._solver = None

    def CreateVoxilizedModel(self, *args):
        """CreateVoxilizedModel(triFaceModelFile, finestResCtrl): voxelise an
        ASCII .ply mesh on the GPU (src/common/CreateVoxilizedModel.m:10-26);
        the voxel edge lengths follow from the mesh bounding box
        (DiscretizeDesignDomain.m:53-65).
        CreateVoxilizedModel(nx, ny, nz): solid cuboid of unit voxels (:27-32)."""
        if len(args) == 2:
            from . import mesh
            vertices, faces = mesh.read_ply(args[0])
            self.voxelizedVolume_, ele = mesh.voxelize(vertices, faces, int(args[1]))
            self.eleSize_ = tuple(float(e) for e in ele)
            self.boundingBox_ = np.stack([vertices.min(axis=0), vertices.max(axis=0)])
        elif len(args) == 3:
            nx, ny, nz = (int(a) for a in args)
            self.voxelizedVolume_ = np.ones((ny, nx, nz), dtype=np.int32)
            self.eleSize_ = (1.0, 1.0, 1.0)
            self.boundingBox_ = np.array([[0.0, 0.0, 0.0], [nx, ny, nz]], dtype=np.float64)
        else:
            raise GMGSError(L.ERR_INVALID_ARGUMENT, "Wrong input for voxelization!")
        self._solver = None
        return self.voxelizedVolume_

    def DiscretizeDesignDomain(self):
        self._solver = Solver(self.voxelizedVolume_, ele_size=self.eleSize_, tol=self.tol_, max_it=self.maxIT_,
                              omega=self.weightFactorJacobi_, youngs_modulus=self.moduls_,
                              poisson_ratio=self.poissonRatio_,
                              coarsest_resolution_control=self.coarsestResolutionControl_,
                              num_levels=self.numLevels_, precision=self.precision_)
        return self._solver

    @property
    def numLevels(self):
        return self._solver.num_levels

    def GetDeformation(self):
        if self._solver is None:
            self.DiscretizeDesignDomain()
        self._solver.set_bc(self.fixingCond_, self.loadingCond_)
        self._solver.set_tolerance(self.tol_, self.maxIT_)
        self.U_ = self._solver.solve(with_history=True)
        self.iterationHist_ = np.vstack([self.iterationHist_, self._solver.history])
        return self.U_

    def GetCartesianStress(self):
        self.cartesianStressField_ = self._solver.stress(per_voxel=False)
        return self.cartesianStressField_

    # ------------------------------------------------ output formats
    def _grid(self):
        """(resolution (x, y, z), padded occupancy, bounding box after padding)
        as DiscretizeDesignDomain.m:37-63 leaves them."""
        if self._solver is None:
            self.DiscretizeDesignDomain()
        ny, nx, nz = self._solver.padded_dims
        vox = np.zeros((ny, nx, nz), dtype=np.int32)
        oy, ox, oz = self.voxelizedVolume_.shape
        vox[:oy, :ox, :oz] = self.voxelizedVolume_
        bb = self.boundingBox_
        if bb is None:
            bb = np.array([[0.0, 0.0, 0.0], [ox * self.eleSize_[0], oy * self.eleSize_[1], oz * self.eleSize_[2]]])
        bb = np.array(bb, dtype=np.float64)
        bb[1] = bb[0] + (bb[1] - bb[0]) * np.array([nx, ny, nz], dtype=np.float64) / np.array([ox, oy, oz], dtype=np.float64)
        return (nx, ny, nz), vox, bb

    def ExportDataset_3DTSV(self, path="dataset_TSV.carti"):
        """The .carti stress dataset (src/common/ExportDataset_3DTSV.m:1-42)."""
        if self.cartesianStressField_ is None:
            import warnings
            warnings.warn("No Cartesian Stress Available!")
            return None
        from . import export
        res, vox, bb = self._grid()
        ele, nod = export.grid_maps(vox)
        export.export_dataset_3dtsv(path, res, bb[0], bb[1], ele, nod, self.fixingCond_, self.loadingCond_,
                                    self.cartesianStressField_)
        return path

    def WrapVoxelFEAmodel(self, path="wrappedVoxelFEAmodel.txt"):
        """The wrapped voxel FEA model (src/common/WrapVoxelFEAmodel.m:1-26)."""
        from . import export
        res, vox, _ = self._grid()
        ele, nod = export.grid_maps(vox)
        export.wrap_voxel_fea_model(path, res, ele, nod, self.fixingCond_, self.loadingCond_)
        return path
