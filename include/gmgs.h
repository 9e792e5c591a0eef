/*
 * gmgs.h - C ABI of libgmgs, a GB300 (sm_103a) implementation of GMGS-3D's
 * geometric-multigrid-preconditioned CG solve for static linear elasticity
 * on Cartesian voxel meshes.
 *
 * The reference is MATLAB and exposes its solve through globals and two
 * functions: GetDeformation() (src/kernel/GetDeformation.m:1-22) and
 * GetCartesianStress() (src/kernel/GetCartesianStress.m:1-42).  Its operator
 * interface is the function-handle pair handed to the Krylov solver,
 *     U_ = CG_solver(@AtX, @Vcycle, F_, tol_, maxIT_, 'printP_ON')
 * (src/kernel/GetDeformation.m:20, src/kernel/CG_solver.m:1).
 * Each entry point below names the reference interface it replaces.
 *
 * Conventions
 *  - Every call returns an int status (GMGS_OK == 0).  gmgs_last_error()
 *    gives a message for the last failing call on a handle.
 *  - Host pointers are caller-owned; data are copied in and out.  The *_dev
 *    variants take device pointers (same layout) and copy nothing to the host.
 *  - Layouts follow the reference: the occupancy is MATLAB's
 *    voxelizedVolume_(y,x,z), column-major (y fastest), value 1 = solid.
 *    Node ids are the reference's compact 1-based numbering of solid nodes
 *    (src/common/DiscretizeDesignDomain.m:76-93).  Displacements are
 *    interleaved per node [u1x u1y u1z u2x ...] (src/common/ApplyBoundaryCondition.m:10).
 *  - One handle per host thread; every handle owns one CUDA stream unless
 *    gmgs_set_stream() supplies one.
 */
#ifndef GMGS_H
#define GMGS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes: replace the reference's error() aborts and warning()+return cases */
enum gmgs_status {
    GMGS_OK = 0,
    GMGS_ERR_INVALID_ARGUMENT = 1,  /* bad pointer, dims, ids, sizes */
    GMGS_ERR_RESOLUTION = 2,        /* too few voxels / levels: DiscretizeDesignDomain.m:30-32, SetupSolver.m:19-21 */
    GMGS_ERR_NO_SOLID = 3,          /* occupancy has no solid voxel */
    GMGS_ERR_NO_LOADS = 4,          /* ApplyBoundaryCondition.m:12 */
    GMGS_ERR_NO_FIXINGS = 5,        /* ApplyBoundaryCondition.m:22 */
    GMGS_ERR_NOT_SPD = 6,           /* coarsest Cholesky failed (the reference ignores chol's flag, SetupSolver.m:259) */
    GMGS_ERR_MAX_ITERATIONS = 7,    /* CG_solver.m:52-55 (a warning there; U is still returned) */
    GMGS_ERR_NONFINITE = 8,         /* NaN/Inf residual */
    GMGS_ERR_NO_SOLUTION = 9,       /* stress/gradient before a solve: GetCartesianStress.m:7-9 */
    GMGS_ERR_CUDA = 10,             /* CUDA runtime failure */
    GMGS_ERR_OUT_OF_MEMORY = 11,
    GMGS_ERR_STATE = 12,            /* call order (e.g. solve before set_bc) */
    GMGS_ERR_MESH = 13              /* a mesh the reference's voxeliser cannot handle (Voxelize.m:176-203) */
};

enum gmgs_precision {
    GMGS_FP64 = 0,   /* plain FP64 V-cycle PCG: the drop-in for the reference solve */
    GMGS_MIXED = 1   /* FP32 V-cycle, double-float (2 x FP32) outer CG state, FP64 dots, coarsest solve and U */
};

/* Solver controls; the reference's globals (src/GlobalVariables.m:3-23). */
typedef struct gmgs_params {
    double tol;                          /* tol_ (1e-3) */
    int32_t max_it;                      /* maxIT_ (20000) */
    double omega;                        /* weightFactorJacobi_ (0.4) */
    double youngs_modulus;               /* moduls_ (1.0) */
    double poisson_ratio;                /* poissonRatio_ (0.3) */
    int64_t coarsest_resolution_control; /* coarsestResolutionControl_ (10000) */
    int32_t num_levels;                  /* 0 = reference rule from the control above; else explicit (>= 2) */
    int32_t precision;                   /* enum gmgs_precision */
    int32_t verbose;                     /* 1 = print per-iteration residuals like 'printP_ON' */
} gmgs_params;

typedef struct gmgs_handle gmgs_handle;

/* Fill *p with the reference defaults (GlobalVariables.m:3-23), GMGS_FP64. */
void gmgs_default_params(gmgs_params* p);

/* Model creation + solver setup independent of boundary conditions.
 * Replaces DiscretizeDesignDomain() (src/common/DiscretizeDesignDomain.m:1-121),
 * BuildingMeshHierarchy() (src/kernel/BuildingMeshHierarchy.m:1-144) and the
 * stiffness part of SetupSolver() (src/kernel/SetupSolver.m:9-244).
 * occupancy: ny*nx*nz int32, column-major (y fastest); ele_size: voxel edge
 * lengths (x, y, z), which the reference derives from its bounding box
 * (DiscretizeDesignDomain.m:65). */
int gmgs_create(const int32_t* occupancy, int32_t ny, int32_t nx, int32_t nz,
                const double ele_size[3], const gmgs_params* params, gmgs_handle** out);

/* Mesh voxelisation; replaces CreateVoxilizedModel(triFaceModelFile,
 * finestResCtrl) (src/common/CreateVoxilizedModel.m:10-26 with
 * AdaptData4Voxelize.m:5-18 and Voxelize.m:1-331): the longest bounding-box
 * side gets finest_resolution voxels, rays along x, y and z through the voxel
 * centres decide inside/outside by crossing parity, a voxel is solid when two
 * of the three directions agree, and the result is flipped along y.
 * vertices: nv x 3 (x, y, z) row-major; faces: nf x 3 0-based vertex ids.
 * dims receives {ny, nx, nz}; with occupancy == NULL only dims are computed,
 * otherwise occupancy (ny*nx*nz int32, y fastest, 1 = solid) is filled.
 * The voxel edge lengths for gmgs_create are the bounding-box extents divided
 * by {nx, ny, nz} (DiscretizeDesignDomain.m:53-65). */
int gmgs_voxelize_mesh(const double* vertices, int64_t nv, const int32_t* faces, int64_t nf,
                       int32_t finest_resolution, int32_t dims[3], int32_t* occupancy);

/* Boundary conditions; replaces ApplyBoundaryCondition()
 * (src/common/ApplyBoundaryCondition.m:1-24) with fixingCond_ / loadingCond_.
 * fixed_nodes: 1-based compact node ids, all three DOFs fixed.
 * loads: nload rows of (id, fx, fy, fz), row-major; a later duplicate id wins.
 * As in the reference, the coarse-level fixed DOFs and the coarsest
 * factorisation are built at the first solve and kept afterwards
 * (GetDeformation.m:12-16 runs SetupSolver() once). */
int gmgs_set_bc(gmgs_handle* h, const int32_t* fixed_nodes, int64_t nfixed,
                const double* loads, int64_t nload);

/* Extension (not in the reference): per-solid-voxel stiffness scale rho^penal
 * on the finest level, in the compact element order (eleMapBack,
 * DiscretizeDesignDomain.m:68).  Rebuilds every coarse operator. */
int gmgs_set_density(gmgs_handle* h, const double* rho, double penal);

/* Solve K U = F.  Replaces GetDeformation() / CG_solver(@AtX,@Vcycle,...)
 * (src/kernel/GetDeformation.m:1-22, src/kernel/CG_solver.m:1-56).
 * U: 3*num_nodes doubles, interleaved, or NULL to keep it on the device.
 * iters / relres: nullable.  hist: nullable, room for 3*(max_it+1) doubles,
 * rows (its, seconds, resnorm) like iterationHist_ (CG_solver.m:49); the
 * number of rows written is *iters - 1 when converged, else *iters.
 * Returns GMGS_ERR_MAX_ITERATIONS (U still written) when not converged. */
int gmgs_solve(gmgs_handle* h, double* U, int32_t* iters, double* relres, double* hist);
int gmgs_solve_dev(gmgs_handle* h, double* U_dev, int32_t* iters, double* relres, double* hist);

/* Nodal Cartesian stress, num_nodes x 6 row-major [xx yy zz yz zx xy];
 * replaces GetCartesianStress() (src/kernel/GetCartesianStress.m:1-42).
 * per_voxel (nullable, extension): num_elements x 6 floats, the mean of the 8
 * Gauss-point stresses of each solid voxel. */
int gmgs_stress(gmgs_handle* h, double* nodal, float* per_voxel);
int gmgs_stress_dev(gmgs_handle* h, double* nodal_dev, float* per_voxel_dev);

/* Extension: gradient w.r.t. rho (needs gmgs_set_density and a solve).
 * ell == NULL: compliance F^T U;  else J = ell^T U with ell a 3*num_nodes
 * interleaved vector (an adjoint solve K lambda = ell with the same PCG).
 * dJdrho: num_elements doubles in the compact element order. */
int gmgs_grad(gmgs_handle* h, const double* ell, double* dJdrho);
int gmgs_grad_dev(gmgs_handle* h, const double* ell_dev, double* dJdrho_dev);

/* Operator handles of CG_solver: AtX(x, level) (src/kernel/AtX.m:1-58) and
 * Vcycle(r) (src/kernel/Vcycle.m:1-36), on compact interleaved vectors of
 * the level's DOFs.  level is 1-based like the reference; the coarse-level
 * numbering is the reference's compact numbering of that level's nodes
 * (BuildingMeshHierarchy.m:101-118).  Available after the first solve. */
int gmgs_apply_operator(gmgs_handle* h, int32_t level, const double* x, double* y);
int gmgs_apply_preconditioner(gmgs_handle* h, const double* r, double* z);
/* The same on device buffers (compact interleaved), on the handle's stream. */
int gmgs_apply_operator_dev(gmgs_handle* h, int32_t level, const double* x_dev, double* y_dev);
int gmgs_apply_preconditioner_dev(gmgs_handle* h, const double* r_dev, double* z_dev);
/* r1'*z2-style inner product of CG_solver.m:26,31,35 on device vectors:
 * deterministic FP64 reduction (fixed partition and summation order, so
 * repeated calls give identical bits) using the handle's scratch memory.
 * *result is written on the host after the handle's stream is synchronised. */
int gmgs_dot_dev(gmgs_handle* h, const double* x_dev, const double* y_dev, int64_t n, double* result);

/* Allocation-free variant of gmgs_dot_dev; no counterpart in the reference.
 * For callers that cannot allocate device memory: hosts whose device memory
 * belongs to their own allocator (a MATLAB MEX shim working on gpuArray
 * buffers, a framework whose caching allocator must see every allocation) and
 * code paths that cannot afford the implicit device synchronisation of
 * cudaMalloc / cudaFree.  It needs no handle and calls no allocating routine.
 * Computes the FP64 inner product of two device vectors of n doubles into
 * the device scalar *result_dev, asynchronously on `stream` (a cudaStream_t;
 * NULL = the legacy default stream).  The result is deterministic for a given
 * n on any GPU (fixed chunks of 8,192 elements, partials summed in chunk
 * order) but not bit-identical to gmgs_dot_dev, which partitions the vectors
 * differently; the two agree to rounding.
 * Scratch: a fixed 512 KiB static device array inside libgmgs (65,536 block
 * partials and an arrival counter), held by every GPU that loads the library
 * until the process exits.  n must not exceed GMGS_DOT_NOALLOC_MAX_N
 * (65,536 blocks x 8,192 elements); longer vectors get
 * GMGS_ERR_INVALID_ARGUMENT (use gmgs_dot_dev).  Every call looks up the
 * array's device address (cudaGetSymbolAddress) for the current device; the
 * first call on a device also loads the library's kernels there, so make that
 * first call before any stream capture.  All calls
 * share the array and each clears the counter it needs before its kernel
 * runs; calls that overlap on the GPU (several streams or host threads at
 * once) race on the array and must be serialised by the caller. */
#define GMGS_DOT_NOALLOC_MAX_N 536870912LL
int gmgs_dot_dev_noalloc(const double* x_dev, const double* y_dev, int64_t n, double* result_dev, void* stream);

/* Sizes */
int gmgs_num_levels(const gmgs_handle* h, int32_t* out);
int gmgs_num_nodes(const gmgs_handle* h, int32_t level, int64_t* out);
int gmgs_num_elements(const gmgs_handle* h, int32_t level, int64_t* out);
int gmgs_padded_dims(const gmgs_handle* h, int32_t dims[3]);   /* (ny, nx, nz) after padding */

/* Run-time controls and diagnostics */
int gmgs_set_stream(gmgs_handle* h, void* cuda_stream);   /* cudaStream_t; NULL = own stream */
int gmgs_set_tolerance(gmgs_handle* h, double tol, int32_t max_it);
int gmgs_device_bytes(const gmgs_handle* h, int64_t* out);   /* device memory held by the handle */
int gmgs_launch_count(const gmgs_handle* h, int64_t* out);   /* kernels launched so far */
/* Device memory of all handles in the process (bytes now held, high-water mark
 * since the last reset), including setup temporaries; reset_peak != 0 sets the
 * mark to the current value after reading. */
int gmgs_memory_stats(int64_t* current_bytes, int64_t* peak_bytes, int32_t reset_peak);
int gmgs_phase_times(const gmgs_handle* h, double out[4]);   /* ms: create, bc-setup, last solve, last stress */
/* Kernel timing with CUDA events on the handle's stream (diagnostics).
 * gmgs_set_profiling(h, 1) clears the records and starts recording;
 * gmgs_kernel_time() sums them.  kernel: 0 = finest-level K*x launches,
 * 1 = whole V-cycles, 2 = whole CG iterations, 3 = finest CG update + Jacobi,
 * 4 = finest V-cycle down-sweep, 5 = finest CG direction + A p, 6 = finest
 * prolongation + post-smooth, 7 = levels 2..L of the V-cycles.  bytes:
 * algorithmic bytes of the recorded launches (0 for whole phases). */
int gmgs_set_profiling(gmgs_handle* h, int32_t enable);
int gmgs_kernel_time(gmgs_handle* h, int32_t kernel, int64_t* launches, double* total_ms, double* bytes);
const char* gmgs_last_error(const gmgs_handle* h);
const char* gmgs_status_string(int status);
void gmgs_destroy(gmgs_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* GMGS_H */
