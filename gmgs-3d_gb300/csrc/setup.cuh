// The state behind one gmgs_handle and the setup / solve entry points used by
// the C ABI (api.cu).
#pragma once

#include "fine.cuh"
#include "gmgs_internal.cuh"

namespace gmgs {

struct Model {
    gmgs_params prm{};
    int nely = 0, nelx = 0, nelz = 0;   // unpadded voxel grid
    int ny = 0, nx = 0, nz = 0;         // padded finest grid
    double ele[3] = {1, 1, 1};
    int num_levels = 0;
    bool has_density = false;
    double penal = 3.0;
    std::vector<Level> levels;
    Ctx ctx;
    bool own_stream = false;
    double ke0_rows[KE];   // Ke0 with row = output DOF
    DevBuf ke0_dev;
    DevBuf galerkin_child; // 8 x 24x24: P_j^T Ke0 P_j per child position j
    bool lean_level1 = false; // level-2 (index 1) matrices kept in FP32 only (mixed precision + density)
    MatCoef<double> mc64;  // Ke0 and the interior stencil of this handle's material and voxel
    MatCoef<float> mc32;
    DevBuf rho;            // compact density (double), extension
    // boundary conditions and solution (finest level, FP64, 3 planes)
    DevBuf F, U;
    double normF = 0;
    // coarsest level
    int nfree = 0;
    DevBuf free_idx, cvec_in, cvec_out;   // free DOF slots; coarse vectors (cb.nb * cb.B long)
    CoarseBlocks cb;
    // outer CG work vectors
    DevBuf cg_x, cg_r, cg_p, cg_dx, cg_q64, cg_y64, cg_z64;   // FP64 path
    DevBuf cg_q32, cg_y32, cg_z32, cg_r32;                     // mixed path
    DevBuf cg_r32b, cg_pa, cg_pb;                              // mixed path double buffers
    Coef32 coef{};                                             // FP32 stencil + element matrix
    TcCoef tcoef{};                                            // Ke as the tensor cores' B operand
    DevBuf tc_err;         // int: set when a tensor-core wait ran out
    bool use_tc = false;   // V-cycle down-sweeps on the tensor cores (environment GMGS_TC)
    DevBuf scal;           // device scalars (see solver.cu)
    DevBuf dot_partials, dot_ticket;
    // CUDA graphs of the mixed PCG iteration body (one per parity), valid for
    // the solution buffer and the work-buffer generation they were captured with
    cudaGraphExec_t cg_graph[2] = {nullptr, nullptr};
    int64_t cg_graph_kernels[2] = {0, 0};
    const double* cg_graph_x = nullptr;
    uint64_t cg_graph_gen = 0, gen = 0;
    double* scal_host = nullptr;   // pinned
    int dot_blocks = 0;
    bool bc_set = false, coarse_ready = false, solved = false, ops_ready = false;
    // diagnostics
    double t_create_ms = 0, t_bc_ms = 0, t_solve_ms = 0, t_stress_ms = 0;
    int last_iters = 0;
    double last_relres = 0;
    std::string err;
};

DevBuf dalloc(size_t bytes);
int64_t exclusive_scan(Ctx& c, int32_t* d, int64_t n);

void element_stiffness(double E, double nu, const double ele[3], double Ke[KE]);
// Isotropic Hooke coefficients (d11, d12, d44) and reciprocal element edges
// (1/dx, 1/dy, 1/dz) for the stress kernels.
template <typename T> inline const MatCoef<T>& mat_coef(const Model& M);
template <> inline const MatCoef<double>& mat_coef<double>(const Model& M) { return M.mc64; }
template <> inline const MatCoef<float>& mat_coef<float>(const Model& M) { return M.mc32; }

void stress_coefficients(double E, double nu, const double ele[3], double c[6]);

// setup.cu
void build_levels(Model& M, const int32_t* occ_dev);
void build_operators(Model& M);
void apply_bc(Model& M, const int32_t* fixed, int64_t nfixed, const double* loads, int64_t nload);
// overlap: see factor_coarse
void build_coarse_bc(Model& M, const std::function<void()>& overlap = {});
void set_density_dev(Model& M, const double* rho_dev);

// solver.cu
void alloc_work(Model& M);
void reset_graphs(Model& M);   // destroy the captured PCG iteration graphs
int pcg_solve(Model& M, const double* b_dense, double* x_dense, int32_t* iters, double* relres, double* hist);
void vcycle_apply_fp64(Model& M, const double* r_dense, double* z_dense);
void apply_operator_dense(Model& M, int level, const double* x_dense, double* y_dense);

// post.cu
void stress_dev(Model& M, const double* U_dense, double* nodal_compact, float* per_voxel_compact);
void grad_dev(Model& M, const double* U_dense, const double* lam_dense, double* dJdrho_compact);

}  // namespace gmgs
