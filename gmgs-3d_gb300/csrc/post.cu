// Post-processing on the solved displacement: nodal-averaged Cartesian stress
// (src/kernel/GetCartesianStress.m:11-41), per-voxel stress and the adjoint
// gradient with respect to the per-voxel stiffness scale (extension).
#include "setup.cuh"

namespace gmgs {

__constant__ double c_mnodal[48 * 24];   // OTP * D * B, rows 6k+a: node k, component a
__constant__ double c_mgauss[48 * 24];   // D * B, rows 6g+a: Gauss point g, component a

static void upload_stress(const Model& M) {
    double Mn[48 * 24], Mg[48 * 24];
    stress_matrices(M.prm.youngs_modulus, M.prm.poisson_ratio, M.ele, Mn, Mg);
    GMGS_CUDA(cudaMemcpyToSymbol(c_mnodal, Mn, sizeof(Mn)));
    GMGS_CUDA(cudaMemcpyToSymbol(c_mgauss, Mg, sizeof(Mg)));
}

// One thread per solid node: sum M_nodal u_e over the node's solid elements,
// divide by their number (numNod2ElesVec_, DiscretizeDesignDomain.m:103-107).
__global__ void __launch_bounds__(128) k_stress_nodal(Grid g, const uint8_t* __restrict__ emask,
                                                      const double* __restrict__ escale,
                                                      const int32_t* __restrict__ node_slot,
                                                      const double* __restrict__ count, int64_t nn,
                                                      const double* __restrict__ U, double* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const int64_t s = node_slot[i];
    const int64_t S = g.slots, sx = g.sx(), sz = g.sz();
    double acc[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;
        const int64_t es = s - A - B * sx - C * sz;
        if (!emask[es]) continue;
        const int cn = corner_of(A, B, C);
        const double sc = escale ? escale[es] : 1.0;
        double t[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t ns = es + corner_y(j) + corner_x(j) * sx + corner_z(j) * sz;
            const double u0 = U[ns], u1 = U[ns + S], u2 = U[ns + 2 * S];
#pragma unroll
            for (int a = 0; a < 6; ++a) {
                const double* m = c_mnodal + (6 * cn + a) * 24 + 3 * j;
                t[a] += m[0] * u0 + m[1] * u1 + m[2] * u2;
            }
        }
#pragma unroll
        for (int a = 0; a < 6; ++a) acc[a] += sc * t[a];
    }
    const double cnt = count[i];
#pragma unroll
    for (int a = 0; a < 6; ++a) out[6 * i + a] = acc[a] / cnt;
}

// One thread per solid voxel: mean of the 8 Gauss-point stresses D B u_e.
__global__ void __launch_bounds__(128) k_stress_voxel(Grid g, const int32_t* __restrict__ elem_slot,
                                                      const double* __restrict__ escale, int64_t ne,
                                                      const double* __restrict__ U, float* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int64_t es = elem_slot[e];
    const int64_t S = g.slots, sx = g.sx(), sz = g.sz();
    double u[24];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int64_t ns = es + corner_y(j) + corner_x(j) * sx + corner_z(j) * sz;
        u[3 * j] = U[ns];
        u[3 * j + 1] = U[ns + S];
        u[3 * j + 2] = U[ns + 2 * S];
    }
    const double sc = escale ? escale[es] : 1.0;
#pragma unroll
    for (int a = 0; a < 6; ++a) {
        double acc = 0;
        for (int gp = 0; gp < 8; ++gp) {
            const double* m = c_mgauss + (6 * gp + a) * 24;
            double t = 0;
#pragma unroll
            for (int k = 0; k < 24; ++k) t += m[k] * u[k];
            acc += t;
        }
        out[6 * e + a] = (float)(sc * acc / 8.0);
    }
}

void stress_dev(Model& M, const double* U, double* nodal, float* per_voxel) {
    Ctx& c = M.ctx;
    upload_stress(M);
    Level& l0 = M.levels[0];
    const double* esc = l0.escale64.as<double>();
    if (nodal) {
        k_stress_nodal<<<(unsigned)((l0.n_node + 127) / 128), 128, 0, c.stream>>>(
            l0.g, l0.emask.as<uint8_t>(), esc, l0.node_slot.as<int32_t>(), l0.node_count.as<double>(), l0.n_node, U,
            nodal);
        GMGS_LAUNCHED(c);
    }
    if (per_voxel) {
        k_stress_voxel<<<(unsigned)((l0.n_elem + 127) / 128), 128, 0, c.stream>>>(
            l0.g, l0.elem_slot.as<int32_t>(), esc, l0.n_elem, U, per_voxel);
        GMGS_LAUNCHED(c);
    }
}

// dJ/drho_e = -penal rho_e^(penal-1) lam_e^T Ke0 u_e, lam = u for compliance.
__global__ void __launch_bounds__(128) k_grad(Grid g, const int32_t* __restrict__ elem_slot, int64_t ne,
                                              const double* __restrict__ ke_rows, const double* __restrict__ rho,
                                              double penal, const double* __restrict__ U,
                                              const double* __restrict__ Lam, double* __restrict__ out) {
    __shared__ double K[KE];
    for (int i = threadIdx.x; i < KE; i += blockDim.x) K[i] = ke_rows[i];
    __syncthreads();
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int64_t es = elem_slot[e];
    const int64_t S = g.slots, sx = g.sx(), sz = g.sz();
    double u[24], l[24];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int64_t ns = es + corner_y(j) + corner_x(j) * sx + corner_z(j) * sz;
        u[3 * j] = U[ns]; u[3 * j + 1] = U[ns + S]; u[3 * j + 2] = U[ns + 2 * S];
        l[3 * j] = Lam[ns]; l[3 * j + 1] = Lam[ns + S]; l[3 * j + 2] = Lam[ns + 2 * S];
    }
    // ke_rows[r][c] = Ke0(c, r)
    double en = 0;
    for (int jc = 0; jc < 24; ++jc) {
        double t = 0;
#pragma unroll
        for (int i = 0; i < 24; ++i) t += l[i] * K[jc * 24 + i];
        en += t * u[jc];
    }
    const double r = rho[e];
    out[e] = -penal * pow(r, penal - 1.0) * en;
}

void grad_dev(Model& M, const double* U, const double* Lam, double* dJ) {
    Ctx& c = M.ctx;
    Level& l0 = M.levels[0];
    k_grad<<<(unsigned)((l0.n_elem + 127) / 128), 128, 0, c.stream>>>(
        l0.g, l0.elem_slot.as<int32_t>(), l0.n_elem, M.ke0_dev.as<double>(), M.rho.as<double>(), M.penal, U, Lam, dJ);
    GMGS_LAUNCHED(c);
}

}  // namespace gmgs
