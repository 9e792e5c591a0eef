// Post-processing on the solved displacement: nodal-averaged Cartesian stress
// (src/kernel/GetCartesianStress.m:11-41), per-voxel stress and the adjoint
// gradient with respect to the per-voxel stiffness scale (extension).
#include <algorithm>

#include "setup.cuh"

namespace gmgs {

// The reference recovers stresses with 48x24 matrices per element
// (GetCartesianStress.m:19-36): nodal = OTP D B (Gauss-point stresses
// extrapolated to the corners), per voxel (extension) = the mean of the 8
// Gauss-point stresses D B_g.  For a trilinear box element du/dx is constant in
// x and bilinear in y, z, so both maps reduce exactly to D B evaluated at a
// point: OTP D B = D B(corner k) and mean_g D B_g = D B(centre).  B at a corner
// is the one-sided edge difference along each axis, B at the centre the mean
// of the four parallel edge differences.  The kernels evaluate those
// differences directly: about 60 FP64 operations per node or voxel instead of
// 1152 FMAs (FP64 runs at 1/64 of the FP32 rate on this part), and no
// cancellation in sums of large terms.
struct StressCoef {
    double d11, d12, d44;   // isotropic D
    double ihx, ihy, ihz;   // reciprocal element edges
};

// g[i][j] = d u_i / d x_j (physical axes) -> [sxx syy szz syz szx sxy] * scale
__device__ __forceinline__ void hooke_apply(const StressCoef& c, const double g[3][3], double scale, double o[6]) {
    const double exx = g[0][0], eyy = g[1][1], ezz = g[2][2];
    o[0] = scale * (c.d11 * exx + c.d12 * (eyy + ezz));
    o[1] = scale * (c.d11 * eyy + c.d12 * (exx + ezz));
    o[2] = scale * (c.d11 * ezz + c.d12 * (exx + eyy));
    o[3] = scale * (c.d44 * (g[1][2] + g[2][1]));
    o[4] = scale * (c.d44 * (g[0][2] + g[2][0]));
    o[5] = scale * (c.d44 * (g[0][1] + g[1][0]));
}

// One thread per solid node.  The element at (A, B, C) = (y, x, z) offsets
// below the node uses the backward difference on an axis where its offset is
// 1 and the forward one where it is 0; physical y runs against the node
// y-index (DiscretizeDesignDomain.m:96).  The node value is the sum over its
// solid elements divided by their number (numNod2ElesVec_,
// GetCartesianStress.m:39-41).
__global__ void __launch_bounds__(128) k_stress_nodal(Grid g, StressCoef cf, const uint8_t* __restrict__ emask,
                                                      const double* __restrict__ escale,
                                                      const int32_t* __restrict__ node_slot, int64_t nn,
                                                      const double* __restrict__ U, double* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const int64_t s = node_slot[i];
    const int64_t S = g.slots, sx = g.sx(), sz = g.sz();
    double w[2][2][2];    // [A][B][C]: element weight (scale, 0 if void)
    int cnt = 0;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;
        const int64_t es = s - A - B * sx - C * sz;
        const bool solid = chk::ld(emask, es, S, chk::STRESS_U) != 0;
        cnt += solid;
        w[A][B][C] = solid ? (escale ? chk::ld(escale, es, S, chk::STRESS_U) : 1.0) : 0.0;
    }
    // per axis: total weight of the elements on the forward (0) and backward (1) side
    double wy[2], wx[2], wz[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        wy[k] = (w[k][0][0] + w[k][1][0]) + (w[k][0][1] + w[k][1][1]);
        wx[k] = (w[0][k][0] + w[1][k][0]) + (w[0][k][1] + w[1][k][1]);
        wz[k] = (w[0][0][k] + w[1][0][k]) + (w[0][1][k] + w[1][1][k]);
    }
    double gr[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int64_t b = c * S + s;
        auto u = [&](int64_t off) { return chk::ld(U, b + off, 3 * S, chk::STRESS_U); };
        const double u0 = u(0);
        gr[c][0] = (wx[0] * (u(sx) - u0) + wx[1] * (u0 - u(-sx))) * cf.ihx;
        gr[c][1] = -(wy[0] * (u(1) - u0) + wy[1] * (u0 - u(-1))) * cf.ihy;
        gr[c][2] = (wz[0] * (u(sz) - u0) + wz[1] * (u0 - u(-sz))) * cf.ihz;
    }
    double o[6];
    hooke_apply(cf, gr, 1.0 / (double)cnt, o);
#pragma unroll
    for (int a = 0; a < 6; ++a) chk::st(out, 6 * i + a, 6 * nn, chk::STRESS_OUT, o[a]);
}

// One thread per solid voxel: D B(centre) u_e times the voxel's scale.
__global__ void __launch_bounds__(128) k_stress_voxel(Grid g, StressCoef cf, const int32_t* __restrict__ elem_slot,
                                                      const double* __restrict__ escale, int64_t ne,
                                                      const double* __restrict__ U, float* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int64_t es = elem_slot[e];
    const int64_t S = g.slots, sx = g.sx(), sz = g.sz();
    double gr[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double u[2][2][2];    // [y][x][z] offsets
#pragma unroll
        for (int j = 0; j < 8; ++j)
            u[j & 1][(j >> 1) & 1][j >> 2] =
                chk::ld(U, c * S + es + (j & 1) + ((j >> 1) & 1) * sx + (j >> 2) * sz, 3 * S, chk::STRESS_U);
        const double dx = ((u[0][1][0] - u[0][0][0]) + (u[1][1][0] - u[1][0][0])) +
                          ((u[0][1][1] - u[0][0][1]) + (u[1][1][1] - u[1][0][1]));
        const double dy = ((u[1][0][0] - u[0][0][0]) + (u[1][1][0] - u[0][1][0])) +
                          ((u[1][0][1] - u[0][0][1]) + (u[1][1][1] - u[0][1][1]));
        const double dz = ((u[0][0][1] - u[0][0][0]) + (u[1][0][1] - u[1][0][0])) +
                          ((u[0][1][1] - u[0][1][0]) + (u[1][1][1] - u[1][1][0]));
        gr[c][0] = 0.25 * dx * cf.ihx;
        gr[c][1] = -0.25 * dy * cf.ihy;
        gr[c][2] = 0.25 * dz * cf.ihz;
    }
    double o[6];
    hooke_apply(cf, gr, escale ? chk::ld(escale, es, S, chk::STRESS_U) : 1.0, o);
#pragma unroll
    for (int a = 0; a < 6; ++a) chk::st(out, 6 * e + a, 6 * ne, chk::STRESS_OUT, (float)o[a]);
}

// ---------------------------------------------------------------------------
// Mixed path: the same stress maps in FP32 arithmetic on a double-float copy
// of U.  GB300 runs FP64 arithmetic and FP32<->FP64 conversions at about 2
// lanes per clock per SM (measured), 1/40 of its FP32 rate, and the FP64
// kernels above spend about 190 such operations per node and voxel.  Here U is
// split once into hi = fl32(u) and lo = fl32(u - hi) (one FP64 subtraction per
// DOF; the conversions on the integer pipe, exact), and every edge difference
// is formed as (hi_j - hi_0) + (lo_j - lo_0): relative error about 2^-24 of
// the difference itself, so the stresses keep FP32 relative accuracy.
// ---------------------------------------------------------------------------
__global__ void k_split_hilo(int64_t n, const double* __restrict__ U, float* __restrict__ hi, float* __restrict__ lo) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double u = chk::ld(U, i, n, chk::STRESS_U);
        const float h = d2f_int(u);
        chk::st(hi, i, n, chk::STRESS_U, h);
        chk::st(lo, i, n, chk::STRESS_U, d2f_int(u - f2d_int(h)));
    }
}

struct StressCoef32 {
    float d11, d12, d44, ihx, ihy, ihz;
};
__device__ __forceinline__ void hooke_apply32(const StressCoef32& c, const float g[3][3], float scale, float o[6]) {
    const float exx = g[0][0], eyy = g[1][1], ezz = g[2][2];
    o[0] = scale * (c.d11 * exx + c.d12 * (eyy + ezz));
    o[1] = scale * (c.d11 * eyy + c.d12 * (exx + ezz));
    o[2] = scale * (c.d11 * ezz + c.d12 * (exx + eyy));
    o[3] = scale * (c.d44 * (g[1][2] + g[2][1]));
    o[4] = scale * (c.d44 * (g[0][2] + g[2][0]));
    o[5] = scale * (c.d44 * (g[0][1] + g[1][0]));
}

// k_stress_nodal in FP32 on (hi, lo); the FP64 output is the exact widening
__global__ void __launch_bounds__(128) k_stress_nodal32(Grid g, StressCoef32 cf, const uint8_t* __restrict__ emask,
                                                        const float* __restrict__ escale,
                                                        const int32_t* __restrict__ node_slot, int64_t nn,
                                                        const float* __restrict__ hi, const float* __restrict__ lo,
                                                        double* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const int s = chk::ld(node_slot, i, nn, chk::STRESS_U);
    const int S = (int)g.slots, sx = g.py, sz = g.py * g.px;
    float w[2][2][2];
    int cnt = 0;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;
        const int es = s - A - B * sx - C * sz;
        const bool solid = chk::ld(emask, es, S, chk::STRESS_U) != 0;
        cnt += solid;
        w[A][B][C] = solid ? (escale ? chk::ld(escale, es, S, chk::STRESS_U) : 1.f) : 0.f;
    }
    float wy[2], wx[2], wz[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        wy[k] = (w[k][0][0] + w[k][1][0]) + (w[k][0][1] + w[k][1][1]);
        wx[k] = (w[0][k][0] + w[1][k][0]) + (w[0][k][1] + w[1][k][1]);
        wz[k] = (w[0][0][k] + w[1][0][k]) + (w[0][1][k] + w[1][1][k]);
    }
    float gr[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int b = c * S + s;
        const float h0 = chk::ld(hi, b, 3ll * S, chk::STRESS_U), l0 = chk::ld(lo, b, 3ll * S, chk::STRESS_U);
        auto d = [&](int off) {   // u(s + off) - u(s)
            return (chk::ld(hi, b + off, 3ll * S, chk::STRESS_U) - h0) + (chk::ld(lo, b + off, 3ll * S, chk::STRESS_U) - l0);
        };
        gr[c][0] = (wx[0] * d(sx) - wx[1] * d(-sx)) * cf.ihx;
        gr[c][1] = -(wy[0] * d(1) - wy[1] * d(-1)) * cf.ihy;
        gr[c][2] = (wz[0] * d(sz) - wz[1] * d(-sz)) * cf.ihz;
    }
    float o[6];
    hooke_apply32(cf, gr, 1.f / (float)cnt, o);
#pragma unroll
    for (int a = 0; a < 6; ++a) chk::st(out, 6 * i + a, 6 * nn, chk::STRESS_OUT, f2d_int(o[a]));
}

// k_stress_voxel in FP32 on (hi, lo): differences against the element's origin node
__global__ void __launch_bounds__(128) k_stress_voxel32(Grid g, StressCoef32 cf, const int32_t* __restrict__ elem_slot,
                                                        const float* __restrict__ escale, int64_t ne,
                                                        const float* __restrict__ hi, const float* __restrict__ lo,
                                                        float* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int es = chk::ld(elem_slot, e, ne, chk::STRESS_U);
    const int S = (int)g.slots, sx = g.py, sz = g.py * g.px;
    float gr[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int b = c * S + es;
        const float h0 = chk::ld(hi, b, 3ll * S, chk::STRESS_U), l0 = chk::ld(lo, b, 3ll * S, chk::STRESS_U);
        float u[2][2][2];    // [y][x][z] offsets: u - u(origin)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int off = (j & 1) + ((j >> 1) & 1) * sx + (j >> 2) * sz;
            u[j & 1][(j >> 1) & 1][j >> 2] =
                j ? (chk::ld(hi, b + off, 3ll * S, chk::STRESS_U) - h0) + (chk::ld(lo, b + off, 3ll * S, chk::STRESS_U) - l0)
                  : 0.f;
        }
        const float dx = ((u[0][1][0] - u[0][0][0]) + (u[1][1][0] - u[1][0][0])) +
                         ((u[0][1][1] - u[0][0][1]) + (u[1][1][1] - u[1][0][1]));
        const float dy = ((u[1][0][0] - u[0][0][0]) + (u[1][1][0] - u[0][1][0])) +
                         ((u[1][0][1] - u[0][0][1]) + (u[1][1][1] - u[0][1][1]));
        const float dz = ((u[0][0][1] - u[0][0][0]) + (u[1][0][1] - u[1][0][0])) +
                         ((u[0][1][1] - u[0][1][0]) + (u[1][1][1] - u[1][1][0]));
        gr[c][0] = 0.25f * dx * cf.ihx;
        gr[c][1] = -0.25f * dy * cf.ihy;
        gr[c][2] = 0.25f * dz * cf.ihz;
    }
    float o[6];
    hooke_apply32(cf, gr, escale ? chk::ld(escale, es, S, chk::STRESS_U) : 1.f, o);
#pragma unroll
    for (int a = 0; a < 6; ++a) chk::st(out, 6 * e + a, 6 * ne, chk::STRESS_OUT, o[a]);
}

void stress_dev(Model& M, const double* U, double* nodal, float* per_voxel) {
    Ctx& c = M.ctx;
    double k[6];
    stress_coefficients(M.prm.youngs_modulus, M.prm.poisson_ratio, M.ele, k);
    const StressCoef cf{k[0], k[1], k[2], k[3], k[4], k[5]};
    Level& l0 = M.levels[0];
    const double* esc = l0.escale64.as<double>();
    // mixed path: FP32 maps on the double-float split of U, held in two FP32
    // work vectors of the PCG (idle between solves)
    const size_t n3 = 3 * (size_t)l0.g.slots;
    if (M.prm.precision == GMGS_MIXED && M.cg_q32.bytes >= n3 * 4 && M.cg_z32.bytes >= n3 * 4 &&
        (!esc || l0.escale32.p)) {
        float* hi = M.cg_q32.as<float>();
        float* lo = M.cg_z32.as<float>();
        const int blocks = (int)std::min<int64_t>((int64_t)(n3 + 255) / 256, (int64_t)c.num_sms * 16);
        k_split_hilo<<<blocks, 256, 0, c.stream>>>((int64_t)n3, U, hi, lo);
        GMGS_LAUNCHED(c);
        const StressCoef32 cf32{(float)k[0], (float)k[1], (float)k[2], (float)k[3], (float)k[4], (float)k[5]};
        const float* esc32 = esc ? l0.escale32.as<float>() : nullptr;
        if (nodal) {
            k_stress_nodal32<<<(unsigned)((l0.n_node + 127) / 128), 128, 0, c.stream>>>(
                l0.g, cf32, l0.emask.as<uint8_t>(), esc32, l0.node_slot.as<int32_t>(), l0.n_node, hi, lo, nodal);
            GMGS_LAUNCHED(c);
        }
        if (per_voxel) {
            k_stress_voxel32<<<(unsigned)((l0.n_elem + 127) / 128), 128, 0, c.stream>>>(
                l0.g, cf32, l0.elem_slot.as<int32_t>(), esc32, l0.n_elem, hi, lo, per_voxel);
            GMGS_LAUNCHED(c);
        }
        return;
    }
    if (nodal) {
        k_stress_nodal<<<(unsigned)((l0.n_node + 127) / 128), 128, 0, c.stream>>>(
            l0.g, cf, l0.emask.as<uint8_t>(), esc, l0.node_slot.as<int32_t>(), l0.n_node, U, nodal);
        GMGS_LAUNCHED(c);
    }
    if (per_voxel) {
        k_stress_voxel<<<(unsigned)((l0.n_elem + 127) / 128), 128, 0, c.stream>>>(
            l0.g, cf, l0.elem_slot.as<int32_t>(), esc, l0.n_elem, U, per_voxel);
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
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            u[3 * j + c] = chk::ld(U, ns + c * S, 3 * S, chk::GRAD);
            l[3 * j + c] = chk::ld(Lam, ns + c * S, 3 * S, chk::GRAD);
        }
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
