// Tiled FP32 operator kernels of the mixed-precision path.
//
// One CTA owns a 32 x 8 column of nodes (y fastest) and streams it through z
// with a three-plane ring of the input field plus a one-node halo in shared
// memory; the field is computed while staging from the kernel's inputs (the
// Jacobi step omega*D^-1 r, or the CG direction z + beta p), so no
// intermediate vector goes through HBM.
//
// Interior nodes (all 8 surrounding elements carry the level's uniform
// matrix) use the assembled 27-point stencil in second-difference form
//     y = s * sum_{d in H} S(d) [(v(n+d) - v(n)) + (v(n-d) - v(n))]
// over the 13 half offsets H (S(-d) = S(d) on the uniform grid and
// sum_d S(d) = 0, rigid translations).  For smooth fields both differences
// are exact in FP32 (Sterbenz), so the product keeps FP32 relative accuracy
// where the plain sum sum_d S(d) v(n+d) would cancel catastrophically.
// Boundary nodes sum their solid elements' rows in first-difference form
// sum_e sum_j K_e[c, j] (v_j - v_n) (each element matrix annihilates
// translations), with per-element matrices where the level stores them
// (the reference's AtX states 0/1/2, src/kernel/AtX.m:1-58).
// Fixed DOF rows are zeroed (AtX.m:57).
#include "fine.cuh"

namespace gmgs {

constexpr int TY = 32, TX = 8;
constexpr int HY = TY + 2, HX = TX + 2;
constexpr int NT = TY * TX;

// displacement component a (0 = x, 1 = y, 2 = z) of stencil offset k = (dz+1)*9 + (dx+1)*3 + (dy+1)
__host__ __device__ constexpr int off_y(int k) { return k % 3 - 1; }
__host__ __device__ constexpr int off_x(int k) { return (k / 3) % 3 - 1; }
__host__ __device__ constexpr int off_z(int k) { return k / 9 - 1; }
__host__ __device__ constexpr int off_comp(int k, int a) { return a == 0 ? off_x(k) : (a == 1 ? off_y(k) : off_z(k)); }
// structural non-zeros of the assembled interior block S(d)[a][b]
__host__ __device__ constexpr bool s_nonzero(int k, int a, int b) {
    return a == b || (off_comp(k, a) != 0 && off_comp(k, b) != 0);
}

// ---------------------------------------------------------------------------
// host: assembled interior stencil from the element matrix (row = output DOF)
// ---------------------------------------------------------------------------
void make_stencil(const double* ke_rows, Coef32& cf) {
    double S[27][9] = {};
    for (int k = 0; k < 27; ++k) {
        const int dy = off_y(k), dx = off_x(k), dz = off_z(k);
        for (int e = 0; e < 8; ++e) {
            const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;     // node = element origin + (A, B, C)
            const int my = A + dy, mx = B + dx, mz = C + dz;       // neighbour relative to the origin
            if (my < 0 || my > 1 || mx < 0 || mx > 1 || mz < 0 || mz > 1) continue;
            const int cn = corner_of(A, B, C), cm = corner_of(my, mx, mz);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) S[k][3 * a + b] += ke_rows[(3 * cn + a) * 24 + 3 * cm + b];
        }
    }
    for (int k = 0; k < 27; ++k)
        for (int i = 0; i < 9; ++i) cf.S[k * 9 + i] = (float)S[k][i];
    for (int i = 0; i < KE; ++i) cf.K[i] = (float)ke_rows[i];
}

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool in_halo_grid(const Grid& g, int iy, int ix, int iz) {
    return iy >= -1 && ix >= -1 && iz >= -1 && iy <= g.ny + 1 && ix <= g.nx + 1 && iz <= g.nz + 1;
}

__device__ __forceinline__ double block_sum_d(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int w = tid >> 5, l = tid & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    v = 0;
    if (w == 0) {
        v = l < NT / 32 ? sh[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;   // valid in thread 0
}

// deterministic grid reduction: partial per block, the last block sums them in order
__device__ void grid_dot_finish(double v, const DotOut& d, double* sh) {
    __shared__ bool last;
    v = block_sum_d(v, sh);
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
    const unsigned b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    if (tid == 0) {
        d.partials[b] = v;
        __threadfence();
        last = atomicAdd(d.ticket, 1u) == nb - 1;
    }
    __syncthreads();
    if (last) {
        __threadfence();
        double t = 0;
        for (unsigned i = tid; i < nb; i += NT) t += ((volatile double*)d.partials)[i];
        t = block_sum_d(t, sh);
        if (tid == 0) {
            *d.out = t;
            *d.ticket = 0;
        }
    }
}

// ---------------------------------------------------------------------------
// the fused streaming kernel
//
// A CTA of 32 x 8 threads owns a 32 x 8 column of nodes and walks it through
// ZC planes in z.  Shared memory holds a ring of three (32+2) x (8+2) planes
// of the input field; the plane two steps ahead is loaded (and transformed)
// into registers while the current plane is computed, so global loads
// overlap the stencil arithmetic.
// ---------------------------------------------------------------------------
constexpr int PLANE = HY * HX;                 // 340 points
constexpr int PPT = (PLANE + NT - 1) / NT;     // points per thread and plane

struct PlaneRegs {
    float v[PPT][3];
};

struct Scalars {
    float beta;      // FM_CG_DIRECTION
    double alpha;    // FM_CG_UPDATE_JACOBI
};

template <int MODE>
__device__ __forceinline__ void fetch_plane(const Grid& g, const FineArgs& a, const Scalars& sc, int y0, int x0, int iz,
                                            int tid, PlaneRegs& pr) {
    const int64_t S = g.slots;
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        const int t = tid + k * NT;
        const int ly = t % HY, lx = t / HY;
        const int iy = y0 - 1 + ly, ix = x0 - 1 + lx;
        float v[3] = {0.f, 0.f, 0.f};
        if (t < PLANE && in_halo_grid(g, iy, ix, iz)) {
            const int64_t s = g.slot(iy, ix, iz);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const int64_t i = s + c * S;
                if (MODE == FM_PLAIN) {
                    v[c] = a.v[i];
                } else if (MODE == FM_VCYCLE_DOWN) {
                    v[c] = a.r32[i] * a.wdinv[i];
                } else if (MODE == FM_CG_UPDATE_JACOBI) {
                    const double rm = a.first ? a.r64[i] : a.r64[i] - sc.alpha * (double)a.q32[i];
                    v[c] = (float)rm * a.wdinv[i];
                } else {   // FM_CG_DIRECTION
                    v[c] = a.first ? a.z32[i] : fmaf(sc.beta, a.pold[i], a.z32[i]);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) pr.v[k][c] = v[c];
    }
}

__device__ __forceinline__ void store_plane(float* __restrict__ ring, int tid, const PlaneRegs& pr) {
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        const int t = tid + k * NT;
        if (t < PLANE) {
#pragma unroll
            for (int c = 0; c < 3; ++c) ring[c * PLANE + t] = pr.v[k][c];
        }
    }
}

// interior node, second-difference form; P[0..2] = planes z-1, z, z+1, p = in-plane index
__device__ __forceinline__ void interior_s(const Coef32& cf, const float* const P[3], int p, float acc[3]) {
    const float c[3] = {P[1][p], P[1][p + PLANE], P[1][p + 2 * PLANE]};
    acc[0] = acc[1] = acc[2] = 0.f;
#pragma unroll
    for (int k = 14; k < 27; ++k) {
        const int o = off_y(k) + off_x(k) * HY;
        const float* up = P[1 + off_z(k)];
        const float* dn = P[1 - off_z(k)];
        float d[3];
#pragma unroll
        for (int b = 0; b < 3; ++b) d[b] = (up[p + o + b * PLANE] - c[b]) + (dn[p - o + b * PLANE] - c[b]);
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
                if (s_nonzero(k, a, b)) acc[a] = fmaf(cf.S[k * 9 + 3 * a + b], d[b], acc[a]);
    }
}

template <int CI>
__device__ __forceinline__ void elem_rows_s(const float* __restrict__ K, float s, const float* const P[3], int p, int A,
                                            int B, int C, const float c[3], float acc[3]) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (j == CI) continue;
        const int dy = corner_y(j) - A, dx = corner_x(j) - B, dz = corner_z(j) - C;
        const float* pl = P[1 + dz];
        const int q = p + dy + dx * HY;
        const float d0 = pl[q] - c[0], d1 = pl[q + PLANE] - c[1], d2 = pl[q + 2 * PLANE] - c[2];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int r = (3 * CI + a) * 24 + 3 * j;
            float t = K[r] * d0;
            t = fmaf(K[r + 1], d1, t);
            t = fmaf(K[r + 2], d2, t);
            acc[a] = fmaf(s, t, acc[a]);
        }
    }
}

template <int E>
__device__ __forceinline__ void boundary_elem_s(const FineLevel& L, const Coef32& cf, const float* const P[3], int p,
                                                int64_t n, const float c[3], float acc[3]) {
    constexpr int A = E & 1, B = (E >> 1) & 1, C = E >> 2;
    constexpr int CI = corner_of(A, B, C);
    const int64_t es = n - A - B * L.g.sx() - C * L.g.sz();
    if (!L.emask[es]) return;
    const int t = L.etype ? L.etype[es] : 0;
    if (t > 0) {
        elem_rows_s<CI>(L.Ks + (int64_t)(t - 1) * KE, 1.0f, P, p, A, B, C, c, acc);
    } else {
        const float s = L.escale ? L.kscale * L.escale[es] : L.kscale;
        elem_rows_s<CI>(cf.K, s, P, p, A, B, C, c, acc);
    }
}

__device__ __noinline__ void boundary_s(const FineLevel& L, const Coef32& cf, const float* const P[3], int p, int64_t n,
                                        float acc[3]) {
    const float c[3] = {P[1][p], P[1][p + PLANE], P[1][p + 2 * PLANE]};
    acc[0] = acc[1] = acc[2] = 0.f;
    boundary_elem_s<0>(L, cf, P, p, n, c, acc);
    boundary_elem_s<1>(L, cf, P, p, n, c, acc);
    boundary_elem_s<2>(L, cf, P, p, n, c, acc);
    boundary_elem_s<3>(L, cf, P, p, n, c, acc);
    boundary_elem_s<4>(L, cf, P, p, n, c, acc);
    boundary_elem_s<5>(L, cf, P, p, n, c, acc);
    boundary_elem_s<6>(L, cf, P, p, n, c, acc);
    boundary_elem_s<7>(L, cf, P, p, n, c, acc);
}

template <int MODE>
__global__ void __launch_bounds__(NT, 3) k_fine(FineLevel L, const __grid_constant__ Coef32 cf, FineArgs a, int zc) {
    __shared__ float ring[3][3 * PLANE];
    __shared__ double sh[32];
    const Grid& g = L.g;
    const int64_t S = g.slots;
    const int y0 = blockIdx.x * TY, x0 = blockIdx.y * TX;
    const int zb = blockIdx.z * zc;
    const int ze = min(zb + zc, g.nz + 1);        // node planes [zb, ze)
    const int tid = threadIdx.x + threadIdx.y * TY;

    Scalars sc;
    sc.beta = 0.f;
    sc.alpha = 0.0;
    if (MODE == FM_CG_DIRECTION && !a.first) sc.beta = (float)(a.scal[a.cur] / a.scal[a.cur ^ 1]);
    if (MODE == FM_CG_UPDATE_JACOBI && !a.first) sc.alpha = a.scal[a.cur] / a.scal[2];

    PlaneRegs pr;
    fetch_plane<MODE>(g, a, sc, y0, x0, zb - 1, tid, pr);
    store_plane(ring[(zb - 1 + 3) % 3], tid, pr);
    fetch_plane<MODE>(g, a, sc, y0, x0, zb, tid, pr);
    store_plane(ring[zb % 3], tid, pr);
    fetch_plane<MODE>(g, a, sc, y0, x0, zb + 1, tid, pr);

    const int iy = y0 + threadIdx.x, ix = x0 + threadIdx.y;
    const bool own = iy <= g.ny && ix <= g.nx;
    const int p = (threadIdx.x + 1) + (threadIdx.y + 1) * HY;
    double dot = 0.0;
#pragma unroll 1
    for (int iz = zb; iz < ze; ++iz) {
        store_plane(ring[(iz + 1) % 3], tid, pr);
        __syncthreads();
        if (iz + 2 <= g.nz + 1) fetch_plane<MODE>(g, a, sc, y0, x0, iz + 2, tid, pr);
        const float* const P[3] = {ring[(iz + 2) % 3], ring[iz % 3], ring[(iz + 1) % 3]};
        if (own) {
            const int64_t n = g.slot(iy, ix, iz);
            const uint8_t f = L.nflag[n];
            if (f & NF_SOLID) {
                float y[3];
                if (f & NF_INTERIOR) {
                    interior_s(cf, P, p, y);
                    y[0] *= L.kscale; y[1] *= L.kscale; y[2] *= L.kscale;
                } else {
                    boundary_s(L, cf, P, p, n, y);
                }
                if (f & NF_FIX_X) y[0] = 0.f;
                if (f & NF_FIX_Y) y[1] = 0.f;
                if (f & NF_FIX_Z) y[2] = 0.f;
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    const int64_t i = n + b * S;
                    const float v = P[1][p + b * PLANE];
                    if (MODE == FM_PLAIN) {
                        a.out32[i] = y[b];
                    } else if (MODE == FM_VCYCLE_DOWN) {
                        a.out32[i] = a.r32[i] - y[b];                    // r' = r - A (omega D^-1 r)
                    } else if (MODE == FM_CG_UPDATE_JACOBI) {
                        // previous iteration's update x += alpha p, r -= alpha q (CG_solver.m:32-33),
                        // then this iteration's Jacobi step (CG_solver.m:18-19), its dx kept pending
                        const double rm = a.first ? a.r64[i] : a.r64[i] - sc.alpha * (double)a.q32[i];
                        if (!a.first) a.x64[i] = (a.x64[i] + (double)a.dxp[i]) + sc.alpha * (double)a.pold[i];
                        a.dxp[i] = v;
                        const double rn = rm - (double)y[b];
                        a.r64out[i] = rn;
                        a.r32out[i] = (float)rn;
                        dot += rm * rm;
                    } else {
                        a.pout[i] = v;
                        a.out32[i] = y[b];                               // q = A p
                        dot += (double)v * (double)y[b];
                    }
                }
            }
        }
        __syncthreads();
    }
    if (MODE == FM_CG_DIRECTION || MODE == FM_CG_UPDATE_JACOBI) grid_dot_finish(dot, a.dot, sh);
}

static int pick_zc(const Grid& g, const Ctx& c) {
    const int64_t cols = (int64_t)((g.ny + 1 + TY - 1) / TY) * ((g.nx + 1 + TX - 1) / TX);
    const int64_t want = (int64_t)c.num_sms * 3 * 6;      // ~6 waves of resident CTAs
    int64_t zc = (cols * (g.nz + 1) + want - 1) / want;
    if (zc < 4) zc = 4;
    if (zc > 64) zc = 64;
    return (int)zc;
}

int fine_grid_blocks(const Grid& g) {
    // upper bound over the z-chunk choices (zc >= 4)
    return ((g.ny + 1 + TY - 1) / TY) * ((g.nx + 1 + TX - 1) / TX) * ((g.nz + 1 + 3) / 4);
}

template <int MODE>
void launch_fine(Ctx& c, const FineLevel& L, const Coef32& cf, const FineArgs& a) {
    const int zc = pick_zc(L.g, c);
    dim3 grid((L.g.ny + 1 + TY - 1) / TY, (L.g.nx + 1 + TX - 1) / TX, (L.g.nz + 1 + zc - 1) / zc);
    k_fine<MODE><<<grid, dim3(TY, TX, 1), 0, c.stream>>>(L, cf, a, zc);
    GMGS_LAUNCHED(c);
}
template void launch_fine<FM_PLAIN>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine<FM_VCYCLE_DOWN>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine<FM_CG_UPDATE_JACOBI>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine<FM_CG_DIRECTION>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);

// ---------------------------------------------------------------------------
// V-cycle up-sweep in FP32 with omega D^-1 precomputed (Vcycle.m:29-32):
// x_f = (w r + P x_c) + w r', optionally the finest-level fixed DOFs zeroed
// and the CG dot r64 . x_f accumulated (CG_solver.m:26).
// ---------------------------------------------------------------------------
template <bool DOT>
__global__ void __launch_bounds__(256) k_up32(Grid gf, Grid gc, const uint8_t* __restrict__ nflag,
                                              const float* __restrict__ wdinv, const float* __restrict__ r,
                                              const float* __restrict__ rp, const float* __restrict__ xc,
                                              float* __restrict__ xf, int zero_fixed, const double* __restrict__ r64,
                                              DotOut dout) {
    __shared__ double sh[32];
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y * blockDim.y + threadIdx.y;
    const int iz = blockIdx.z;
    double dot = 0.0;
    if (iy <= gf.ny && ix <= gf.nx) {
        const int64_t fs = gf.slot(iy, ix, iz);
        const uint8_t fl = nflag[fs];
        if (fl & NF_SOLID) {
            const int64_t Sf = gf.slots, Sc = gc.slots;
            const int Iy = iy >> 1, Ix = ix >> 1, Iz = iz >> 1;
            const int oy = iy & 1, ox = ix & 1, oz = iz & 1;
            const int64_t c0 = gc.slot(Iy, Ix, Iz);
            const int64_t csx = gc.sx(), csz = gc.sz();
            const float w = (oy ? 0.5f : 1.f) * (ox ? 0.5f : 1.f) * (oz ? 0.5f : 1.f);
#pragma unroll
            for (int comp = 0; comp < 3; ++comp) {
                const float* x = xc + comp * Sc;
                float v = 0.f;
                for (int cz = 0; cz <= oz; ++cz)
                    for (int b = 0; b <= ox; ++b)
                        for (int a = 0; a <= oy; ++a) v += x[c0 + a + b * csx + cz * csz];
                const int64_t i = fs + comp * Sf;
                const float wd = wdinv[i];
                float out = (wd * r[i] + w * v) + wd * rp[i];
                if (zero_fixed && (fl & (NF_FIX_X << comp))) out = 0.f;
                xf[i] = out;
                if (DOT) dot += r64[i] * (double)out;
            }
        }
    }
    if (DOT) {
        // reuse the tiled reduction (blockDim 32 x 8 = NT)
        grid_dot_finish(dot, dout, sh);
    }
}

void launch_up32(Ctx& c, const Grid& gf, const Grid& gc, const uint8_t* nflag, const float* wdinv, const float* r,
                 const float* rp, const float* xc, float* xf, bool zero_fixed, const double* r64, const DotOut* dot) {
    dim3 blk(32, 8, 1);
    dim3 grid((gf.ny + 1 + 31) / 32, (gf.nx + 1 + 7) / 8, gf.nz + 1);
    if (dot) {
        k_up32<true><<<grid, blk, 0, c.stream>>>(gf, gc, nflag, wdinv, r, rp, xc, xf, zero_fixed, r64, *dot);
    } else {
        k_up32<false><<<grid, blk, 0, c.stream>>>(gf, gc, nflag, wdinv, r, rp, xc, xf, zero_fixed, nullptr, DotOut{});
    }
    GMGS_LAUNCHED(c);
}

int up32_grid_blocks(const Grid& gf) { return ((gf.ny + 1 + 31) / 32) * ((gf.nx + 1 + 7) / 8) * (gf.nz + 1); }

// ---------------------------------------------------------------------------
// CG update (CG_solver.m:31-35): x += alpha p, r -= alpha q, r.r
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_xr32(int64_t n, double* __restrict__ x, double* __restrict__ r,
                                              const float* __restrict__ p, const float* __restrict__ q,
                                              const double* __restrict__ scal, int cur, DotOut dout) {
    __shared__ double sh[32];
    __shared__ bool last;
    const double alpha = scal[cur] / scal[2];
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = x[i] + alpha * (double)p[i];
        const double rn = r[i] - alpha * (double)q[i];
        r[i] = rn;
        acc += rn * rn;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    }
    if (threadIdx.x == 0) {
        dout.partials[blockIdx.x] = acc;
        __threadfence();
        last = atomicAdd(dout.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) {
        __threadfence();
        double t = 0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) t += ((volatile double*)dout.partials)[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        __syncthreads();
        if (l == 0) sh[w] = t;
        __syncthreads();
        if (threadIdx.x < 32) {
            t = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (threadIdx.x == 0) {
                *dout.out = t;
                *dout.ticket = 0;
            }
        }
    }
}

void launch_xr32(Ctx& c, int64_t n, double* x, double* r, const float* p, const float* q, const double* scal, int cur,
                 const DotOut& d, int blocks) {
    k_xr32<<<blocks, 256, 0, c.stream>>>(n, x, r, p, q, scal, cur, d);
    GMGS_LAUNCHED(c);
}

// omega / diag in FP32 (0 where the diagonal is 0)
__global__ void k_wdinv(int64_t n, const double* __restrict__ d, double omega, float* __restrict__ w) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        w[i] = d[i] != 0.0 ? (float)(omega / d[i]) : 0.f;
}
void launch_wdinv(Ctx& c, int64_t n, const double* d, double omega, float* w) {
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)c.num_sms * 16);
    k_wdinv<<<blocks, 256, 0, c.stream>>>(n, d, omega, w);
    GMGS_LAUNCHED(c);
}

}  // namespace gmgs
