// Tiled FP32 operator kernels of the mixed-precision path.
//
// One CTA owns a 32 x 8 x 4 block of nodes (y fastest) and stages the input
// field on the block plus a one-node halo (34 x 10 x 6 points, 3 components,
// 24 KB) in shared memory; the field is computed while staging from the
// kernel's inputs (the Jacobi step omega*D^-1 r, or the CG direction
// z + beta p), so no intermediate vector goes through HBM.
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

constexpr int TY = 32, TX = 8, TZ = 4;
constexpr int HY = TY + 2, HX = TX + 2, HZ = TZ + 2;
constexpr int TILE = HY * HX * HZ;
constexpr int NT = TY * TX;
constexpr int SX = HY, SZ = HY * HX;

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

// interior node: second-difference form of the uniform stencil
__device__ __forceinline__ void interior(const Coef32& cf, const float* __restrict__ sv, int p, float& y0, float& y1,
                                         float& y2) {
    const float c[3] = {sv[p], sv[p + TILE], sv[p + 2 * TILE]};
    float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 14; k < 27; ++k) {
        const int o = off_y(k) + off_x(k) * SX + off_z(k) * SZ;
        float d[3];
#pragma unroll
        for (int b = 0; b < 3; ++b) d[b] = (sv[p + o + b * TILE] - c[b]) + (sv[p - o + b * TILE] - c[b]);
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
                if (s_nonzero(k, a, b)) acc[a] = fmaf(cf.S[k * 9 + 3 * a + b], d[b], acc[a]);
    }
    y0 = acc[0]; y1 = acc[1]; y2 = acc[2];
}

// one element's rows for the node at local corner CI, first-difference form
template <int CI, bool GLOBALK>
__device__ __forceinline__ void elem_rows(const float* __restrict__ K, float s, const float* __restrict__ sv, int pe,
                                          const float c[3], float acc[3]) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (j == CI) continue;
        const int q = pe + corner_y(j) + corner_x(j) * SX + corner_z(j) * SZ;
        const float d0 = sv[q] - c[0], d1 = sv[q + TILE] - c[1], d2 = sv[q + 2 * TILE] - c[2];
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
__device__ __forceinline__ void boundary_elem(const FineLevel& L, const Coef32& cf, const float* __restrict__ sv, int p,
                                              int64_t n, const float c[3], float acc[3]) {
    constexpr int A = E & 1, B = (E >> 1) & 1, C = E >> 2;
    constexpr int CI = corner_of(A, B, C);
    const int64_t es = n - A - B * L.g.sx() - C * L.g.sz();
    if (!L.emask[es]) return;
    const int pe = p - A - B * SX - C * SZ;      // element origin in the tile
    const int t = L.etype ? L.etype[es] : 0;
    if (t > 0) {
        elem_rows<CI, true>(L.Ks + (int64_t)(t - 1) * KE, 1.0f, sv, pe, c, acc);
    } else {
        const float s = L.escale ? L.kscale * L.escale[es] : L.kscale;
        elem_rows<CI, false>(cf.K, s, sv, pe, c, acc);
    }
}

__device__ __forceinline__ void boundary(const FineLevel& L, const Coef32& cf, const float* __restrict__ sv, int p,
                                         int64_t n, float& y0, float& y1, float& y2) {
    const float c[3] = {sv[p], sv[p + TILE], sv[p + 2 * TILE]};
    float acc[3] = {0.f, 0.f, 0.f};
    boundary_elem<0>(L, cf, sv, p, n, c, acc);
    boundary_elem<1>(L, cf, sv, p, n, c, acc);
    boundary_elem<2>(L, cf, sv, p, n, c, acc);
    boundary_elem<3>(L, cf, sv, p, n, c, acc);
    boundary_elem<4>(L, cf, sv, p, n, c, acc);
    boundary_elem<5>(L, cf, sv, p, n, c, acc);
    boundary_elem<6>(L, cf, sv, p, n, c, acc);
    boundary_elem<7>(L, cf, sv, p, n, c, acc);
    y0 = acc[0]; y1 = acc[1]; y2 = acc[2];
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
// the fused kernel
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(NT, 2) k_fine(FineLevel L, const __grid_constant__ Coef32 cf, FineArgs a) {
    __shared__ float sv[3 * TILE];
    __shared__ double sh[32];
    const Grid& g = L.g;
    const int64_t S = g.slots;
    const int y0 = blockIdx.x * TY, x0 = blockIdx.y * TX, z0 = blockIdx.z * TZ;
    const int tid = threadIdx.x + threadIdx.y * TY;

    float beta = 0.f;
    if (MODE == FM_CG_DIRECTION && !a.first) beta = (float)(a.scal[a.cur] / a.scal[a.cur ^ 1]);

    // stage the input field v on the tile + halo
    for (int t = tid; t < TILE; t += NT) {
        const int ly = t % HY, lx = (t / HY) % HX, lz = t / (HY * HX);
        const int iy = y0 - 1 + ly, ix = x0 - 1 + lx, iz = z0 - 1 + lz;
        float v0 = 0.f, v1 = 0.f, v2 = 0.f;
        if (in_halo_grid(g, iy, ix, iz)) {
            const int64_t s = g.slot(iy, ix, iz);
            if (MODE == FM_PLAIN) {
                v0 = a.v[s]; v1 = a.v[s + S]; v2 = a.v[s + 2 * S];
            } else if (MODE == FM_VCYCLE_DOWN) {
                v0 = a.r32[s] * a.wdinv[s];
                v1 = a.r32[s + S] * a.wdinv[s + S];
                v2 = a.r32[s + 2 * S] * a.wdinv[s + 2 * S];
            } else if (MODE == FM_CG_JACOBI) {
                v0 = (float)a.r64[s] * a.wdinv[s];
                v1 = (float)a.r64[s + S] * a.wdinv[s + S];
                v2 = (float)a.r64[s + 2 * S] * a.wdinv[s + 2 * S];
            } else {   // FM_CG_DIRECTION
                v0 = a.first ? a.z32[s] : fmaf(beta, a.pold[s], a.z32[s]);
                v1 = a.first ? a.z32[s + S] : fmaf(beta, a.pold[s + S], a.z32[s + S]);
                v2 = a.first ? a.z32[s + 2 * S] : fmaf(beta, a.pold[s + 2 * S], a.z32[s + 2 * S]);
            }
        }
        sv[t] = v0;
        sv[t + TILE] = v1;
        sv[t + 2 * TILE] = v2;
    }
    __syncthreads();

    double dot = 0.0;
    const int iy = y0 + threadIdx.x, ix = x0 + threadIdx.y;
#pragma unroll 1
    for (int kz = 0; kz < TZ; ++kz) {
        const int iz = z0 + kz;
        if (iy > g.ny || ix > g.nx || iz > g.nz) break;
        const int64_t n = g.slot(iy, ix, iz);
        const uint8_t f = L.nflag[n];
        if (!(f & NF_SOLID)) continue;
        const int p = (threadIdx.x + 1) + (threadIdx.y + 1) * SX + (kz + 1) * SZ;
        float y0v, y1v, y2v;
        if (f & NF_INTERIOR) {
            interior(cf, sv, p, y0v, y1v, y2v);
            y0v *= L.kscale; y1v *= L.kscale; y2v *= L.kscale;
        } else {
            boundary(L, cf, sv, p, n, y0v, y1v, y2v);
        }
        if (f & NF_FIX_X) y0v = 0.f;
        if (f & NF_FIX_Y) y1v = 0.f;
        if (f & NF_FIX_Z) y2v = 0.f;
        const float yv[3] = {y0v, y1v, y2v};
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const int64_t i = n + b * S;
            const float v = sv[p + b * TILE];
            if (MODE == FM_PLAIN) {
                a.out32[i] = yv[b];
            } else if (MODE == FM_VCYCLE_DOWN) {
                a.out32[i] = a.r32[i] - yv[b];                       // r' = r - A (omega D^-1 r)
            } else if (MODE == FM_CG_JACOBI) {
                a.x64[i] += (double)v;                               // x += dx
                const double rn = a.r64[i] - (double)yv[b];          // r -= A dx
                a.r64out[i] = rn;
                a.r32out[i] = (float)rn;
            } else {
                a.pout[i] = v;
                a.out32[i] = yv[b];                                  // q = A p
                dot += (double)v * (double)yv[b];
            }
        }
    }
    if (MODE == FM_CG_DIRECTION) grid_dot_finish(dot, a.dot, sh);
}

int fine_grid_blocks(const Grid& g) {
    return ((g.ny + 1 + TY - 1) / TY) * ((g.nx + 1 + TX - 1) / TX) * ((g.nz + 1 + TZ - 1) / TZ);
}

template <int MODE>
void launch_fine(Ctx& c, const FineLevel& L, const Coef32& cf, const FineArgs& a) {
    dim3 grid((L.g.ny + 1 + TY - 1) / TY, (L.g.nx + 1 + TX - 1) / TX, (L.g.nz + 1 + TZ - 1) / TZ);
    k_fine<MODE><<<grid, dim3(TY, TX, 1), 0, c.stream>>>(L, cf, a);
    GMGS_LAUNCHED(c);
}
template void launch_fine<FM_PLAIN>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine<FM_VCYCLE_DOWN>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine<FM_CG_JACOBI>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
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
