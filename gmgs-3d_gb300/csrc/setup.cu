// Solver setup on the GPU: finest discretisation, 2x2x2 hierarchy, Galerkin
// coarse element matrices, Jacobi diagonals, boundary conditions, coarse fixed
// DOFs and the coarsest-level factorisation.
//
// Reference: src/common/DiscretizeDesignDomain.m:29-116,
// src/kernel/BuildingMeshHierarchy.m:8-142, src/kernel/SetupSolver.m:9-259,
// src/kernel/DirectlyAssembleStifnessMatrix.m:24-34,
// src/common/ApplyBoundaryCondition.m:7-23.

#include <algorithm>
#include <cmath>

#include "element_host.h"
#include "setup.cuh"

namespace gmgs {

void stress_coefficients(double E, double nu, const double ele[3], double c[6]) {
    double S[6][6];
    hooke(E, nu, S);
    c[0] = S[0][0];        // isotropic D: d11 on the normal diagonal,
    c[1] = S[0][1];        // d12 off it,
    c[2] = S[3][3];        // d44 on the engineering shear strains
    c[3] = 1.0 / ele[0];
    c[4] = 1.0 / ele[1];
    c[5] = 1.0 / ele[2];
}

// ---------------------------------------------------------------------------
// exclusive scan of int32 counts (in place), deterministic three-phase
// ---------------------------------------------------------------------------
constexpr int SCAN_T = 1024, SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_T * SCAN_ITEMS;

__global__ void k_scan_reduce(const int32_t* __restrict__ d, int64_t n, int64_t* __restrict__ bsum) {
    __shared__ int64_t sh[32];
    const int64_t base = blockIdx.x * (int64_t)SCAN_TILE;
    int64_t s = 0;
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        const int64_t k = base + i * SCAN_T + threadIdx.x;
        if (k < n) s += d[k];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = sh[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) bsum[blockIdx.x] = s;
    }
}

__global__ void k_scan_blocks(int64_t* bsum, int64_t nb, int64_t* total) {
    // single thread block: sequential chunks, exclusive scan of block sums
    __shared__ int64_t carry;
    __shared__ int64_t sh[SCAN_T];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t b0 = 0; b0 < nb; b0 += SCAN_T) {
        const int64_t k = b0 + threadIdx.x;
        const int64_t v = k < nb ? bsum[k] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < SCAN_T; o <<= 1) {
            int64_t t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (k < nb) bsum[k] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == SCAN_T - 1) carry += sh[SCAN_T - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_apply(int32_t* __restrict__ d, int64_t n, const int64_t* __restrict__ bsum) {
    __shared__ int64_t sh[SCAN_T];
    const int64_t base = blockIdx.x * (int64_t)SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int32_t v[SCAN_ITEMS];
    int64_t s = 0;
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        v[i] = base + i < n ? d[base + i] : 0;
        s += v[i];
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < SCAN_T; o <<= 1) {
        int64_t t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    int64_t run = bsum[blockIdx.x] + sh[threadIdx.x] - s;
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        if (base + i < n) d[base + i] = (int32_t)run;
        run += v[i];
    }
}

int64_t exclusive_scan(Ctx& c, int32_t* d, int64_t n) {
    const int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    DevBuf bs = dalloc((nb + 1) * sizeof(int64_t));
    int64_t* bsum = bs.as<int64_t>();
    k_scan_reduce<<<(unsigned)nb, SCAN_T, 0, c.stream>>>(d, n, bsum);
    GMGS_LAUNCHED(c);
    k_scan_blocks<<<1, SCAN_T, 0, c.stream>>>(bsum, nb, bsum + nb);
    GMGS_LAUNCHED(c);
    k_scan_apply<<<(unsigned)nb, SCAN_T, 0, c.stream>>>(d, n, bsum);
    GMGS_LAUNCHED(c);
    int64_t total = 0;
    GMGS_CUDA(cudaMemcpyAsync(&total, bsum + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, c.stream));
    GMGS_CUDA(cudaStreamSynchronize(c.stream));
    if (total > INT32_MAX) throw Error(GMGS_ERR_INVALID_ARGUMENT, "model too large for 32-bit compact ids");
    return total;
}

DevBuf dalloc(size_t bytes) {
    DevBuf b;
    if (bytes == 0) bytes = 16;
    GMGS_CUDA(cudaMalloc(&b.p, bytes));
    b.bytes = bytes;
    count_alloc((int64_t)bytes);
    return b;
}

static int blocks_for(const Ctx& c, int64_t n) {
    int64_t b = (n + 255) / 256;
    const int64_t cap = (int64_t)c.num_sms * 32;
    return (int)std::max<int64_t>(1, std::min(b, cap));
}

#define GRID_STRIDE(i, n) \
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

__device__ __forceinline__ void slot_coords(const Grid& g, int64_t s, int& iy, int& ix, int& iz) {
    g.coords(s, iy, ix, iz);
}

// ---------------------------------------------------------------------------
// masks
// ---------------------------------------------------------------------------
// finest element mask from the (unpadded) occupancy; only 1 is solid (DiscretizeDesignDomain.m:68)
__global__ void k_emask_l1(Grid g, const int32_t* __restrict__ occ, int nely, int nelx, int nelz,
                           uint8_t* __restrict__ emask) {
    GRID_STRIDE(s, g.slots) {
        int iy, ix, iz;
        slot_coords(g, s, iy, ix, iz);
        uint8_t v = 0;
        if (iy >= 0 && ix >= 0 && iz >= 0 && iy < nely && ix < nelx && iz < nelz)
            v = occ[iy + (int64_t)nely * (ix + (int64_t)nelx * iz)] == 1;
        emask[s] = v;
    }
}

// coarse element = non-empty if any child is solid (BuildingMeshHierarchy.m:70).
// kmode: 0 none, 1 "unique if a child is void" (SetupSolver.m:43-44),
// 2 "unique if a non-void child is unique on the finer level" (SetupSolver.m:96-101),
// 3 every non-empty element gets its own matrix (state 1).
__global__ void k_coarsen(Grid gc, Grid gf, const uint8_t* __restrict__ emf, const int32_t* __restrict__ etf,
                          int kmode, uint8_t* __restrict__ emc, int32_t* __restrict__ needK) {
    GRID_STRIDE(s, gc.slots) {
        int iy, ix, iz;
        slot_coords(gc, s, iy, ix, iz);
        uint8_t any = 0, allsolid = 1, kid_unique = 0;
        if (iy >= 0 && ix >= 0 && iz >= 0 && iy < gc.ny && ix < gc.nx && iz < gc.nz) {
            for (int j = 0; j < 8; ++j) {
                const int64_t fs = gf.slot(2 * iy + (j & 1), 2 * ix + ((j >> 1) & 1), 2 * iz + (j >> 2));
                const uint8_t m = emf[fs];
                any |= m;
                allsolid &= m;
                if (m && etf && etf[fs] > 0) kid_unique = 1;
            }
        } else {
            allsolid = 0;
        }
        emc[s] = any;
        int32_t nk = 0;
        if (any) {
            if (kmode == 1) nk = !allsolid;
            else if (kmode == 2) nk = kid_unique;
            else if (kmode == 3) nk = 1;
        }
        if (needK) needK[s] = nk;
    }
}

__global__ void k_node_flags(Grid g, const uint8_t* __restrict__ emask, uint8_t* __restrict__ nflag,
                             int32_t* __restrict__ cnt) {
    GRID_STRIDE(s, g.slots) {
        int iy, ix, iz;
        slot_coords(g, s, iy, ix, iz);
        int n = 0;
        if (iy >= 0 && ix >= 0 && iz >= 0 && iy <= g.ny && ix <= g.nx && iz <= g.nz) {
            for (int e = 0; e < 8; ++e)
                n += emask[s - (e & 1) - ((e >> 1) & 1) * g.sx() - (e >> 2) * g.sz()];
        }
        nflag[s] = n ? NF_SOLID : 0;
        if (cnt) cnt[s] = n;
    }
}

// NF_INTERIOR: the node's 8 elements all carry the level's uniform matrix
// kscale * Ke0; NF_PEREL: one of them has its own stored matrix
__global__ void k_interior_flags(Grid g, const uint8_t* __restrict__ emask, const int32_t* __restrict__ etype,
                                 uint8_t* __restrict__ nflag, int32_t* __restrict__ perel) {
    GRID_STRIDE(s, g.slots) {
        uint8_t f = nflag[s] & (uint8_t) ~(NF_INTERIOR | NF_PEREL);
        if (f & NF_SOLID) {
            bool all = true, pe = false;
            for (int e = 0; e < 8; ++e) {
                const int64_t es = s - (e & 1) - ((e >> 1) & 1) * g.sx() - (e >> 2) * g.sz();
                all = all && emask[es] && (!etype || etype[es] == 0);
                pe = pe || (etype && emask[es] && etype[es] > 0);
            }
            if (all) f |= NF_INTERIOR;
            if (pe) f |= NF_PEREL;
        }
        nflag[s] = f;
        if (perel) perel[s] = (f & NF_PEREL) ? 1 : 0;
    }
}

__global__ void k_flag_to_count(int64_t n, const uint8_t* __restrict__ f, uint8_t bit, int32_t* __restrict__ out) {
    GRID_STRIDE(i, n) out[i] = (f[i] & bit) ? 1 : 0;
}

// slots with count 1 before the scan -> compact list (scan holds the exclusive prefix)
__global__ void k_compact(int64_t n, const uint8_t* __restrict__ f, uint8_t bit, const int32_t* __restrict__ scan,
                          int32_t* __restrict__ list) {
    GRID_STRIDE(i, n) if (f[i] & bit) list[scan[i]] = (int32_t)i;
}

__global__ void k_etype(int64_t n, const uint8_t* __restrict__ emask, const int32_t* __restrict__ needK_scan,
                        const int32_t* __restrict__ needK_flag, int32_t* __restrict__ etype,
                        int32_t* __restrict__ kslot) {
    GRID_STRIDE(i, n) {
        int32_t t = -1;
        if (emask[i]) {
            const bool nk = needK_flag[i] != 0;
            t = nk ? needK_scan[i] + 1 : 0;
            if (nk) kslot[needK_scan[i]] = (int32_t)i;
        }
        etype[i] = t;
    }
}

// Level 2 with a uniform finest material (SetupSolver.m:39-68): a "unique"
// element's Galerkin matrix is the sum of P_j^T Ke0 P_j over its solid
// children, so it is fixed by the 8-bit child-occupancy pattern.  One matrix
// per pattern present replaces one per element: pat[s] = pattern (0 for
// void and all-solid elements), rep[p] = the lowest slot with pattern p.
__global__ void k_child_pattern(Grid gc, Grid gf, const uint8_t* __restrict__ emf, const int32_t* __restrict__ needK,
                                int32_t* __restrict__ pat, int32_t* __restrict__ rep) {
    GRID_STRIDE(s, gc.slots) {
        int32_t p = 0;
        if (needK[s]) {
            int iy, ix, iz;
            slot_coords(gc, s, iy, ix, iz);
            for (int j = 0; j < 8; ++j)
                if (emf[gf.slot(2 * iy + (j & 1), 2 * ix + ((j >> 1) & 1), 2 * iz + (j >> 2))]) p |= 1 << j;
            atomicMin(rep + p, (int32_t)s);
        }
        pat[s] = p;
    }
}
// etype = 1 + the rank of the element's pattern among the patterns present
__global__ void k_etype_pattern(int64_t n, const uint8_t* __restrict__ emask, const int32_t* __restrict__ pat,
                                const int32_t* __restrict__ rank, int32_t* __restrict__ etype) {
    GRID_STRIDE(i, n) etype[i] = emask[i] ? (pat[i] ? rank[pat[i]] + 1 : 0) : -1;
}

// ---------------------------------------------------------------------------
// Galerkin coarse element matrices: Ks_c = sum_j P_j^T K_j P_j over solid
// children j (SetupSolver.m:36-196 with the 81x24 trilinear table).
// One block per coarse element, FP64.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double tri_w(int pos, int corner2) {
    const int d = pos > corner2 ? pos - corner2 : corner2 - pos;
    return d == 0 ? 1.0 : (d == 1 ? 0.5 : 0.0);
}

__global__ void __launch_bounds__(192) k_galerkin(Grid gc, Grid gf, const int32_t* __restrict__ kslot,
                                                  const uint8_t* __restrict__ emf, const int32_t* __restrict__ etf,
                                                  const double* __restrict__ Ksf, const double* __restrict__ G,
                                                  double kscale_f, const double* __restrict__ escale_f,
                                                  double* __restrict__ Ks_out, float* __restrict__ Ks32_out) {
    __shared__ double K[KE], T[KE], W[64];
    const int64_t s = kslot[blockIdx.x];
    int Ey, Ex, Ez;
    slot_coords(gc, s, Ey, Ex, Ez);
    double acc[3] = {0, 0, 0};    // 576 / 192 entries per thread
    for (int j = 0; j < 8; ++j) {
        const int dy = j & 1, dx = (j >> 1) & 1, dz = j >> 2;
        const int64_t fs = gf.slot(2 * Ey + dy, 2 * Ex + dx, 2 * Ez + dz);
        if (!emf[fs]) continue;       // uniform branch across the block
        const int t = etf ? etf[fs] : 0;
        if (t == 0) {                 // a scaled Ke0 child: sc * (P_j^T Ke0 P_j), precomputed
            const double sc = kscale_f * (escale_f ? escale_f[fs] : 1.0);
            for (int k = 0; k < 3; ++k) acc[k] += sc * G[j * KE + threadIdx.x + k * blockDim.x];
            continue;
        }
        for (int i = threadIdx.x; i < KE; i += blockDim.x) K[i] = Ksf[(int64_t)(t - 1) * KE + i];
        if (threadIdx.x < 64) {
            const int q = threadIdx.x >> 3, b = threadIdx.x & 7;   // W[q][b]: corner b at child-local node q
            W[threadIdx.x] = tri_w(dy + corner_y(q), 2 * corner_y(b)) * tri_w(dx + corner_x(q), 2 * corner_x(b)) *
                             tri_w(dz + corner_z(q), 2 * corner_z(b));
        }
        __syncthreads();
        // T = K P : T[r][3b+be] = sum_q K[r][3q+be] W[q][b]
        for (int i = threadIdx.x; i < KE; i += blockDim.x) {
            const int r = i / 24, col = i % 24, b = col / 3, be = col % 3;
            double v = 0;
            for (int q = 0; q < 8; ++q) v += K[r * 24 + 3 * q + be] * W[q * 8 + b];
            T[i] = v;
        }
        __syncthreads();
        // out += P^T T : out[3a+al][col] += sum_p W[p][a] T[3p+al][col]
        for (int k = 0; k < 3; ++k) {
            const int i = threadIdx.x + k * blockDim.x;
            const int row = i / 24, col = i % 24, a = row / 3, al = row % 3;
            double v = 0;
            for (int p = 0; p < 8; ++p) v += W[p * 8 + a] * T[(3 * p + al) * 24 + col];
            acc[k] += v;
        }
        __syncthreads();
    }
    for (int k = 0; k < 3; ++k) {
        const int64_t o = (int64_t)blockIdx.x * KE + threadIdx.x + k * blockDim.x;
        if (Ks_out) Ks_out[o] = acc[k];
        if (Ks32_out) Ks32_out[o] = (float)acc[k];
    }
}

// Level 3 straight from the finest level when every level-2 element is the
// scaled-children sum sum_j s_j G_j (a density field): K = sum over the 64
// finest descendants of s * G2[c][j], G2[c][j] = P_c^T G_j P_c, so the
// level-2 matrices are never needed in FP64.  One block per coarse element.
__global__ void __launch_bounds__(192) k_galerkin_grand(Grid g2, Grid g1, Grid g0, const int32_t* __restrict__ kslot,
                                                        const uint8_t* __restrict__ em1, const uint8_t* __restrict__ em0,
                                                        const double* __restrict__ esc0, double kscale0,
                                                        const double* __restrict__ G2, double* __restrict__ Ks_out) {
    const int64_t s = kslot[blockIdx.x];
    int Ey, Ex, Ez;
    slot_coords(g2, s, Ey, Ex, Ez);
    double acc[3] = {0, 0, 0};
    for (int c = 0; c < 8; ++c) {
        const int cy = 2 * Ey + (c & 1), cx = 2 * Ex + ((c >> 1) & 1), cz = 2 * Ez + (c >> 2);
        if (!em1[g1.slot(cy, cx, cz)]) continue;          // uniform branch across the block
        for (int j = 0; j < 8; ++j) {
            const int64_t fs = g0.slot(2 * cy + (j & 1), 2 * cx + ((j >> 1) & 1), 2 * cz + (j >> 2));
            if (!em0[fs]) continue;
            const double sc = kscale0 * esc0[fs];
            const double* Gc = G2 + (int64_t)(c * 8 + j) * KE;
            for (int k = 0; k < 3; ++k) acc[k] += sc * Gc[threadIdx.x + k * blockDim.x];
        }
    }
    for (int k = 0; k < 3; ++k) Ks_out[(int64_t)blockIdx.x * KE + threadIdx.x + k * blockDim.x] = acc[k];
}

// ---------------------------------------------------------------------------
// Jacobi diagonal: sum of the element diagonals at each node (SetupSolver.m:204-244)
// ---------------------------------------------------------------------------
__global__ void k_diag(Grid g, const uint8_t* __restrict__ emask, const uint8_t* __restrict__ nflag,
                       const int32_t* __restrict__ etype, const double* __restrict__ Ks, const double* __restrict__ ke0,
                       double kscale, const double* __restrict__ escale, double* __restrict__ d) {
    GRID_STRIDE(s, g.slots) {
        double a[3] = {0, 0, 0};
        if (nflag[s] & NF_SOLID) {
            for (int e = 0; e < 8; ++e) {
                const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;
                const int64_t es = s - A - B * g.sx() - C * g.sz();
                if (!emask[es]) continue;
                const int c = corner_of(A, B, C);
                const int t = etype ? etype[es] : 0;
                for (int al = 0; al < 3; ++al) {
                    const int ii = (3 * c + al) * 24 + 3 * c + al;
                    a[al] += t > 0 ? Ks[(int64_t)(t - 1) * KE + ii] : kscale * (escale ? escale[es] : 1.0) * ke0[ii];
                }
            }
        }
        d[s] = a[0];
        d[s + g.slots] = a[1];
        d[s + 2 * g.slots] = a[2];
    }
}

// On a level whose solid elements all carry kscale * Ke0 (no per-element
// matrices, no element scales) a node's diagonal depends only on which of its
// 8 elements are solid: the 256 masks' sums (in k_diag's element order, each
// product and sum rounded separately), then one table lookup per node.
__device__ __forceinline__ void diag_of_mask(uint32_t mask, const double* __restrict__ ke0, double kscale,
                                             const double* __restrict__ escale, double a[3]) {
    a[0] = a[1] = a[2] = 0.0;
    for (int e = 0; e < 8; ++e) {
        if (!((mask >> e) & 1u)) continue;
        const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;
        const int c = corner_of(A, B, C);
        for (int al = 0; al < 3; ++al) {
            const int ii = (3 * c + al) * 24 + 3 * c + al;
            a[al] = __dadd_rn(a[al], __dmul_rn(__dmul_rn(kscale, escale ? escale[0] : 1.0), ke0[ii]));
        }
    }
}
__global__ void k_diag_table(const double* __restrict__ ke0, double kscale, const double* __restrict__ escale,
                             double* __restrict__ table) {
    const uint32_t m = threadIdx.x;   // one thread per mask, 256 threads
    double a[3];
    diag_of_mask(m, ke0, kscale, escale, a);
    for (int al = 0; al < 3; ++al) table[3 * m + al] = a[al];
}
__global__ void k_diag_uniform(Grid g, const uint8_t* __restrict__ emask, const uint8_t* __restrict__ nflag,
                               const double* __restrict__ table, double* __restrict__ d) {
    __shared__ double t[3 * 256];
    for (int i = threadIdx.x; i < 3 * 256; i += blockDim.x) t[i] = table[i];
    __syncthreads();
    GRID_STRIDE(s, g.slots) {
        uint32_t mask = 0;
        if (nflag[s] & NF_SOLID)
            for (int e = 0; e < 8; ++e) {
                const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;
                if (emask[s - A - B * g.sx() - C * g.sz()]) mask |= 1u << e;
            }
        d[s] = t[3 * mask];
        d[s + g.slots] = t[3 * mask + 1];
        d[s + 2 * g.slots] = t[3 * mask + 2];
    }
}

// Level-2 diagonal when its element matrices are the scaled-children sums
// sum_j s_j G_j and only their FP32 copies are kept: each element's diagonal
// entry is summed exactly as k_galerkin sums it, so the result equals k_diag
// on the FP64 matrices.
__global__ void k_diag_children(Grid g1, Grid g0, const uint8_t* __restrict__ em1, const uint8_t* __restrict__ nflag1,
                                const uint8_t* __restrict__ em0, const double* __restrict__ esc0, double kscale0,
                                const double* __restrict__ G, double* __restrict__ d) {
    GRID_STRIDE(s, g1.slots) {
        double a[3] = {0, 0, 0};
        if (nflag1[s] & NF_SOLID) {
            for (int e = 0; e < 8; ++e) {
                const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;
                const int64_t es = s - A - B * g1.sx() - C * g1.sz();
                if (!em1[es]) continue;
                int Ey, Ex, Ez;
                slot_coords(g1, es, Ey, Ex, Ez);
                const int cn = corner_of(A, B, C);
                for (int al = 0; al < 3; ++al) {
                    const int ii = (3 * cn + al) * 24 + 3 * cn + al;
                    double v = 0;
                    for (int j = 0; j < 8; ++j) {
                        const int64_t fs = g0.slot(2 * Ey + (j & 1), 2 * Ex + ((j >> 1) & 1), 2 * Ez + (j >> 2));
                        if (!em0[fs]) continue;
                        const double sc = kscale0 * esc0[fs];
                        v += sc * G[j * KE + ii];
                    }
                    a[al] += v;
                }
            }
        }
        d[s] = a[0];
        d[s + g1.slots] = a[1];
        d[s + 2 * g1.slots] = a[2];
    }
}

// ---------------------------------------------------------------------------
// boundary conditions
// ---------------------------------------------------------------------------
constexpr uint8_t NF_KEEP = NF_SOLID | NF_INTERIOR | NF_PEREL;   // flags that do not depend on the BCs

__global__ void k_clear_fixed(int64_t n, uint8_t* f) {
    GRID_STRIDE(i, n) f[i] &= NF_KEEP;
}
__global__ void k_set_fixed(int64_t n, const int32_t* __restrict__ ids, const int32_t* __restrict__ node_slot,
                            uint8_t* __restrict__ f) {
    GRID_STRIDE(i, n) f[node_slot[ids[i] - 1]] |= (NF_FIX_X | NF_FIX_Y | NF_FIX_Z);
}
// loads rows (id, fx, fy, fz), 1-based compact node ids validated on the host;
// the last row of each node wins (ApplyBoundaryCondition.m:9): its index is
// the maximum over the node's rows
__global__ void k_load_last(int64_t n, const double* __restrict__ loads, int32_t* __restrict__ last) {
    GRID_STRIDE(i, n) atomicMax(last + ((int64_t)loads[4 * i] - 1), (int32_t)i);
}
__global__ void k_set_loads(int64_t n, const double* __restrict__ loads, const int32_t* __restrict__ last,
                            const int32_t* __restrict__ node_slot, int64_t S, double* __restrict__ F) {
    GRID_STRIDE(i, n) {
        const int64_t id = (int64_t)loads[4 * i] - 1;
        if (last[id] != (int32_t)i) continue;
        const int64_t s = node_slot[id];
        F[s] = loads[4 * i + 1];
        F[s + S] = loads[4 * i + 2];
        F[s + 2 * S] = loads[4 * i + 3];
    }
}
// coarse fixed DOFs: restricted indicator != 0 (SetupSolver.m:247-254)
__global__ void k_fixed_from_indicator(int64_t S, const float* __restrict__ ind, uint8_t* __restrict__ f) {
    GRID_STRIDE(s, S) {
        uint8_t v = f[s] & NF_KEEP;
        if (v & NF_SOLID) {
            if (ind[s] != 0.f) v |= NF_FIX_X;
            if (ind[s + S] != 0.f) v |= NF_FIX_Y;
            if (ind[s + 2 * S] != 0.f) v |= NF_FIX_Z;
        }
        f[s] = v;
    }
}
__global__ void k_indicator(int64_t S, const uint8_t* __restrict__ f, float* __restrict__ ind) {
    GRID_STRIDE(s, S) {
        ind[s] = (f[s] & NF_FIX_X) ? 1.f : 0.f;
        ind[s + S] = (f[s] & NF_FIX_Y) ? 1.f : 0.f;
        ind[s + 2 * S] = (f[s] & NF_FIX_Z) ? 1.f : 0.f;
    }
}

// free DOFs of the coarsest level, node-major then component (reference freeDOFs order)
__global__ void k_free_count(int64_t S, const uint8_t* __restrict__ f, int32_t* __restrict__ cnt) {
    GRID_STRIDE(i, 3 * S) {
        const int64_t s = i / 3;
        const int comp = (int)(i % 3);
        cnt[i] = (f[s] & NF_SOLID) && !(f[s] & (NF_FIX_X << comp));
    }
}
__global__ void k_free_list(int64_t S, const uint8_t* __restrict__ f, const int32_t* __restrict__ scan,
                            int32_t* __restrict__ idx) {
    GRID_STRIDE(i, 3 * S) {
        const int64_t s = i / 3;
        const int comp = (int)(i % 3);
        if ((f[s] & NF_SOLID) && !(f[s] & (NF_FIX_X << comp))) idx[scan[i]] = (int32_t)(s + comp * S);
    }
}

// dense coarsest matrix on the free DOFs, K[row][col] = sum_e Ks_e(i, j) with
// row = dof of local i, col = dof of local j (DirectlyAssembleStifnessMatrix.m:25-32).
// Stored matrices have row = output DOF, so Ks_e(i, j) = M_e[j][i].
// One thread per (free row, neighbour dof); deterministic element order.
// Entry t = (row, k) of the coarsest free-DOF matrix: row = free DOF, k =
// (neighbour offset, component) of the column; the value sums the
// contributions of the solid elements shared by the two nodes
// (DirectlyAssembleStifnessMatrix.m:24-34 restricted to the free DOFs).
// Returns false when the column DOF is fixed or outside the level.
__device__ __forceinline__ bool coarse_entry(const Grid& g, int64_t t, const int32_t* __restrict__ freeidx,
                                             const int32_t* __restrict__ rank, const uint8_t* __restrict__ emask,
                                             const int32_t* __restrict__ etype, const double* __restrict__ Ks,
                                             const double* __restrict__ ke0, double kscale, int& row, int& col,
                                             double& v) {
    row = (int)(t / 81);
    const int k = (int)(t % 81);
    const int off = k / 3, be = k % 3;
    const int oa = off % 3 - 1, ob = (off / 3) % 3 - 1, oc = off / 9 - 1;
    const int64_t ri = freeidx[row];
    const int64_t S = g.slots;
    const int al = (int)(ri / S);
    const int64_t n = ri % S;
    const int64_t m = n + oa + ob * g.sx() + oc * g.sz();
    col = rank[m + be * S];
    if (col < 0) return false;
    v = 0;
    for (int e = 0; e < 8; ++e) {
        const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;
        const int64_t es = n - A - B * g.sx() - C * g.sz();
        // element must also contain m: m - es in {0,1}^3
        const int my = A + oa, mx = B + ob, mz = C + oc;
        if (my < 0 || my > 1 || mx < 0 || mx > 1 || mz < 0 || mz > 1) continue;
        if (!emask[es]) continue;
        const int cn = corner_of(A, B, C), cm = corner_of(my, mx, mz);
        const int t2 = etype ? etype[es] : 0;
        const int ii = (3 * cm + be) * 24 + 3 * cn + al;
        v += t2 > 0 ? Ks[(int64_t)(t2 - 1) * KE + ii] : kscale * ke0[ii];
    }
    return true;
}

// half bandwidth: max |col - row| over non-zero entries
__global__ void k_coarse_bandwidth(Grid g, int nf, const int32_t* __restrict__ freeidx,
                                   const int32_t* __restrict__ rank, const uint8_t* __restrict__ emask,
                                   const int32_t* __restrict__ etype, const double* __restrict__ Ks,
                                   const double* __restrict__ ke0, double kscale, int* __restrict__ bw) {
    int best = 0;
    GRID_STRIDE(t, (int64_t)nf * 81) {
        int row, col;
        double v;
        if (coarse_entry(g, t, freeidx, rank, emask, etype, Ks, ke0, kscale, row, col, v) && v != 0.0)
            best = max(best, col > row ? col - row : row - col);
    }
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) atomicMax(bw, best);
}

// the diagonal blocks A_ii (both triangles) and sub-diagonal blocks
// A_(i,i-1) of the block-tridiagonal form, column-major B x B
__global__ void k_assemble_blocks(Grid g, int nf, const int32_t* __restrict__ freeidx,
                                  const int32_t* __restrict__ rank, const uint8_t* __restrict__ emask,
                                  const int32_t* __restrict__ etype, const double* __restrict__ Ks,
                                  const double* __restrict__ ke0, double kscale, int B, double* __restrict__ diag,
                                  double* __restrict__ sub) {
    const int64_t B2 = (int64_t)B * B;
    GRID_STRIDE(t, (int64_t)nf * 81) {
        int row, col;
        double v;
        if (!coarse_entry(g, t, freeidx, rank, emask, etype, Ks, ke0, kscale, row, col, v)) continue;
        const int bi = row / B, bj = col / B;
        const int64_t at = (int64_t)(row % B) + (int64_t)(col % B) * B;
        if (bi == bj) diag[bi * B2 + at] = v;
        else if (bi == bj + 1) sub[bi * B2 + at] = v;
    }
}

// identity on the padding rows of the last diagonal block
__global__ void k_pad_identity(int n, int npad, int B, double* __restrict__ diag) {
    const int i = n + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    const int64_t B2 = (int64_t)B * B;
    diag[(int64_t)(i / B) * B2 + (int64_t)(i % B) * (B + 1)] = 1.0;
}
__global__ void k_rank_fill(int64_t n, int32_t* r) { GRID_STRIDE(i, n) r[i] = -1; }
__global__ void k_rank_set(int64_t nf, const int32_t* __restrict__ idx, int32_t* __restrict__ r) {
    GRID_STRIDE(i, nf) r[idx[i]] = (int32_t)i;
}
__global__ void k_to_float(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    GRID_STRIDE(i, n) b[i] = (float)a[i];
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
void build_levels(Model& M, const int32_t* occ_dev) {
    Ctx& c = M.ctx;
    const int L = M.num_levels;
    if (occ_dev) {
        M.levels.clear();
        M.levels.resize(L);
    } else {
        // rebuild the coarse levels, keep the finest masks and element scale
        for (int l = 1; l < L; ++l) M.levels[l] = Level();
    }
    for (int l = 0; l < L; ++l) {
        Level& lv = M.levels[l];
        lv.g = Grid::make(M.ny >> l, M.nx >> l, M.nz >> l);
        lv.kscale = std::ldexp(1.0, l);   // Ke0 * eleSize_l / eleSize_1 (SetupSolver.m:37)
        if (!lv.emask.p) lv.emask = dalloc(lv.g.slots);
        if (!lv.nflag.p) lv.nflag = dalloc(lv.g.slots);
    }
    // finest masks
    if (occ_dev) {
        Level& lv = M.levels[0];
        k_emask_l1<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g, occ_dev, M.nely, M.nelx, M.nelz,
                                                                     lv.emask.as<uint8_t>());
        GMGS_LAUNCHED(c);
    }
    c.trace_point("create: level buffers + finest mask");
    // coarse masks + per-element matrix selection
    for (int l = 1; l < L; ++l) {
        Level& lv = M.levels[l];
        Level& fv = M.levels[l - 1];
        int kmode;
        if (M.has_density) kmode = 3;
        else if (l == 1 && L > 2) kmode = 1;        // SetupSolver.m:39-68
        else if (l == 2 && L > 3) kmode = 2;        // SetupSolver.m:90-131
        else kmode = 3;                              // state 1
        lv.state = kmode == 3 ? 1 : 2;
        DevBuf need = dalloc(lv.g.slots * sizeof(int32_t));
        DevBuf need0 = dalloc(lv.g.slots * sizeof(int32_t));
        k_coarsen<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g, fv.g, fv.emask.as<uint8_t>(),
                                                                    fv.etype.as<int32_t>(), kmode,
                                                                    lv.emask.as<uint8_t>(), need.as<int32_t>());
        GMGS_LAUNCHED(c);
        if (kmode == 1) {
            // one Galerkin matrix per child-occupancy pattern present (at most 254)
            DevBuf rep = dalloc(256 * sizeof(int32_t));
            GMGS_CUDA(cudaMemsetAsync(rep.p, 0x7f, 256 * sizeof(int32_t), c.stream));   // > any slot
            k_child_pattern<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(
                lv.g, fv.g, fv.emask.as<uint8_t>(), need.as<int32_t>(), need0.as<int32_t>(), rep.as<int32_t>());
            GMGS_LAUNCHED(c);
            int32_t hrep[256];
            GMGS_CUDA(cudaMemcpyAsync(hrep, rep.p, sizeof(hrep), cudaMemcpyDeviceToHost, c.stream));
            GMGS_CUDA(cudaStreamSynchronize(c.stream));
            int32_t hrank[256], hslot[256];
            int nk = 0;
            for (int p = 0; p < 256; ++p) {
                hrank[p] = -1;
                if (p > 0 && hrep[p] != 0x7f7f7f7f) {
                    hrank[p] = nk;
                    hslot[nk++] = hrep[p];
                }
            }
            lv.nK = nk;
            lv.etype = dalloc(lv.g.slots * sizeof(int32_t));
            lv.kslot = dalloc(std::max(1, nk) * sizeof(int32_t));
            DevBuf drank = dalloc(256 * sizeof(int32_t));
            GMGS_CUDA(cudaMemcpyAsync(drank.p, hrank, sizeof(hrank), cudaMemcpyHostToDevice, c.stream));
            if (nk > 0)
                GMGS_CUDA(cudaMemcpyAsync(lv.kslot.p, hslot, nk * sizeof(int32_t), cudaMemcpyHostToDevice, c.stream));
            k_etype_pattern<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(
                lv.g.slots, lv.emask.as<uint8_t>(), need0.as<int32_t>(), drank.as<int32_t>(), lv.etype.as<int32_t>());
            GMGS_LAUNCHED(c);
            GMGS_CUDA(cudaStreamSynchronize(c.stream));
            continue;
        }
        GMGS_CUDA(cudaMemcpyAsync(need0.p, need.p, lv.g.slots * sizeof(int32_t), cudaMemcpyDeviceToDevice, c.stream));
        lv.nK = exclusive_scan(c, need.as<int32_t>(), lv.g.slots);
        lv.etype = dalloc(lv.g.slots * sizeof(int32_t));
        lv.kslot = dalloc(std::max<int64_t>(1, lv.nK) * sizeof(int32_t));
        // etype: need0 holds the 0/1 flags, need the exclusive prefix
        k_etype<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(
            lv.g.slots, lv.emask.as<uint8_t>(), need.as<int32_t>(), need0.as<int32_t>(), lv.etype.as<int32_t>(),
            lv.kslot.as<int32_t>());
        GMGS_LAUNCHED(c);
        GMGS_CUDA(cudaStreamSynchronize(c.stream));   // temporaries are freed at scope exit
    }
    c.trace_point("create: coarse masks + matrix selection");
    // node flags, compact node maps, element counts
    for (int l = 0; l < L; ++l) {
        Level& lv = M.levels[l];
        k_node_flags<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g, lv.emask.as<uint8_t>(),
                                                                       lv.nflag.as<uint8_t>(), nullptr);
        GMGS_LAUNCHED(c);
        DevBuf sc = dalloc(lv.g.slots * sizeof(int32_t));
        k_flag_to_count<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g.slots, lv.nflag.as<uint8_t>(), NF_SOLID,
                                                                          sc.as<int32_t>());
        GMGS_LAUNCHED(c);
        lv.n_node = exclusive_scan(c, sc.as<int32_t>(), lv.g.slots);
        lv.node_slot = dalloc(std::max<int64_t>(1, lv.n_node) * sizeof(int32_t));
        k_compact<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g.slots, lv.nflag.as<uint8_t>(), NF_SOLID,
                                                                    sc.as<int32_t>(), lv.node_slot.as<int32_t>());
        GMGS_LAUNCHED(c);
        // elements
        k_flag_to_count<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g.slots, lv.emask.as<uint8_t>(), 1,
                                                                          sc.as<int32_t>());
        GMGS_LAUNCHED(c);
        lv.n_elem = exclusive_scan(c, sc.as<int32_t>(), lv.g.slots);
        lv.elem_slot = dalloc(std::max<int64_t>(1, lv.n_elem) * sizeof(int32_t));
        k_compact<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g.slots, lv.emask.as<uint8_t>(), 1,
                                                                    sc.as<int32_t>(), lv.elem_slot.as<int32_t>());
        GMGS_LAUNCHED(c);
        GMGS_CUDA(cudaStreamSynchronize(c.stream));
    }
    if (M.levels[0].n_elem == 0) throw Error(GMGS_ERR_NO_SOLID, "the occupancy has no solid voxel");
    GMGS_CUDA(cudaStreamSynchronize(c.stream));
    c.trace_point("create: node/element lists");
}

__global__ void k_escale(int64_t ne, const int32_t* __restrict__ elem_slot, const double* __restrict__ rho,
                         double penal, double* __restrict__ esc) {
    GRID_STRIDE(e, ne) esc[elem_slot[e]] = pow(rho[e], penal);
}

// Extension: finest element scale rho^penal; every coarse level then stores
// one Galerkin matrix per element.
void set_density_dev(Model& M, const double* rho_dev) {
    Ctx& c = M.ctx;
    Level& l0 = M.levels[0];
    M.rho = dalloc(l0.n_elem * sizeof(double));
    GMGS_CUDA(cudaMemcpyAsync(M.rho.p, rho_dev, l0.n_elem * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    l0.escale64 = dalloc(l0.g.slots * sizeof(double));
    GMGS_CUDA(cudaMemsetAsync(l0.escale64.p, 0, l0.g.slots * sizeof(double), c.stream));
    k_escale<<<blocks_for(c, l0.n_elem), 256, 0, c.stream>>>(l0.n_elem, l0.elem_slot.as<int32_t>(), M.rho.as<double>(),
                                                             M.penal, l0.escale64.as<double>());
    GMGS_LAUNCHED(c);
    l0.escale32.release();
    M.has_density = true;
    build_levels(M, nullptr);
    build_operators(M);
}

void build_operators(Model& M) {
    Ctx& c = M.ctx;
    const int L = M.num_levels;
    double Ke[KE], KeT[KE];
    element_stiffness(M.prm.youngs_modulus, M.prm.poisson_ratio, M.ele, Ke);
    for (int i = 0; i < 24; ++i)
        for (int j = 0; j < 24; ++j) KeT[i * 24 + j] = Ke[j * 24 + i];   // row = output DOF
    std::copy(KeT, KeT + KE, M.ke0_rows);
    make_mat_coef(KeT, M.mc64, M.mc32);
    make_stencil(KeT, M.coef);
    make_tc_coef(KeT, M.tcoef);
    for (int l = 0; l < L; ++l) {
        Level& lv = M.levels[l];
        const bool uniform_ok = !(l == 0 && lv.escale64.p);
        lv.n_perel = 0;
        if (uniform_ok) {
            DevBuf cnt = dalloc(lv.g.slots * sizeof(int32_t));
            k_interior_flags<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g, lv.emask.as<uint8_t>(),
                                                                               lv.etype.as<int32_t>(),
                                                                               lv.nflag.as<uint8_t>(),
                                                                               cnt.as<int32_t>());
            GMGS_LAUNCHED(c);
            if (lv.etype.p) {
                lv.n_perel = exclusive_scan(c, cnt.as<int32_t>(), lv.g.slots);
                lv.perel_nodes = dalloc(std::max<int64_t>(1, lv.n_perel) * sizeof(int32_t));
                k_compact<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g.slots, lv.nflag.as<uint8_t>(),
                                                                            NF_PEREL, cnt.as<int32_t>(),
                                                                            lv.perel_nodes.as<int32_t>());
                GMGS_LAUNCHED(c);
            }
            GMGS_CUDA(cudaStreamSynchronize(c.stream));
        }
    }
    c.trace_point("create: interior flags");
    if (c.trace)
        for (int l = 0; l < L; ++l)
            std::fprintf(stderr, "[gmgs] level %d: %lld nodes, %lld elements, %lld own matrices, %lld nodes on them\n",
                         l + 1, (long long)M.levels[l].n_node, (long long)M.levels[l].n_elem,
                         (long long)M.levels[l].nK, (long long)M.levels[l].n_perel);
    M.ke0_dev = dalloc(KE * sizeof(double));
    GMGS_CUDA(cudaMemcpyAsync(M.ke0_dev.p, KeT, KE * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    const double* ke0 = M.ke0_dev.as<double>();
    // G_j = P_j^T Ke0 P_j for the 8 child positions j (SetupSolver.m:53-66 applied to one solid child)
    static_assert(KE == 576, "24x24 element matrices");
    auto child_product = [](const double* K, int j, double* out) {     // out = P_j^T K P_j
        const int dy = j & 1, dx = (j >> 1) & 1, dz = j >> 2;
        double W[8][8];
        for (int q = 0; q < 8; ++q)
            for (int b = 0; b < 8; ++b) {
                auto w1 = [](int pos, int c2) { const int d = pos > c2 ? pos - c2 : c2 - pos; return d == 0 ? 1.0 : (d == 1 ? 0.5 : 0.0); };
                W[q][b] = w1(dy + corner_y(q), 2 * corner_y(b)) * w1(dx + corner_x(q), 2 * corner_x(b)) *
                          w1(dz + corner_z(q), 2 * corner_z(b));
            }
        double T[KE];
        for (int r = 0; r < 24; ++r)
            for (int col = 0; col < 24; ++col) {
                double v = 0;
                for (int q = 0; q < 8; ++q) v += K[r * 24 + 3 * q + col % 3] * W[q][col / 3];
                T[r * 24 + col] = v;
            }
        for (int row = 0; row < 24; ++row)
            for (int col = 0; col < 24; ++col) {
                double v = 0;
                for (int p = 0; p < 8; ++p) v += W[p][row / 3] * T[(3 * p + row % 3) * 24 + col];
                out[row * 24 + col] = v;
            }
    };
    std::vector<double> Gh(8 * KE, 0.0);
    for (int j = 0; j < 8; ++j) child_product(KeT, j, &Gh[j * KE]);
    M.galerkin_child = dalloc(8 * KE * sizeof(double));
    GMGS_CUDA(cudaMemcpyAsync(M.galerkin_child.p, Gh.data(), 8 * KE * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    // Mixed precision with a density field: the level-2 matrices are kept in
    // FP32 only and level 3 is built from the 64 finest descendants
    // (about 60 % less device memory on large models).
    const bool lean = M.has_density && M.prm.precision == GMGS_MIXED && L >= 3;
    DevBuf G2;
    if (lean) {
        std::vector<double> G2h(64 * KE);
        for (int cc = 0; cc < 8; ++cc)
            for (int j = 0; j < 8; ++j) child_product(&Gh[j * KE], cc, &G2h[(cc * 8 + j) * KE]);
        G2 = dalloc(64 * KE * sizeof(double));
        GMGS_CUDA(cudaMemcpyAsync(G2.p, G2h.data(), 64 * KE * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    }
    M.lean_level1 = lean;
    // Galerkin matrices level by level
    for (int l = 1; l < L; ++l) {
        Level& lv = M.levels[l];
        Level& fv = M.levels[l - 1];
        if (lean && l == 1) {
            lv.Ks64.release();
            lv.Ks32 = dalloc(std::max<int64_t>(1, lv.nK) * KE * sizeof(float));
            if (lv.nK > 0) {
                k_galerkin<<<(unsigned)lv.nK, 192, 0, c.stream>>>(
                    lv.g, fv.g, lv.kslot.as<int32_t>(), fv.emask.as<uint8_t>(), fv.etype.as<int32_t>(), nullptr,
                    M.galerkin_child.as<double>(), fv.kscale, fv.escale64.as<double>(), nullptr, lv.Ks32.as<float>());
                GMGS_LAUNCHED(c);
            }
            continue;
        }
        lv.Ks64 = dalloc(std::max<int64_t>(1, lv.nK) * KE * sizeof(double));
        if (lv.nK > 0 && lean && l == 2) {
            Level& l0 = M.levels[0];
            k_galerkin_grand<<<(unsigned)lv.nK, 192, 0, c.stream>>>(
                lv.g, fv.g, l0.g, lv.kslot.as<int32_t>(), fv.emask.as<uint8_t>(), l0.emask.as<uint8_t>(),
                l0.escale64.as<double>(), l0.kscale, G2.as<double>(), lv.Ks64.as<double>());
            GMGS_LAUNCHED(c);
        } else if (lv.nK > 0) {
            k_galerkin<<<(unsigned)lv.nK, 192, 0, c.stream>>>(
                lv.g, fv.g, lv.kslot.as<int32_t>(), fv.emask.as<uint8_t>(), fv.etype.as<int32_t>(),
                fv.Ks64.as<double>(), M.galerkin_child.as<double>(), fv.kscale,
                l == 1 ? fv.escale64.as<double>() : nullptr, lv.Ks64.as<double>(), nullptr);
            GMGS_LAUNCHED(c);
        }
    }
    c.trace_point("create: Galerkin coarse matrices");
    // diagonals (levels 1..L-1) and FP32 copies for the mixed V-cycle
    for (int l = 0; l < L; ++l) {
        Level& lv = M.levels[l];
        if (l < L - 1) {
            lv.diag64 = dalloc(3 * lv.g.slots * sizeof(double));
            if (lean && l == 1) {
                Level& l0 = M.levels[0];
                k_diag_children<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(
                    lv.g, l0.g, lv.emask.as<uint8_t>(), lv.nflag.as<uint8_t>(), l0.emask.as<uint8_t>(),
                    l0.escale64.as<double>(), l0.kscale, M.galerkin_child.as<double>(), lv.diag64.as<double>());
            } else if (!lv.etype.p && !(l == 0 && lv.escale64.p)) {
                DevBuf table = dalloc(3 * 256 * sizeof(double));
                k_diag_table<<<1, 256, 0, c.stream>>>(ke0, lv.kscale, nullptr, table.as<double>());
                GMGS_LAUNCHED(c);
                k_diag_uniform<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(
                    lv.g, lv.emask.as<uint8_t>(), lv.nflag.as<uint8_t>(), table.as<double>(), lv.diag64.as<double>());
                GMGS_LAUNCHED(c);
                GMGS_CUDA(cudaStreamSynchronize(c.stream));
            } else {
                k_diag<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(
                    lv.g, lv.emask.as<uint8_t>(), lv.nflag.as<uint8_t>(), lv.etype.as<int32_t>(), lv.Ks64.as<double>(),
                    ke0, lv.kscale, l == 0 ? lv.escale64.as<double>() : nullptr, lv.diag64.as<double>());
            }
            GMGS_LAUNCHED(c);
        }
        if (M.prm.precision == GMGS_MIXED) {
            if (lv.nK > 0 && l < L - 1 && !(lean && l == 1)) {
                lv.Ks32 = dalloc(lv.nK * KE * sizeof(float));
                k_to_float<<<blocks_for(c, lv.nK * KE), 256, 0, c.stream>>>(lv.nK * KE, lv.Ks64.as<double>(),
                                                                             lv.Ks32.as<float>());
                GMGS_LAUNCHED(c);
            }
            if (l < L - 1) {
                lv.diag32 = dalloc(3 * lv.g.slots * sizeof(float));
                k_to_float<<<blocks_for(c, 3 * lv.g.slots), 256, 0, c.stream>>>(3 * lv.g.slots, lv.diag64.as<double>(),
                                                                                 lv.diag32.as<float>());
                GMGS_LAUNCHED(c);
            }
            if (l == 0 && lv.escale64.p) {
                lv.escale32 = dalloc(lv.g.slots * sizeof(float));
                k_to_float<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g.slots, lv.escale64.as<double>(),
                                                                             lv.escale32.as<float>());
                GMGS_LAUNCHED(c);
            }
        }
    }
    GMGS_CUDA(cudaStreamSynchronize(c.stream));
    c.trace_point("create: diagonals + FP32 copies");
}

void apply_bc(Model& M, const int32_t* fixed, int64_t nfixed, const double* loads, int64_t nload) {
    Ctx& c = M.ctx;
    Level& lv = M.levels[0];
    const int64_t nn = lv.n_node;
    for (int64_t i = 0; i < nfixed; ++i)
        if (fixed[i] < 1 || fixed[i] > nn) throw Error(GMGS_ERR_INVALID_ARGUMENT, "fixed node id out of range");
    for (int64_t i = 0; i < nload; ++i) {
        const double idd = loads[4 * i];
        if (!(idd >= 1 && idd <= (double)nn) || idd != std::floor(idd))
            throw Error(GMGS_ERR_INVALID_ARGUMENT, "load node id out of range");
        for (int k = 1; k < 4; ++k)
            if (!std::isfinite(loads[4 * i + k])) throw Error(GMGS_ERR_NONFINITE, "non-finite load");
    }
    DevBuf dfix = dalloc(std::max<int64_t>(1, nfixed) * sizeof(int32_t));
    DevBuf dld = dalloc(std::max<int64_t>(1, nload) * 4 * sizeof(double));
    DevBuf last = dalloc(std::max<int64_t>(1, nn) * sizeof(int32_t));
    GMGS_CUDA(cudaMemcpyAsync(dfix.p, fixed, nfixed * sizeof(int32_t), cudaMemcpyHostToDevice, c.stream));
    GMGS_CUDA(cudaMemcpyAsync(dld.p, loads, nload * 4 * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    GMGS_CUDA(cudaMemsetAsync(last.p, 0xff, std::max<int64_t>(1, nn) * sizeof(int32_t), c.stream));   // -1
    k_clear_fixed<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g.slots, lv.nflag.as<uint8_t>());
    GMGS_LAUNCHED(c);
    k_set_fixed<<<blocks_for(c, nfixed), 256, 0, c.stream>>>(nfixed, dfix.as<int32_t>(), lv.node_slot.as<int32_t>(),
                                                              lv.nflag.as<uint8_t>());
    GMGS_LAUNCHED(c);
    if (!M.F.p) M.F = dalloc(3 * lv.g.slots * sizeof(double));
    GMGS_CUDA(cudaMemsetAsync(M.F.p, 0, 3 * lv.g.slots * sizeof(double), c.stream));
    k_load_last<<<blocks_for(c, nload), 256, 0, c.stream>>>(nload, dld.as<double>(), last.as<int32_t>());
    GMGS_LAUNCHED(c);
    k_set_loads<<<blocks_for(c, nload), 256, 0, c.stream>>>(nload, dld.as<double>(), last.as<int32_t>(),
                                                            lv.node_slot.as<int32_t>(), lv.g.slots, M.F.as<double>());
    GMGS_LAUNCHED(c);
    GMGS_CUDA(cudaStreamSynchronize(c.stream));
}

void build_coarse_bc(Model& M, const std::function<void()>& overlap) {
    Ctx& c = M.ctx;
    const int L = M.num_levels;
    // restricted fixed indicator, level by level (SetupSolver.m:247-254)
    // the indicator in FP32: its restrictions sum non-negative terms (0/1 values
    // times the weights 1, 1/2, 1/4, 1/8), so a coarse entry is nonzero exactly
    // when one of its terms is, in FP32 as in FP64; only that test is used
    DevBuf ind = dalloc(3 * M.levels[0].g.slots * sizeof(float));
    k_indicator<<<blocks_for(c, M.levels[0].g.slots), 256, 0, c.stream>>>(
        M.levels[0].g.slots, M.levels[0].nflag.as<uint8_t>(), ind.as<float>());
    GMGS_LAUNCHED(c);
    for (int l = 1; l < L; ++l) {
        Level& lv = M.levels[l];
        DevBuf indc = dalloc(3 * lv.g.slots * sizeof(float));
        GMGS_CUDA(cudaMemsetAsync(indc.p, 0, 3 * lv.g.slots * sizeof(float), c.stream));
        launch_restrict<float>(c, M.levels[l - 1].g, lv.g, lv.nflag.as<uint8_t>(), ind.as<float>(),
                               indc.as<float>());
        k_fixed_from_indicator<<<blocks_for(c, lv.g.slots), 256, 0, c.stream>>>(lv.g.slots, indc.as<float>(),
                                                                                 lv.nflag.as<uint8_t>());
        GMGS_LAUNCHED(c);
        GMGS_CUDA(cudaStreamSynchronize(c.stream));
        ind = std::move(indc);
    }
    c.trace_point("bc: restricted fixed indicator");
    // coarsest free DOFs and their block-tridiagonal factorisation
    Level& lc = M.levels[L - 1];
    const int64_t S = lc.g.slots;
    DevBuf cnt = dalloc(3 * S * sizeof(int32_t));
    k_free_count<<<blocks_for(c, 3 * S), 256, 0, c.stream>>>(S, lc.nflag.as<uint8_t>(), cnt.as<int32_t>());
    GMGS_LAUNCHED(c);
    const int64_t nf = exclusive_scan(c, cnt.as<int32_t>(), 3 * S);
    if (nf == 0) throw Error(GMGS_ERR_NOT_SPD, "no free DOFs on the coarsest level");
    M.nfree = (int)nf;
    M.free_idx = dalloc(nf * sizeof(int32_t));
    k_free_list<<<blocks_for(c, 3 * S), 256, 0, c.stream>>>(S, lc.nflag.as<uint8_t>(), cnt.as<int32_t>(),
                                                             M.free_idx.as<int32_t>());
    GMGS_LAUNCHED(c);
    DevBuf rank = dalloc(3 * S * sizeof(int32_t));
    k_rank_fill<<<blocks_for(c, 3 * S), 256, 0, c.stream>>>(3 * S, rank.as<int32_t>());
    GMGS_LAUNCHED(c);
    k_rank_set<<<blocks_for(c, nf), 256, 0, c.stream>>>(nf, M.free_idx.as<int32_t>(), rank.as<int32_t>());
    GMGS_LAUNCHED(c);
    // The free DOFs are numbered node by node in slot order, so the matrix is
    // banded: blocks of order B >= the half bandwidth make it block
    // tridiagonal (factor_coarse, coarse.cu).
    const int n = (int)nf;
    int bw = 0;
    {
        DevBuf dbw = dalloc(sizeof(int));
        GMGS_CUDA(cudaMemsetAsync(dbw.p, 0, sizeof(int), c.stream));
        k_coarse_bandwidth<<<blocks_for(c, (int64_t)n * 81), 256, 0, c.stream>>>(
            lc.g, n, M.free_idx.as<int32_t>(), rank.as<int32_t>(), lc.emask.as<uint8_t>(), lc.etype.as<int32_t>(),
            lc.Ks64.as<double>(), M.ke0_dev.as<double>(), lc.kscale, dbw.as<int>());
        GMGS_LAUNCHED(c);
        GMGS_CUDA(cudaMemcpyAsync(&bw, dbw.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        GMGS_CUDA(cudaStreamSynchronize(c.stream));
    }
    CoarseBlocks& cb = M.cb;
    cb = CoarseBlocks();
    cb.n = n;
    cb.B = coarse_block_order(n, bw);
    cb.nb = (n + cb.B - 1) / cb.B;
    const int64_t npad = (int64_t)cb.nb * cb.B;
    const size_t blk_bytes = (size_t)cb.nb * cb.B * cb.B * sizeof(double);
    if (blk_bytes > ((size_t)16 << 30))
        throw Error(GMGS_ERR_RESOLUTION, "coarsest level too large for the block factorisation; use more levels");
    cb.sinv = dalloc(blk_bytes);
    cb.g = dalloc(blk_bytes);
    GMGS_CUDA(cudaMemsetAsync(cb.sinv.p, 0, blk_bytes, c.stream));
    GMGS_CUDA(cudaMemsetAsync(cb.g.p, 0, blk_bytes, c.stream));
    k_assemble_blocks<<<blocks_for(c, (int64_t)n * 81), 256, 0, c.stream>>>(
        lc.g, n, M.free_idx.as<int32_t>(), rank.as<int32_t>(), lc.emask.as<uint8_t>(), lc.etype.as<int32_t>(),
        lc.Ks64.as<double>(), M.ke0_dev.as<double>(), lc.kscale, cb.B, cb.sinv.as<double>(), cb.g.as<double>());
    GMGS_LAUNCHED(c);
    if (npad > n) {
        k_pad_identity<<<(unsigned)((npad - n + 255) / 256), 256, 0, c.stream>>>(n, (int)npad, cb.B,
                                                                               cb.sinv.as<double>());
        GMGS_LAUNCHED(c);
    }
    c.trace_point("bc: coarsest free DOFs + block assembly");
    factor_coarse(c, cb, overlap);
    M.cvec_in = dalloc(npad * sizeof(double));
    M.cvec_out = dalloc(npad * sizeof(double));
    GMGS_CUDA(cudaMemsetAsync(M.cvec_in.p, 0, npad * sizeof(double), c.stream));
    GMGS_CUDA(cudaMemsetAsync(M.cvec_out.p, 0, npad * sizeof(double), c.stream));
    GMGS_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace gmgs
