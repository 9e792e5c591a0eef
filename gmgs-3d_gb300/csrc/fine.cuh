// Tiled FP32 operator kernels of the mixed-precision path (fine.cu).
#pragma once

#include <cuda.h>                   // CUtensorMap (types only; the encoder is fetched from the driver at run time)

#include "gmgs_internal.cuh"
#include "gmgs_default_stencil.h"   // generated at build time (build.py)

namespace gmgs {

// coefficients passed by value as a __grid_constant__ kernel parameter, so
// handles with different materials never share device state
struct Coef32 {
    float S[27 * 9];   // assembled interior stencil, block k = (dz+1)*9 + (dx+1)*3 + (dy+1), row-major 3x3
    float K[KE];       // element matrix Ke0, row = output DOF
};

// one level as the fused kernels see it
struct FineLevel {
    Grid g;
    const uint8_t* emask;
    const uint8_t* nflag;    // NF_INTERIOR: all 8 elements carry kscale * Ke0
    const uint8_t* emask8;   // per node: bit A + 2B + 4C set when the element at node - (A, B, C) is solid
    const int32_t* etype;    // null: every solid element uses kscale * Ke0
    const float* Ks;         // per-element matrices (FP32), row = output DOF
    int64_t nK = 0;          // matrices held in Ks (the extent checked builds test element types against)
    const float* escale;     // finest-level element scale or null
    float kscale;
    const uint8_t* tile_occ; // per (z plane, x tile, y tile) of the streaming kernel: any solid node; null = all
};

struct DotOut {
    double* partials = nullptr;   // one per block
    unsigned int* ticket = nullptr;
    double* out = nullptr;
};

enum FineMode {
    FM_PLAIN = 0,             // y = A v
    FM_VCYCLE_DOWN = 1,       // v = w r, out = r - A v               (Vcycle.m:14, JacobiSmoother.m:5-9)
    FM_CG_UPDATE_JACOBI = 2,  // previous CG update r_m = r - alpha q, x += alpha p, r_m.r_m;
                              // then the Jacobi step v = fl32(w r_m), x += v, r = r_m - A v
                              // (x and r double-float)           (CG_solver.m:31-35, 18-19)
    FM_CG_DIRECTION = 3       // v = fl32(z + beta p_old), p = v, q = A v, p.q  (CG_solver.m:23-31)
};

struct FineArgs {
    const float* v = nullptr;        // FM_PLAIN input
    const float* r32 = nullptr;      // FM_VCYCLE_DOWN residual; FM_CG_UPDATE_JACOBI: its high part (read on the halo)
    float* r_lo = nullptr;           // FM_CG_UPDATE_JACOBI residual, low part (owned nodes, updated in place)
    const float* wdinv = nullptr;    // omega / diag (3 planes)
    const float* z32 = nullptr;      // FM_CG_DIRECTION preconditioned residual
    const float* pold = nullptr;     // previous direction (FM_CG_DIRECTION: p_{k-1}; FM_CG_UPDATE_JACOBI: p_k)
    const float* q32 = nullptr;      // FM_CG_UPDATE_JACOBI: q = A p of the previous iteration
    const double* scal = nullptr;    // CG scalars: [0],[1] r.z by parity, [2] p.q
    int cur = 0, first = 0;
    float* out32 = nullptr;          // y / r' / q
    float* pout = nullptr;           // new direction (must not alias pold)
    float* x_hi = nullptr;           // solution, double-float high and low parts (owned nodes, in place)
    float* x_lo = nullptr;
    float* r32out = nullptr;         // high part of the updated residual (must not alias r32)
    DotOut dot;
    int* err = nullptr;              // set when a bounded wait for staged operands ran out
};

// TMA descriptors of the streaming kernels, each a (y, x, z, component)
// tensor over the dense slot grid:
//  m: FM_CG_UPDATE_JACOBI's per-node operands (r high, r low, x high, x low,
//     q, p), a 32 x 8 x 1 x 3 box: one tile plane of all three components;
//  f: the field inputs of the mode (FM_PLAIN v; FM_VCYCLE_DOWN r, omega/diag;
//     FM_CG_UPDATE_JACOBI r high, omega/diag, q; FM_CG_DIRECTION z, p), a
//     40 x 10 x 1 x 3 box: the tile plane with its one-node halo, from y - 4
//     so that the box starts on a 16-byte boundary.
constexpr int EPI_ARRAYS = 6;
constexpr int FIELD_ARRAYS = 3;
struct EpiMaps {
    CUtensorMap m[EPI_ARRAYS];
    CUtensorMap f[FIELD_ARRAYS];
};


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
// reductions
// ---------------------------------------------------------------------------
struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

__device__ __forceinline__ double block_sum_d(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int w = tid >> 5, l = tid & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    v = 0;
    if (w == 0) {
        v = l < (int)((blockDim.x * blockDim.y) >> 5) ? sh[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;   // valid in thread 0
}

// deterministic grid reduction: partial per block, the last block sums them in order
__device__ inline void grid_dot_finish(double v, const DotOut& d, double* sh) {
    __shared__ bool last;
    v = block_sum_d(v, sh);
    const int nthr = blockDim.x * blockDim.y;
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
        for (unsigned i = tid; i < nb; i += nthr) t += __ldcg(d.partials + i);
        t = block_sum_d(t, sh);
        if (tid == 0) {
            *d.out = t;
            *d.ticket = 0;
        }
    }
}

// input field at one point (3 components) from the kernel's inputs
template <int MODE>
__device__ __forceinline__ void field_at(const FineArgs& a, int S, int s, float beta, float alpha, float v[3]) {
    const long long n3 = 3ll * S;
    constexpr int F = chk::FINE_FIELD;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int i = s + c * S;
        if (MODE == FM_PLAIN) {
            v[c] = chk::ld(a.v, i, n3, F);
        } else if (MODE == FM_VCYCLE_DOWN) {
            v[c] = chk::ld(a.r32, i, n3, F) * chk::ld(a.wdinv, i, n3, F);
        } else if (MODE == FM_CG_UPDATE_JACOBI) {
            const float r = chk::ld(a.r32, i, n3, F);
            const float rm = a.first ? r : fmaf(-alpha, chk::ld(a.q32, i, n3, F), r);
            v[c] = rm * chk::ld(a.wdinv, i, n3, F);
        } else {   // FM_CG_DIRECTION
            const float z = chk::ld(a.z32, i, n3, F);
            v[c] = a.first ? z : fmaf(beta, chk::ld(a.pold, i, n3, F), z);
        }
    }
}

// ---------------------------------------------------------------------------
// stencil arithmetic on the shared-memory ring
// ---------------------------------------------------------------------------
// interior node, second-difference form; P0, P1, P2 = planes z-1, z, z+1
// DEF: the coefficients are the compiled-in default-material tables (dflt::S,
// dflt::K: instruction immediates) instead of the kernel parameter cf
template <int RP, int PLANE, bool DEF = false>
__device__ __forceinline__ void interior_s(const Coef32& cf, const float* __restrict__ P0, const float* __restrict__ P1,
                                           const float* __restrict__ P2, int p, float& y0, float& y1, float& y2) {
    constexpr long long R = 3 * PLANE;   // one ring slot
    const float c0 = chk::ld(P1, p, R, chk::FINE_RING), c1 = chk::ld(P1, p + PLANE, R, chk::FINE_RING),
                c2 = chk::ld(P1, p + 2 * PLANE, R, chk::FINE_RING);
    float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 14; k < 27; ++k) {
        const int o = off_y(k) + off_x(k) * RP;
        const float* up = off_z(k) > 0 ? P2 : (off_z(k) < 0 ? P0 : P1);
        const float* dn = off_z(k) > 0 ? P0 : (off_z(k) < 0 ? P2 : P1);
        float d[3];
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const float cb = b == 0 ? c0 : (b == 1 ? c1 : c2);
            d[b] = (chk::ld(up, p + o + b * PLANE, R, chk::FINE_RING) - cb) +
                   (chk::ld(dn, p - o + b * PLANE, R, chk::FINE_RING) - cb);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
                if (s_nonzero(k, a, b)) acc[a] = fmaf(DEF ? dflt::S(k * 9 + 3 * a + b) : cf.S[k * 9 + 3 * a + b], d[b], acc[a]);
    }
    y0 = acc[0]; y1 = acc[1]; y2 = acc[2];
}

// rows of one element (node at corner CI of the element with origin offset
// (A, B, C)), first-difference form, coefficients K (row = output DOF) * s
template <int RP, int PLANE, int A, int B, int C, bool PARAM, bool DEF = false>
__device__ __forceinline__ void elem_rows(const Coef32& cf, const float* __restrict__ Kg, float s,
                                          const float* __restrict__ P0, const float* __restrict__ P1,
                                          const float* __restrict__ P2, int p, float c0, float c1, float c2,
                                          float& y0, float& y1, float& y2) {
    constexpr int CI = corner_of(A, B, C);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (j == CI) continue;
        const int dy = corner_y(j) - A, dx = corner_x(j) - B, dz = corner_z(j) - C;
        const float* pl = dz > 0 ? P2 : (dz < 0 ? P0 : P1);
        const int q = p + dy + dx * RP;
        constexpr long long R = 3 * PLANE;
        const float d0 = chk::ld(pl, q, R, chk::FINE_RING) - c0, d1 = chk::ld(pl, q + PLANE, R, chk::FINE_RING) - c1,
                    d2 = chk::ld(pl, q + 2 * PLANE, R, chk::FINE_RING) - c2;
        float t[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int r = (3 * CI + a) * 24 + 3 * j;
            if (PARAM && DEF) {
                t[a] = fmaf(dflt::K(r + 2), d2, fmaf(dflt::K(r + 1), d1, dflt::K(r) * d0));
            } else if (PARAM) {
                t[a] = fmaf(cf.K[r + 2], d2, fmaf(cf.K[r + 1], d1, cf.K[r] * d0));
            } else {
                t[a] = fmaf(Kg[r + 2], d2, fmaf(Kg[r + 1], d1, Kg[r] * d0));
            }
        }
        y0 = fmaf(s, t[0], y0);
        y1 = fmaf(s, t[1], y1);
        y2 = fmaf(s, t[2], y2);
    }
}

template <int RP, int PLANE, int E, bool DEF = false>
__device__ __forceinline__ void boundary_elem(const FineLevel& L, const Coef32& cf, uint32_t e8, int n,
                                              const float* __restrict__ P0, const float* __restrict__ P1,
                                              const float* __restrict__ P2, int p, float c0, float c1, float c2,
                                              float& y0, float& y1, float& y2) {
    constexpr int A = E & 1, B = (E >> 1) & 1, C = E >> 2;
    if (!((e8 >> E) & 1u)) return;
    const int es = n - A - B * L.g.py - C * L.g.py * L.g.px;
    float s = L.kscale;
    if (L.etype) {
        const int t = chk::ld(L.etype, es, L.g.slots, chk::FINE_ELEM);
        if (t > 0) {
            if (chk::ok(t - 1, L.nK, chk::FINE_KS))
                elem_rows<RP, PLANE, A, B, C, false>(cf, L.Ks + (int64_t)(t - 1) * KE, 1.f, P0, P1, P2, p, c0, c1, c2,
                                                     y0, y1, y2);
            return;
        }
    }
    if (L.escale) s *= chk::ld(L.escale, es, L.g.slots, chk::FINE_ELEM);
    elem_rows<RP, PLANE, A, B, C, true, DEF>(cf, nullptr, s, P0, P1, P2, p, c0, c1, c2, y0, y1, y2);
}

template <int RP, int PLANE, bool DEF = false>
__device__ __forceinline__ void boundary_s(const FineLevel& L, const Coef32& cf, uint32_t e8, int n,
                                           const float* __restrict__ P0, const float* __restrict__ P1,
                                           const float* __restrict__ P2, int p, float& y0, float& y1, float& y2) {
    constexpr long long R = 3 * PLANE;
    const float c0 = chk::ld(P1, p, R, chk::FINE_RING), c1 = chk::ld(P1, p + PLANE, R, chk::FINE_RING),
                c2 = chk::ld(P1, p + 2 * PLANE, R, chk::FINE_RING);
    y0 = y1 = y2 = 0.f;
    boundary_elem<RP, PLANE, 0, DEF>(L, cf, e8, n, P0, P1, P2, p, c0, c1, c2, y0, y1, y2);
    boundary_elem<RP, PLANE, 1, DEF>(L, cf, e8, n, P0, P1, P2, p, c0, c1, c2, y0, y1, y2);
    boundary_elem<RP, PLANE, 2, DEF>(L, cf, e8, n, P0, P1, P2, p, c0, c1, c2, y0, y1, y2);
    boundary_elem<RP, PLANE, 3, DEF>(L, cf, e8, n, P0, P1, P2, p, c0, c1, c2, y0, y1, y2);
    boundary_elem<RP, PLANE, 4, DEF>(L, cf, e8, n, P0, P1, P2, p, c0, c1, c2, y0, y1, y2);
    boundary_elem<RP, PLANE, 5, DEF>(L, cf, e8, n, P0, P1, P2, p, c0, c1, c2, y0, y1, y2);
    boundary_elem<RP, PLANE, 6, DEF>(L, cf, e8, n, P0, P1, P2, p, c0, c1, c2, y0, y1, y2);
    boundary_elem<RP, PLANE, 7, DEF>(L, cf, e8, n, P0, P1, P2, p, c0, c1, c2, y0, y1, y2);
}


constexpr uint8_t NF_PEREL = 32;     // node touches an element with its own stored matrix

// B operand of the tensor-core element kernels (tc.cu): Ke (row = output DOF)
// as TF32 in the tensor cores' K-major no-swizzle shared-memory layout, N
// padded to 32 rows.
struct TcCoef {
    float B[32 * 24];
};
void make_tc_coef(const double* ke_rows, TcCoef& c);
// V-cycle down-sweep out = r - A (w r) on the tensor cores, element form
// (err: device flag set when a tensor-core wait runs out)
void launch_tc_vdown(Ctx& c, const FineLevel& L, const TcCoef& cf, const float* r32, const float* wdinv, float* out,
                     int* err);
size_t tc_tile_occ_bytes(const Grid& g);
void launch_tc_tile_occ(Ctx& c, const Grid& g, const uint8_t* nflag, uint8_t* occ);

void make_stencil(const double* ke_rows, Coef32& cf);
int fine_grid_blocks(const Grid& g);
int up32_grid_blocks(const Grid& gf);

template <int MODE>
void launch_fine(Ctx& c, const FineLevel& L, const Coef32& cf, const FineArgs& a);

void launch_up32(Ctx& c, const Grid& gf, const Grid& gc, const uint8_t* nflag, const uint8_t* tile_occ,
                 const float* wdinv, const float* r, const float* rp, const float* xc, float* xf, bool zero_fixed,
                 const DotOut* dot);
void launch_wdinv(Ctx& c, int64_t n, const double* d, double omega, float* w);
void launch_perel_vdown(Ctx& c, const FineLevel& L, const Coef32& cf, const int32_t* nodes, int count, const float* r,
                        const float* w, float* out);
void launch_emask8(Ctx& c, const Grid& g, const uint8_t* emask, uint8_t* e8);
size_t tile_occ_bytes(const Grid& g);
void launch_tile_occ(Ctx& c, const Grid& g, const uint8_t* nflag, uint8_t* occ);
void launch_to_f32(Ctx& c, int64_t n, const double* a, float* b);
// x = x_hi + x_lo - (the last Jacobi step), written in FP64
void launch_drop_last_dx(Ctx& c, int64_t n, double* x, float* x_hi, float* x_lo, const float* r32, const float* q,
                         const float* w, const double* scal, int cur, int first);
// b -> (hi, lo) = (fl32(b), fl32(b - hi))
void launch_df_split(Ctx& c, int64_t n, const double* b, float* hi, float* lo);

}  // namespace gmgs
