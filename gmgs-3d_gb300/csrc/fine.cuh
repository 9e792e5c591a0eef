// Tiled FP32 operator kernels of the mixed-precision path (fine.cu).
#pragma once

#include "gmgs_internal.cuh"

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
    const float* escale;     // finest-level element scale or null
    float kscale;
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
                              //                                  (CG_solver.m:31-35, 18-19)
    FM_CG_DIRECTION = 3       // v = fl32(z + beta p_old), p = v, q = A v, p.q  (CG_solver.m:23-31)
};

struct FineArgs {
    const float* v = nullptr;        // FM_PLAIN input
    const float* r32 = nullptr;      // FM_VCYCLE_DOWN / FM_CG_UPDATE_JACOBI residual in FP32 (read on the halo)
    double* r64 = nullptr;           // FM_CG_UPDATE_JACOBI residual in FP64 (owned nodes, updated in place)
    const float* wdinv = nullptr;    // omega / diag (3 planes)
    const float* z32 = nullptr;      // FM_CG_DIRECTION preconditioned residual
    const float* pold = nullptr;     // previous direction (FM_CG_DIRECTION: p_{k-1}; FM_CG_UPDATE_JACOBI: p_k)
    const float* q32 = nullptr;      // FM_CG_UPDATE_JACOBI: q = A p of the previous iteration
    const double* scal = nullptr;    // CG scalars: [0],[1] r.z by parity, [2] p.q
    int cur = 0, first = 0;
    float* out32 = nullptr;          // y / r' / q
    float* pout = nullptr;           // new direction (must not alias pold)
    double* x64 = nullptr;           // solution (owned nodes, in place)
    float* r32out = nullptr;         // FP32 copy of the updated residual (must not alias r32)
    DotOut dot;
};

constexpr uint8_t NF_INTERIOR = 16;
constexpr uint8_t NF_PEREL = 32;     // node touches an element with its own stored matrix

void make_stencil(const double* ke_rows, Coef32& cf);
int fine_grid_blocks(const Grid& g);
int up32_grid_blocks(const Grid& gf);

template <int MODE>
void launch_fine(Ctx& c, const FineLevel& L, const Coef32& cf, const FineArgs& a);

void launch_up32(Ctx& c, const Grid& gf, const Grid& gc, const uint8_t* nflag, const float* wdinv, const float* r,
                 const float* rp, const float* xc, float* xf, bool zero_fixed, const DotOut* dot);
void launch_wdinv(Ctx& c, int64_t n, const double* d, double omega, float* w);
void launch_perel_vdown(Ctx& c, const FineLevel& L, const Coef32& cf, const int32_t* nodes, int count, const float* r,
                        const float* w, float* out);
void launch_emask8(Ctx& c, const Grid& g, const uint8_t* emask, uint8_t* e8);
void launch_to_f32(Ctx& c, int64_t n, const double* a, float* b);
void launch_drop_last_dx(Ctx& c, int64_t n, double* x, const float* r32, const float* q, const float* w,
                         const double* scal, int cur, int first);

}  // namespace gmgs
