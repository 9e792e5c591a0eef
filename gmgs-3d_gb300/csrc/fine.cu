// Streaming FP32 operator kernels of the mixed-precision path.
//
// One CTA owns a 32 x 8 column of nodes (y fastest) and walks it through z
// with a four-plane ring of the input field (plus a one-node halo) in shared
// memory.  The field is formed while staging from the kernel's inputs (the
// Jacobi step omega*D^-1 r, or the CG direction z + beta p), so no
// intermediate vector goes through HBM.  The field inputs of the plane two
// steps ahead (with the halo) and, in the CG update, the per-node operands of
// the current plane are copied into shared-memory stages by TMA
// (cp.async.bulk.tensor, one thread per CTA, mbarrier completion) while the
// current plane is computed, so the loads overlap the stencil arithmetic
// without holding registers; the per-thread register form of both remains
// (GMGS_FIELD_TMA=0, GMGS_EPI_TMA=0, or no tensor-map encoder in the driver).
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
//
// The outer CG keeps x and r as double-float vectors (hi + lo, two FP32
// arrays, about 48 significant bits) updated with FP32-formed increments by
// two-sums on the FP32 pipe; the high part of r is the FP32 residual the
// stencil reads.  Dot products sum FP32 products with per-thread compensated
// (Kahan) FP32 sums and FP64 across threads and blocks.  (GB300 issues FP64
// arithmetic and FP32<->FP64 conversions at about 2 lanes per clock per SM,
// 1/64 of its FP32 rate: in FP64 the five operations per DOF of the state
// update kept that pipe 53 % busy and the kernel at 2.41 ms on the 153M-DOF
// model.)
#include <atomic>
#include <cstring>
#include <type_traits>

#include "element_host.h"
#include "fine.cuh"
#include "tcgen05.cuh"

namespace gmgs {

constexpr int TY = 32, TX = 8;
constexpr int HY = TY + 2, HX = TX + 2;
constexpr int NT = TY * TX;
constexpr int RP = 40;                  // shared-memory row pitch (>= HY; 8 mod 32 keeps 8x4 warp patches conflict-free)
constexpr int PLANE = RP * HX;          // floats per component plane (34 x 10 points used)
constexpr int NHALO = HY * HX - NT;     // 84 halo points per plane
// Four ring slots need one barrier per plane: the slot written for plane z+1
// in step z differs from the three slots (z-2, z-1, z) a thread still in step
// z-1 may be reading.
constexpr int RING = 4;

// ---------------------------------------------------------------------------
// host: assembled interior stencil from the element matrix (row = output DOF)
// ---------------------------------------------------------------------------
void make_stencil(const double* ke_rows, Coef32& cf) {
    double S[27][9];
    stencil_from_rows(ke_rows, S);
    for (int k = 0; k < 27; ++k)
        for (int i = 0; i < 9; ++i) cf.S[k * 9 + i] = (float)S[k][i];
    for (int i = 0; i < KE; ++i) cf.K[i] = (float)ke_rows[i];
}

// ---------------------------------------------------------------------------
// the fused streaming kernel
// ---------------------------------------------------------------------------
// per-node epilogue inputs, loaded before the stencil arithmetic of the plane
struct EpiData {
    float r[3];       // FM_VCYCLE_DOWN: r;  FM_CG_UPDATE_JACOBI: r32
    float q[3];       // FM_CG_UPDATE_JACOBI
    float pp[3];      // FM_CG_UPDATE_JACOBI: p
    float rl[3];      // FM_CG_UPDATE_JACOBI: low part of r
    float xh[3];      // FM_CG_UPDATE_JACOBI: x, loaded with the other operands, before the stencil
    float xl[3];
};

template <int MODE>
__device__ __forceinline__ void epi_fetch(const FineArgs& a, int S, int n, EpiData& d) {
    const long long n3 = 3ll * S;
    constexpr int E = chk::FINE_EPI;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int i = n + c * S;
        if (MODE == FM_VCYCLE_DOWN) d.r[c] = chk::ld(a.r32, i, n3, E);
        if (MODE == FM_CG_UPDATE_JACOBI) {
            d.r[c] = chk::ld(a.r32, i, n3, E);
            d.rl[c] = chk::ld((const float*)a.r_lo, i, n3, E);
            d.xh[c] = chk::ld((const float*)a.x_hi, i, n3, E);
            d.xl[c] = chk::ld((const float*)a.x_lo, i, n3, E);
            if (!a.first) {
                d.q[c] = chk::ld(a.q32, i, n3, E);
                d.pp[c] = chk::ld(a.pold, i, n3, E);
            }
        }
    }
}

// --- TMA staging of the CG update's per-node operands ------------------------
// One tile plane of one array (32 y x 8 x, three components) is a 3 KB box;
// the six arrays of a plane make one 18 KB stage in dynamic shared memory.
// The boxes are written with the 128-byte swizzle: the 16-byte chunk index
// (address bits 4-6) is XORed with the 128-byte row index (bits 7-9), and a
// row here is one x column of 32 y values, so the stage base is aligned to
// 1024 bytes and node (ly, lx) of component c sits at float
//   c * 256 + 32 * lx + ((((ly >> 2) ^ lx) << 2) | (ly & 3)).
constexpr int EPI_BOX = 3 * NT;                              // floats per array and plane
constexpr int EPI_STAGE_BYTES = EPI_ARRAYS * EPI_BOX * 4;
constexpr size_t EPI_DYN_SMEM = EPI_STAGE_BYTES + 1024;      // + alignment slack
constexpr uint64_t EPI_WAIT_NS = 5000000ull;                 // a plane's copies take microseconds
// the thread that arms the stage: lane 0 of the last warp, which stages no
// halo points (threads 0..83 do), so the copies do not lengthen the warp the
// plane's barrier waits for (measured 1.854 -> 1.835 ms against thread 0)
constexpr int EPI_ISSUER = NT - 32;
// The field stage: the mode's field inputs of one plane with the one-node
// halo, a 40 (y, from y0 - 4) x 10 (x, from x0 - 1) x 3 box per array,
// unswizzled (a warp reads an 8 x 4 node patch at row pitch 40, like the
// ring), each array padded to a multiple of 128 bytes.  Ring point p (pitch
// RP = 40, from y0 - 1) is box element p + 3.
constexpr int FLD_BOX = 3 * PLANE;                            // 1200 floats
constexpr int FLD_PITCH = (FLD_BOX * 4 + 127) / 128 * 32;     // 1216 floats
static_assert(RP == 40 && HX == 10, "the field box and the ring share their pitch");
__host__ __device__ constexpr int field_arrays(int mode) {
    return mode == FM_PLAIN ? 1 : (mode == FM_CG_UPDATE_JACOBI ? 3 : 2);
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(mbar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void fence_proxy_async_cta() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// box at (y slot index, x slot index, z slot index, component 0) of a tensor map
__device__ __forceinline__ void tma_load_plane(float* dst, const CUtensorMap* map, int sy, int sx, int sz,
                                               uint64_t* mbar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(tc::smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(sy), "r"(sx), "r"(sz), "r"(0), "r"(tc::smem_u32(mbar))
        : "memory");
}
__device__ __forceinline__ void epi_from_stage(const float* st, int sidx, bool first, EpiData& d) {
    constexpr long long N = EPI_ARRAYS * EPI_BOX;
    constexpr int R = chk::FINE_RING;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int i = c * NT + sidx;
        d.r[c] = chk::ld(st, i, N, R);
        d.rl[c] = chk::ld(st, EPI_BOX + i, N, R);
        d.xh[c] = chk::ld(st, 2 * EPI_BOX + i, N, R);
        d.xl[c] = chk::ld(st, 3 * EPI_BOX + i, N, R);
        if (!first) {
            d.q[c] = chk::ld(st, 4 * EPI_BOX + i, N, R);
            d.pp[c] = chk::ld(st, 5 * EPI_BOX + i, N, R);
        }
    }
}

// 48 registers (5 CTAs per SM) for the stencil-only modes, 40 (6 CTAs) for
// the CG direction with its field staged by TMA (1.073 -> 1.063 ms; the
// down-sweep, which also holds r for its output, spills at 40); the CG update
// holds the state update's operands and keeps 80 registers (3 CTAs), or,
// with the operands staged by TMA (STG bit 0), 64 registers (4 CTAs; 5 CTAs
// at 48 registers spilled and took 2.31 ms against 1.86 ms).
// Measured on the 153M-DOF model: 5 CTAs/SM took the down-sweep from 1.16 to
// 1.13 ms and the direction kernel from 1.26 to 1.22 ms against 4 CTAs/SM.
// STG bit 0: the CG update's operands staged by TMA; bit 1: the field inputs
// staged by TMA (else loaded per thread into registers one plane ahead)
template <int MODE, bool DEF = false, int STG = 0>
__global__ void __launch_bounds__(NT, MODE == FM_CG_UPDATE_JACOBI ? ((STG & 1) ? 4 : 3) : ((MODE == FM_CG_DIRECTION && (STG & 2)) ? 6 : 5))
    k_fine(FineLevel L, const __grid_constant__ Coef32 cf, FineArgs a, int zc, const __grid_constant__ EpiMaps em) {
    constexpr bool TMA = (STG & 1) != 0, FTMA = (STG & 2) != 0;
    static_assert(!TMA || MODE == FM_CG_UPDATE_JACOBI, "operand staging is for the CG update");
    __shared__ float ring[RING][3 * PLANE];
    __shared__ double sh[32];
    const Grid& g = L.g;
    const int S = (int)g.slots;
    const int sz = g.py * g.px;
    const int y0 = blockIdx.x * TY, x0 = blockIdx.y * TX;
    const int zb = blockIdx.z * zc;
    const int ze = min(zb + zc, g.nz + 1);        // node planes [zb, ze)
    if (L.tile_occ) {                             // no solid node in this column tile: nothing to compute
        int any = 0;
        for (int iz = zb; iz < ze; ++iz) any |= L.tile_occ[((int64_t)iz * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x];
        if (!any) {
            if (MODE == FM_CG_DIRECTION || MODE == FM_CG_UPDATE_JACOBI) grid_dot_finish(0.0, a.dot, sh);
            return;
        }
    }
    // warps cover 8 (y) x 4 (x) node patches, so a face of the domain
    // crosses few warps and the boundary path rarely diverges
    const int tid = threadIdx.x + threadIdx.y * TY;
    const int wrp = tid >> 5, lane = tid & 31;
    const int ly = (wrp & 3) * 8 + (lane & 7), lx = (wrp >> 2) * 4 + (lane >> 3);

    // TMA: the plane's six operand arrays go to a shared-memory stage, loaded by
    // one thread (EPI_ISSUER) at the top of the plane's step and read after the stencil
    // arithmetic, so no registers hold them across it; the step's barrier
    // orders the previous plane's reads before the next load
    extern __shared__ unsigned char fine_dyn[];
    __shared__ uint64_t ebar, fbar;
    __shared__ int efail;
    float* stage = nullptr;
    float* fstage = nullptr;
    int sidx = 0;
    int last_phase = -1;      // EPI_ISSUER: the last phase it armed
    if constexpr (TMA) {
        stage = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(fine_dyn) + 1023) & ~uintptr_t(1023));
        sidx = 32 * lx + ((((ly >> 2) ^ lx) << 2) | (ly & 3));
    }
    if constexpr (FTMA) {
        fstage = TMA ? stage + EPI_ARRAYS * EPI_BOX
                     : reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(fine_dyn) + 127) & ~uintptr_t(127));
    }
    if constexpr (TMA || FTMA) {
        if (tid == 0) {
            if (TMA) tc::mbar_init(&ebar, 1);
            if (FTMA) tc::mbar_init(&fbar, 1);
            efail = 0;
            tc::mbar_fence_init();
        }
    }

    // beta = r.z / r_old.z_old, alpha = r.z / p.q: one FP64 division per CTA
    // instead of one per thread on GB300's narrow FP64 pipe
    float beta = 0.f, alpha = 0.f;
    if ((MODE == FM_CG_DIRECTION || MODE == FM_CG_UPDATE_JACOBI) && !a.first) {
        __shared__ float s_ab;
        if (threadIdx.x == 0 && threadIdx.y == 0)
            s_ab = (float)(a.scal[a.cur] / a.scal[MODE == FM_CG_DIRECTION ? (a.cur ^ 1) : 2]);
        __syncthreads();
        (MODE == FM_CG_DIRECTION ? beta : alpha) = s_ab;
    }

    // this thread's centre point and (for tid < NHALO) one halo point of every plane
    const int cy = y0 + ly, cx = x0 + lx;
    const int pc = (ly + 1) + (lx + 1) * RP;
    const bool ccol = cy <= g.ny + 1 && cx <= g.nx + 1;
    const int cbase = (cx + 1) * g.py + (cy + Grid::YOFF) + sz;  // slot(cy, cx, iz) = cbase + iz * sz
    int ph = 0, hbase = 0;
    bool hcol = false;
    if (tid < NHALO) {
        int hy_, hx_;
        if (tid < 2 * HX) { hy_ = (tid & 1) ? HY - 1 : 0; hx_ = tid >> 1; }
        else { const int k = tid - 2 * HX; hx_ = (k & 1) ? HX - 1 : 0; hy_ = 1 + (k >> 1); }
        ph = hy_ + hx_ * RP;
        const int hy = y0 - 1 + hy_, hx = x0 - 1 + hx_;
        hcol = hy >= -1 && hx >= -1 && hy <= g.ny + 1 && hx <= g.nx + 1;
        hbase = (hx + 1) * g.py + (hy + Grid::YOFF) + sz;
    }
    auto fetch = [&](int iz, float vc[3], float vh[3]) {
        vc[0] = vc[1] = vc[2] = 0.f;
        vh[0] = vh[1] = vh[2] = 0.f;
        const bool zok = iz >= -1 && iz <= g.nz + 1;
        if (zok && ccol) field_at<MODE>(a, S, cbase + iz * sz, beta, alpha, vc);
        if (zok && hcol) field_at<MODE>(a, S, hbase + iz * sz, beta, alpha, vh);
    };
    auto store = [&](float* r, const float vc[3], const float vh[3]) {
        constexpr long long R = 3 * PLANE;
#pragma unroll
        for (int c = 0; c < 3; ++c) chk::st(r, pc + c * PLANE, R, chk::FINE_RING, vc[c]);
        if (tid < NHALO) {
#pragma unroll
            for (int c = 0; c < 3; ++c) chk::st(r, ph + c * PLANE, R, chk::FINE_RING, vh[c]);
        }
    };

    float vc[3], vh[3];
    fetch(zb - 1, vc, vh);
    store(ring[(zb - 1 + RING) % RING], vc, vh);
    fetch(zb, vc, vh);
    store(ring[zb % RING], vc, vh);
    fetch(zb + 1, vc, vh);

    const bool own = cy <= g.ny && cx <= g.nx;
    uint32_t f_next = 0, e8_next = 0;
    if (own) {
        f_next = chk::ld(L.nflag, cbase + zb * sz, g.slots, chk::FINE_FLAGS);
        e8_next = chk::ld(L.emask8, cbase + zb * sz, g.slots, chk::FINE_FLAGS);
    }
    Kahan dot;
    // FTMA: the field of plane z from the field stage (ring point p is box element p + 3)
    int nfa = field_arrays(MODE);                 // the first CG iteration has no q / p term
    if (a.first && (MODE == FM_CG_DIRECTION || MODE == FM_CG_UPDATE_JACOBI)) --nfa;
    auto form = [&](int p, float v[3]) {
        constexpr long long N = field_arrays(MODE) * FLD_PITCH;
        constexpr int R = chk::FINE_RING;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int i = c * PLANE + p + 3;
            const float f0 = chk::ld(fstage, i, N, R);
            if (MODE == FM_PLAIN) {
                v[c] = f0;
            } else if (MODE == FM_VCYCLE_DOWN) {
                v[c] = f0 * chk::ld(fstage, FLD_PITCH + i, N, R);                      // r * omega/diag
            } else if (MODE == FM_CG_UPDATE_JACOBI) {
                const float rm = a.first ? f0 : fmaf(-alpha, chk::ld(fstage, 2 * FLD_PITCH + i, N, R), f0);
                v[c] = rm * chk::ld(fstage, FLD_PITCH + i, N, R);
            } else {
                v[c] = a.first ? f0 : fmaf(beta, chk::ld(fstage, FLD_PITCH + i, N, R), f0);   // z + beta p
            }
        }
    };
#pragma unroll 1
    for (int iz = zb; iz < ze; ++iz) {
        if constexpr (FTMA) {
            if (iz == zb) {
                store(ring[(iz + 1) % RING], vc, vh);      // the prologue's per-thread fetch
            } else {
                float fc[3] = {0.f, 0.f, 0.f}, fh[3] = {0.f, 0.f, 0.f};
                if (iz + 1 <= g.nz + 1) {                  // armed in the previous step; every thread waits
                    if (!efail && !tc::mbar_wait_bounded(&fbar, (uint32_t)(iz - 1 - zb) & 1u, EPI_WAIT_NS)) {
                        efail = 1;
                        if (a.err) atomicExch(a.err, 1);
                    }
                    form(pc, fc);
                    if (tid < NHALO) form(ph, fh);
                }
                store(ring[(iz + 1) % RING], fc, fh);
            }
        } else {
            store(ring[(iz + 1) % RING], vc, vh);
        }
        __syncthreads();
        if constexpr (FTMA) {
            // plane iz + 2, read at the top of the next step (armed only when that step exists)
            if (tid == EPI_ISSUER && !efail && iz + 1 < ze && iz + 2 <= g.nz + 1) {
                fence_proxy_async_cta();
                mbar_expect_tx(&fbar, (uint32_t)(nfa * FLD_BOX * 4));
                for (int j = 0; j < nfa; ++j)
                    tma_load_plane(fstage + j * FLD_PITCH, &em.f[j], y0, x0, iz + 3, &fbar);
            }
        }
        if constexpr (TMA) {
            if (tid == EPI_ISSUER && !efail) {
                // the previous plane's copies have landed long ago; waiting for
                // them keeps one phase of the barrier in flight at a time
                const int k = iz - zb;
                if (k == 0 || tc::mbar_wait_bounded(&ebar, (k - 1) & 1, EPI_WAIT_NS)) {
                    const int na = a.first ? 4 : EPI_ARRAYS;
                    fence_proxy_async_cta();
                    mbar_expect_tx(&ebar, (uint32_t)(na * EPI_BOX * 4));
                    for (int j = 0; j < na; ++j)
                        tma_load_plane(stage + j * EPI_BOX, &em.m[j], y0 + Grid::YOFF, x0 + 1, iz + 1, &ebar);
                    last_phase = k;
                } else {
                    efail = 1;
                    if (a.err) atomicExch(a.err, 1);
                }
            }
        }
        if (!FTMA && iz + 2 <= g.nz + 1) fetch(iz + 2, vc, vh);
        const uint32_t f = f_next, e8 = e8_next;
        if (own && iz + 1 < ze) {
            f_next = chk::ld(L.nflag, cbase + (iz + 1) * sz, g.slots, chk::FINE_FLAGS);
            e8_next = chk::ld(L.emask8, cbase + (iz + 1) * sz, g.slots, chk::FINE_FLAGS);
        }
        const float* P0 = ring[(iz - 1 + RING) % RING];
        const float* P1 = ring[iz % RING];
        const float* P2 = ring[(iz + 1) % RING];
        const bool node = own && (f & NF_SOLID) && !(f & NF_PEREL);
        if (node) {
            const int n = cbase + iz * sz;
            EpiData ed;
            if constexpr (!TMA) epi_fetch<MODE>(a, S, n, ed);       // in flight during the stencil arithmetic
            float y[3];
            if (f & NF_INTERIOR) {
                interior_s<RP, PLANE, DEF>(cf, P0, P1, P2, pc, y[0], y[1], y[2]);
                y[0] *= L.kscale; y[1] *= L.kscale; y[2] *= L.kscale;
            } else {
                boundary_s<RP, PLANE, DEF>(L, cf, e8, n, P0, P1, P2, pc, y[0], y[1], y[2]);
            }
            if (f & NF_FIX_X) y[0] = 0.f;
            if (f & NF_FIX_Y) y[1] = 0.f;
            if (f & NF_FIX_Z) y[2] = 0.f;
            if constexpr (TMA) {
                if (!efail && !tc::mbar_wait_bounded(&ebar, (iz - zb) & 1, EPI_WAIT_NS)) {
                    efail = 1;
                    if (a.err) atomicExch(a.err, 1);
                }
                epi_from_stage(stage, sidx, a.first, ed);
            }
            const long long n3 = 3ll * S;
            constexpr int O = chk::FINE_OUT;
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const int i = n + b * S;
                const float v = chk::ld(P1, pc + b * PLANE, 3 * PLANE, chk::FINE_RING);
                if (MODE == FM_PLAIN) {
                    chk::st(a.out32, i, n3, O, y[b]);
                } else if (MODE == FM_VCYCLE_DOWN) {
                    chk::st(a.out32, i, n3, O, ed.r[b] - y[b]);         // r' = r - A (omega D^-1 r)
                } else if (MODE == FM_CG_UPDATE_JACOBI) {
                    // previous iteration's update x += alpha p, r -= alpha q (CG_solver.m:32-33),
                    // then this iteration's Jacobi step x += dx, r -= A dx (CG_solver.m:18-19);
                    // the caller removes the last dx when the solve stops
                    float rinc = y[b];
                    float rm32 = ed.r[b];
                    float xinc = v;
                    if (!a.first) {
                        xinc = fmaf(alpha, ed.pp[b], v);
                        rinc = fmaf(alpha, ed.q[b], rinc);
                        rm32 = fmaf(-alpha, ed.q[b], rm32);
                    }
                    float xh = ed.xh[b], xl = ed.xl[b], rh = ed.r[b], rl = ed.rl[b];
                    df_add(xh, xl, xinc);
                    df_add(rh, rl, -rinc);
                    chk::st(a.x_hi, i, n3, O, xh);
                    chk::st(a.x_lo, i, n3, O, xl);
                    chk::st(a.r_lo, i, n3, O, rl);
                    chk::st(a.r32out, i, n3, O, rh);
                    dot.add(__fmul_rn(rm32, rm32));
                } else {
                    chk::st(a.pout, i, n3, O, v);
                    chk::st(a.out32, i, n3, O, y[b]);                   // q = A p
                    dot.add(__fmul_rn(v, y[b]));
                }
            }
        }
        if constexpr (TMA) {
            // every thread sees each phase complete within its step, so no
            // thread's wait in the next step can meet this phase still pending
            // (a parity wait cannot tell phase k from phase k + 2)
            if (!node && !efail && !tc::mbar_wait_bounded(&ebar, (iz - zb) & 1, EPI_WAIT_NS)) {
                efail = 1;
                if (a.err) atomicExch(a.err, 1);
            }
        }
    }
    if constexpr (TMA) {
        // no copy may still be in flight when the CTA's shared memory is released
        // (every earlier phase completed before the next one was armed)
        if (tid == EPI_ISSUER && last_phase >= 0) tc::mbar_wait_bounded(&ebar, last_phase & 1, EPI_WAIT_NS);
    }
    if (MODE == FM_CG_DIRECTION || MODE == FM_CG_UPDATE_JACOBI) grid_dot_finish(dot.value(), a.dot, sh);
}

static int pick_zc(const Grid& g, const Ctx& c, int per_sm = 3) {
    const int64_t cols = (int64_t)((g.ny + 1 + TY - 1) / TY) * ((g.nx + 1 + TX - 1) / TX);
    // ~24 waves of 3 resident CTAs: shorter z-chunks balance the tail and let
    // empty column tiles of real geometry skip more (12 waves: 214 -> 208 ms
    // on the 153M-DOF block, 286 -> 271 ms on kitten 512; 48 waves: slower)
    const int64_t want = (int64_t)c.num_sms * per_sm * 24;
    int64_t zc = (cols * (g.nz + 1) + want - 1) / want;
    // at least 6 planes per CTA where that still leaves four CTAs per SM (each
    // chunk stages two planes beyond its own: coarse levels 22.17 -> 21.96 ms
    // per solve against 4; 8 was slower), else at least 4 (small grids keep
    // their CTAs spread over all SMs)
    // (the 42x37x64 model: 31.9 ms with 6 everywhere, 30.1 ms so)
    const int64_t zmin = cols * ((g.nz + 1 + 5) / 6) < 4 * (int64_t)c.num_sms ? 4 : 6;
    if (zc < zmin) zc = zmin;
    if (zc > 64) zc = 64;
    return (int)zc;
}

int fine_grid_blocks(const Grid& g) {
    // upper bound over the z-chunk choices (zc >= 4)
    return ((g.ny + 1 + TY - 1) / TY) * ((g.nx + 1 + TX - 1) / TX) * ((g.nz + 1 + 3) / 4);
}

// true when cf holds exactly the compiled-in default-material tables (then
// the kernels with the coefficients as immediates give the same results)
static bool coef_is_default(const Coef32& cf) {
    for (int i = 0; i < 27 * 9; ++i)
        if (cf.S[i] != dflt::S(i) || std::signbit(cf.S[i]) != std::signbit(dflt::S(i))) return false;
    for (int i = 0; i < KE; ++i)
        if (cf.K[i] != dflt::K(i) || std::signbit(cf.K[i]) != std::signbit(dflt::K(i))) return false;
    const char* e = std::getenv("GMGS_DEFAULT_STENCIL");
    return !(e && e[0] == '0');
}

// cuTensorMapEncodeTiled from the driver (the library links only the runtime)
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn tensor_map_encoder() {
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// (y, x, z, component) view of one dense-slot vector: strides py, py*px and
// the component plane (all multiples of 32 bytes: py is a multiple of 8);
// boxes over the grid edge read zeros.  The CG update's stage: one tile plane
// (32 x 8) with the 128-byte swizzle, which spreads its 8 x 4 node patches
// over the banks; the field stage: the tile plane with its halo (40 x 10, from
// y0 - 4 and x0 - 1), unswizzled.
static bool encode_plane_map(CUtensorMap* m, const Grid& g, const float* base, bool field) {
    const EncodeTiledFn fn = tensor_map_encoder();
    if (!fn || !base || (reinterpret_cast<uintptr_t>(base) & 15)) return false;
    const cuuint64_t dim[4] = {(cuuint64_t)g.py, (cuuint64_t)g.px, (cuuint64_t)g.pz, 3};
    const cuuint64_t stride[3] = {(cuuint64_t)g.py * 4, (cuuint64_t)g.py * g.px * 4, (cuuint64_t)g.slots * 4};
    const cuuint32_t box_epi[4] = {TY, TX, 1, 3}, box_fld[4] = {RP, HX, 1, 3};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dim, stride, field ? box_fld : box_epi,
              es, CU_TENSOR_MAP_INTERLEAVE_NONE, field ? CU_TENSOR_MAP_SWIZZLE_NONE : CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// GMGS_EPI_TMA=0 keeps the CG update's operands in registers (per-thread
// loads issued before the stencil arithmetic) instead of the TMA stage;
// GMGS_FIELD_TMA=0 keeps the per-thread field loads one plane ahead instead
// of the field stage
static bool env_on(const char* name) {
    const char* e = std::getenv(name);
    return !(e && e[0] == '0');
}

template <int MODE, bool DEF, int STG>
static void launch_stg(Ctx& c, dim3 grid, const FineLevel& L, const Coef32& cf, const FineArgs& a, int zc,
                       const EpiMaps& em) {
    size_t dyn = 0;
    if (STG & 1) dyn += (size_t)EPI_STAGE_BYTES + 1024;
    if (STG & 2) dyn += (size_t)field_arrays(MODE) * FLD_PITCH * 4 + ((STG & 1) ? 0 : 128);
    // both stages with the ring exceed the default 48 KB per CTA: opt in once
    // per kernel and device (the attribute belongs to the device's context;
    // the first launch on a device is eager, before any graph capture)
    if (dyn + sizeof(float) * RING * 3 * PLANE > 48 * 1024) {
        static std::atomic<unsigned long long> opted{0};
        int dev = 0;
        GMGS_CUDA(cudaGetDevice(&dev));
        const unsigned long long bit = 1ull << (dev & 63);
        if (!(opted.load() & bit)) {
            GMGS_CUDA(cudaFuncSetAttribute(k_fine<MODE, DEF, STG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)dyn));
            opted.fetch_or(bit);
        }
    }
    k_fine<MODE, DEF, STG><<<grid, dim3(TY, TX, 1), dyn, c.stream>>>(L, cf, a, zc, em);
}

template <int MODE>
void launch_fine(Ctx& c, const FineLevel& L, const Coef32& cf, const FineArgs& a) {
    // the CG update with its staged operands: longer z-chunks (2 instead of 3
    // in the wave count: 1.820 -> 1.792 ms, 1 gave 1.820 ms; the other modes
    // were slower with 2)
    const int zc = pick_zc(L.g, c, MODE == FM_CG_UPDATE_JACOBI ? 2 : 3);
    dim3 grid((L.g.ny + 1 + TY - 1) / TY, (L.g.nx + 1 + TX - 1) / TX, (L.g.nz + 1 + zc - 1) / zc);
    const bool def = coef_is_default(cf);
    EpiMaps em;
    std::memset(&em, 0, sizeof(em));
    const float* fld[FIELD_ARRAYS] = {nullptr, nullptr, nullptr};
    if (MODE == FM_PLAIN) fld[0] = a.v;
    if (MODE == FM_VCYCLE_DOWN) { fld[0] = a.r32; fld[1] = a.wdinv; }
    if (MODE == FM_CG_UPDATE_JACOBI) { fld[0] = a.r32; fld[1] = a.wdinv; fld[2] = a.q32; }
    if (MODE == FM_CG_DIRECTION) { fld[0] = a.z32; fld[1] = a.pold; }
    bool ftma = env_on("GMGS_FIELD_TMA");
    for (int j = 0; j < field_arrays(MODE) && ftma; ++j) ftma = encode_plane_map(&em.f[j], L.g, fld[j], true);
    bool etma = false;
    if (MODE == FM_CG_UPDATE_JACOBI) {
        const float* arr[EPI_ARRAYS] = {a.r32, a.r_lo, a.x_hi, a.x_lo, a.q32, a.pold};
        etma = env_on("GMGS_EPI_TMA");
        for (int j = 0; j < EPI_ARRAYS && etma; ++j) etma = encode_plane_map(&em.m[j], L.g, arr[j], false);
    }
    // the per-node operand stage exists for the CG update only
    const int stg = (etma ? 1 : 0) | (ftma ? 2 : 0);
    auto go = [&](auto tag) {
        constexpr int G = decltype(tag)::value;
        if (def) launch_stg<MODE, true, G>(c, grid, L, cf, a, zc, em);
        else launch_stg<MODE, false, G>(c, grid, L, cf, a, zc, em);
    };
    if constexpr (MODE == FM_CG_UPDATE_JACOBI) {
        if (stg == 3) go(std::integral_constant<int, 3>{});
        else if (stg == 1) go(std::integral_constant<int, 1>{});
        else if (stg == 2) go(std::integral_constant<int, 2>{});
        else go(std::integral_constant<int, 0>{});
    } else {
        if (ftma) go(std::integral_constant<int, 2>{});
        else go(std::integral_constant<int, 0>{});
    }
    GMGS_LAUNCHED(c);
}
template void launch_fine<FM_PLAIN>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine<FM_VCYCLE_DOWN>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine<FM_CG_UPDATE_JACOBI>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine<FM_CG_DIRECTION>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);

// ---------------------------------------------------------------------------
// V-cycle up-sweep in FP32 with omega D^-1 precomputed (Vcycle.m:29-32):
// x_f = (w r + P x_c) + w r', optionally the finest-level fixed DOFs zeroed
// and the CG dot r . x_f accumulated (CG_solver.m:26).
// ---------------------------------------------------------------------------
// 32 x 8 node tiles, one thread per (iy, ix) column walking a chunk of z
// planes; tiles without a solid node (k_tile_occ) are skipped.  The kernel is
// bound by memory latency, so each thread keeps two fine planes in flight:
// the flags, omega/diag, r and r' of plane z + 1 are loaded before plane z is
// computed, and only solid nodes are written.  The four coarse values of a
// coarse plane (Iy + {0,1}, Ix + {0,1}) stay in registers for the two fine
// planes that use them (in-bounds: the halo covers Iy + 1, Ix + 1, Iz + 1).
// z = w r + P z_c + w r' (Vcycle.m:27-32 with the stale residual r'), each
// rounding explicit so that every kernel forming it gives the same bits
__device__ __forceinline__ float up_post(float w, float r, float rp, float wp, float t) {
    return __fadd_rn(fmaf(w, r, __fmul_rn(wp, t)), __fmul_rn(w, rp));
}

template <bool DOT>
__global__ void __launch_bounds__(256, 4) k_up32(Grid gf, Grid gc, const uint8_t* __restrict__ nflag,
                                              const uint8_t* __restrict__ tile_occ, int zc,
                                              const float* __restrict__ wdinv, const float* __restrict__ r,
                                              const float* __restrict__ rp, const float* __restrict__ xc,
                                              float* __restrict__ xf, int zero_fixed, DotOut dout) {
    __shared__ double sh[32];
    const int Sf = (int)gf.slots, Sc = (int)gc.slots;
    const int csx = gc.py, csz = gc.py * gc.px, fsz = gf.py * gf.px;
    const int iy = blockIdx.x * TY + threadIdx.x, ix = blockIdx.y * TX + threadIdx.y;
    const int zb = blockIdx.z * zc, ze = min(zb + zc, gf.nz + 1);
    Kahan dot;
    if (iy <= gf.ny && ix <= gf.nx) {
        const int Iy = iy >> 1, Ix = ix >> 1;
        const int oy = iy & 1, ox = ix & 1;
        const float wyx = (oy ? 0.5f : 1.f) * (ox ? 0.5f : 1.f);
        const int fcol = (int)gf.slot(iy, ix, 0), ccol = (int)gc.slot(Iy, Ix, 0);
        const int64_t trow = (int64_t)gridDim.y * gridDim.x, tcol = (int64_t)blockIdx.y * gridDim.x + blockIdx.x;
        auto occ = [&](int z) { return !tile_occ || tile_occ[z * trow + tcol] != 0; };
        float qa[3][4], qb[3][4];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int k = 0; k < 4; ++k) qa[c][k] = qb[c][k] = 0.f;
        int qa_z = -1;
        auto load_q = [&](int Z, float (&q)[3][4]) {
            const long long n3c = 3ll * Sc;
            constexpr int U = chk::UP_COARSE;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const int x = c * Sc + ccol + Z * csz;
                q[c][0] = chk::ld(xc, x, n3c, U);
                q[c][1] = chk::ld(xc, x + 1, n3c, U);
                q[c][2] = chk::ld(xc, x + csx, n3c, U);
                q[c][3] = chk::ld(xc, x + csx + 1, n3c, U);
            }
        };
        uint8_t flc = 0, fln = 0;
        float wdc[3] = {}, rc[3] = {}, rpc[3] = {}, wdn[3] = {}, rn[3] = {}, rpn[3] = {};
        auto fetch = [&](int z, uint8_t& fl, float (&wd)[3], float (&rr)[3], float (&rq)[3]) {
            const int fs = fcol + z * fsz;
            const long long n3f = 3ll * Sf;
            constexpr int U = chk::UP_FINE;
            fl = chk::ld(nflag, fs, Sf, U);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                wd[c] = chk::ld(wdinv, fs + c * Sf, n3f, U);
                rr[c] = chk::ld(r, fs + c * Sf, n3f, U);
                rq[c] = chk::ld(rp, fs + c * Sf, n3f, U);
            }
        };
        bool okc = zb < ze && occ(zb);
        if (okc) fetch(zb, flc, wdc, rc, rpc);
        for (int iz = zb; iz < ze; ++iz) {
            const bool okn = iz + 1 < ze && occ(iz + 1);
            if (okn) fetch(iz + 1, fln, wdn, rn, rpn);
            if (okc) {
                const int Iz = iz >> 1, oz = iz & 1;
                if (qa_z != Iz) { load_q(Iz, qa); qa_z = Iz; }
                if (oz) load_q(Iz + 1, qb);
                const float w = wyx * (oz ? 0.5f : 1.f);
                if (flc & NF_SOLID) {
                    const int fs = fcol + iz * fsz;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        // the trilinear sum in a fixed order; absent terms add an exact zero
                        float t = qa[c][0];
                        t += oy ? qa[c][1] : 0.f;
                        t += ox ? qa[c][2] : 0.f;
                        t += (ox & oy) ? qa[c][3] : 0.f;
                        t += oz ? qb[c][0] : 0.f;
                        t += (oz & oy) ? qb[c][1] : 0.f;
                        t += (oz & ox) ? qb[c][2] : 0.f;
                        t += (oz & ox & oy) ? qb[c][3] : 0.f;
                        float out = up_post(wdc[c], rc[c], rpc[c], w, t);
                        if (zero_fixed && (flc & (NF_FIX_X << c))) out = 0.f;
                        chk::st(xf, fs + c * Sf, 3ll * Sf, chk::UP_OUT, out);
                        if (DOT) dot.add(__fmul_rn(rc[c], out));
                    }
                }
                if (oz) {
#pragma unroll
                    for (int c = 0; c < 3; ++c)
#pragma unroll
                        for (int k = 0; k < 4; ++k) qa[c][k] = qb[c][k];
                    qa_z = Iz + 1;
                }
            }
            flc = fln;
#pragma unroll
            for (int c = 0; c < 3; ++c) { wdc[c] = wdn[c]; rc[c] = rn[c]; rpc[c] = rpn[c]; }
            okc = okn;
        }
    }
    if (DOT) grid_dot_finish(dot.value(), dout, sh);
}

static int up32_zc(const Grid& g, const Ctx& c) {
    const int64_t cols = (int64_t)((g.ny + 1 + TY - 1) / TY) * ((g.nx + 1 + TX - 1) / TX);
    const int64_t want = (int64_t)c.num_sms * 4 * 8;      // ~8 waves of 4 resident CTAs per SM
    return (int)std::min<int64_t>(64, std::max<int64_t>(2, (cols * (g.nz + 1) + want - 1) / want));
}

void launch_up32(Ctx& c, const Grid& gf, const Grid& gc, const uint8_t* nflag, const uint8_t* tile_occ,
                 const float* wdinv, const float* r, const float* rp, const float* xc, float* xf, bool zero_fixed,
                 const DotOut* dot) {
    const int zc = up32_zc(gf, c);
    const dim3 grid((gf.ny + 1 + TY - 1) / TY, (gf.nx + 1 + TX - 1) / TX, (gf.nz + 1 + zc - 1) / zc);
    const dim3 blk(TY, TX, 1);
    if (dot) {
        k_up32<true><<<grid, blk, 0, c.stream>>>(gf, gc, nflag, tile_occ, zc, wdinv, r, rp, xc, xf, zero_fixed, *dot);
    } else {
        k_up32<false><<<grid, blk, 0, c.stream>>>(gf, gc, nflag, tile_occ, zc, wdinv, r, rp, xc, xf, zero_fixed,
                                                   DotOut{});
    }
    GMGS_LAUNCHED(c);
}

// upper bound of the k_up32 grid over the z-chunk choices (zc >= 2)
int up32_grid_blocks(const Grid& g) {
    return ((g.ny + 1 + TY - 1) / TY) * ((g.nx + 1 + TX - 1) / TX) * ((g.nz + 1 + 1) / 2);
}

// (x_hi, x_lo) -= the last, not yet cancelled Jacobi step dx = fl32(fl32(r32 - alpha q) * w),
// then x = x_hi + x_lo in FP64 (exact: the parts' 48 bits fit a double)
__global__ void k_drop_last_dx(int64_t n, double* __restrict__ x, float* __restrict__ xh, float* __restrict__ xl,
                               const float* __restrict__ r32, const float* __restrict__ q,
                               const float* __restrict__ w, const double* __restrict__ scal, int cur, int first) {
    const float alpha = first ? 0.f : (float)(scal[cur] / scal[2]);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float rm = first ? r32[i] : fmaf(-alpha, q[i], r32[i]);
        const float dx = rm * w[i];
        float h = xh[i], l = xl[i];
        if (dx != 0.f) {
            df_add(h, l, -dx);
            xh[i] = h;
            xl[i] = l;
        }
        x[i] = f2d_int(h) + f2d_int(l);
    }
}
void launch_drop_last_dx(Ctx& c, int64_t n, double* x, float* x_hi, float* x_lo, const float* r32, const float* q,
                         const float* w, const double* scal, int cur, int first) {
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)c.num_sms * 16);
    k_drop_last_dx<<<blocks, 256, 0, c.stream>>>(n, x, x_hi, x_lo, r32, q, w, scal, cur, first);
    GMGS_LAUNCHED(c);
}

// (the load vector is zero almost everywhere: zeros, tested on the integer
// pipe, skip the FP64 subtraction)
__global__ void k_df_split(int64_t n, const double* __restrict__ b, float* __restrict__ hi, float* __restrict__ lo) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = b[i];
        float h = 0.f, l = 0.f;
        if ((__double_as_longlong(v) << 1) != 0) {
            h = d2f_int(v);
            l = d2f_int(v - f2d_int(h));
        }
        hi[i] = h;
        lo[i] = l;
    }
}
void launch_df_split(Ctx& c, int64_t n, const double* b, float* hi, float* lo) {
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)c.num_sms * 16);
    k_df_split<<<blocks, 256, 0, c.stream>>>(n, b, hi, lo);
    GMGS_LAUNCHED(c);
}

// ---------------------------------------------------------------------------
// V-cycle down-sweep at nodes that touch elements with their own Galerkin
// matrix: eight lanes per node (four nodes per warp).  For each of the
// node's 8 elements, lane j multiplies the node's three rows of the element
// matrix at columns 3j..3j+2 (the coupling to element node j) with node j's
// Jacobi step w r; each lane keeps the three row sums across the elements and
// a shuffle reduction over the 8 lanes (xor 1, 2, 4) adds them up.  The
// per-lane sums and the reduction order are those of a lane per (row,
// column group), so the result does not depend on the lane layout.
// out = r - A (w r) with fixed rows zeroed (AtX.m:57).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_perel_vdown(FineLevel L, const __grid_constant__ Coef32 cf,
                                                     const int32_t* __restrict__ nodes, int count,
                                                     const float* __restrict__ r, const float* __restrict__ w,
                                                     float* __restrict__ out) {
    const int gl = blockIdx.x * blockDim.x + threadIdx.x;
    const int node = gl >> 3, j = gl & 7;
    const bool active = node < count;          // whole 8-lane groups; idle groups still shuffle
    const Grid& g = L.g;
    const int S = (int)g.slots, sx = g.py, sz = g.py * g.px;
    const int n = active ? chk::ld(nodes, node, count, chk::PEREL_NODE) : 0;
    const long long n3 = 3ll * S;
    float acc[3] = {0.f, 0.f, 0.f};
    if (active) {
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;
            const int es = n - A - B * sx - C * sz;
            if (!chk::ld(L.emask, es, S, chk::PEREL_ELEM)) continue;   // uniform across the node's lanes
            const int ci = corner_of(A, B, C);
            const int t = L.etype ? chk::ld(L.etype, es, S, chk::PEREL_ELEM) : 0;
            const int nj = es + corner_y(j) + corner_x(j) * sx + corner_z(j) * sz;
            constexpr int V = chk::PEREL_VEC;
            const float d0 = chk::ld(r, nj, n3, V) * chk::ld(w, nj, n3, V);
            const float d1 = chk::ld(r, nj + S, n3, V) * chk::ld(w, nj + S, n3, V);
            const float d2 = chk::ld(r, nj + 2 * S, n3, V) * chk::ld(w, nj + 2 * S, n3, V);
            if (t > 0 && !chk::ok(t - 1, L.nK, chk::PEREL_KS)) continue;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const int off = (3 * ci + a) * 24 + 3 * j;
                if (t > 0) {
                    const float* K = L.Ks + (int64_t)(t - 1) * KE + off;
                    acc[a] = fmaf(K[0], d0, fmaf(K[1], d1, fmaf(K[2], d2, acc[a])));
                } else {
                    const float k = L.kscale;
                    acc[a] = fmaf(k * cf.K[off], d0, fmaf(k * cf.K[off + 1], d1, fmaf(k * cf.K[off + 2], d2, acc[a])));
                }
            }
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], 1);
        acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], 2);
        acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], 4);
    }
    if (active && j < 3) {
        const uint32_t f = chk::ld(L.nflag, n, S, chk::PEREL_ELEM);
        const float y = j == 0 ? acc[0] : (j == 1 ? acc[1] : acc[2]);
        const int i = n + j * S;
        chk::st(out, i, n3, chk::PEREL_OUT, chk::ld(r, i, n3, chk::PEREL_VEC) - ((f & (NF_FIX_X << j)) ? 0.f : y));
    }
}

void launch_perel_vdown(Ctx& c, const FineLevel& L, const Coef32& cf, const int32_t* nodes, int count, const float* r,
                        const float* w, float* out) {
    if (count <= 0) return;
    const int blocks = (int)(((int64_t)count * 8 + 255) / 256);
    k_perel_vdown<<<blocks, 256, 0, c.stream>>>(L, cf, nodes, count, r, w, out);
    GMGS_LAUNCHED(c);
}

// occupancy of the streaming kernel's node tiles: one block per (y tile,
// x tile, z plane), 1 when any of its 32 x 8 nodes is solid.  Real geometry
// leaves most of the padded box empty; CTAs whose whole z-chunk of tiles is
// empty skip all work.
__global__ void k_tile_occ(Grid g, const uint8_t* __restrict__ nflag, uint8_t* __restrict__ occ) {
    const int ty = threadIdx.x & 31, tx = threadIdx.x >> 5;
    const int iy = blockIdx.x * TY + ty, ix = blockIdx.y * TX + tx, iz = blockIdx.z;
    const bool solid = iy <= g.ny && ix <= g.nx && (nflag[g.slot(iy, ix, iz)] & NF_SOLID);
    const int any = __syncthreads_or(solid);
    if (threadIdx.x == 0) occ[((int64_t)iz * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = any ? 1 : 0;
}
size_t tile_occ_bytes(const Grid& g) {
    return (size_t)((g.ny + 1 + TY - 1) / TY) * ((g.nx + 1 + TX - 1) / TX) * (g.nz + 1);
}
void launch_tile_occ(Ctx& c, const Grid& g, const uint8_t* nflag, uint8_t* occ) {
    dim3 grid((g.ny + 1 + TY - 1) / TY, (g.nx + 1 + TX - 1) / TX, g.nz + 1);
    k_tile_occ<<<grid, NT, 0, c.stream>>>(g, nflag, occ);
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

// per-node bit mask of the 8 surrounding solid elements, bit A + 2B + 4C for
// the element whose origin is the node minus (A, B, C)
__global__ void k_emask8(Grid g, const uint8_t* __restrict__ emask, uint8_t* __restrict__ e8) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < g.slots; s += (int64_t)gridDim.x * blockDim.x) {
        int iy, ix, iz;
        g.coords(s, iy, ix, iz);
        uint8_t m = 0;
        if (iy >= 0 && ix >= 0 && iz >= 0 && iy <= g.ny && ix <= g.nx && iz <= g.nz)
            for (int e = 0; e < 8; ++e)
                if (emask[s - (e & 1) - ((e >> 1) & 1) * g.sx() - (e >> 2) * g.sz()]) m |= (uint8_t)(1u << e);
        e8[s] = m;
    }
}
void launch_emask8(Ctx& c, const Grid& g, const uint8_t* emask, uint8_t* e8) {
    const int blocks = (int)std::min<int64_t>((g.slots + 255) / 256, (int64_t)c.num_sms * 16);
    k_emask8<<<blocks, 256, 0, c.stream>>>(g, emask, e8);
    GMGS_LAUNCHED(c);
}

// r32 = fl32(b) for the first Jacobi step
__global__ void k_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}
void launch_to_f32(Ctx& c, int64_t n, const double* a, float* b) {
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)c.num_sms * 16);
    k_to_f32<<<blocks, 256, 0, c.stream>>>(n, a, b);
    GMGS_LAUNCHED(c);
}

}  // namespace gmgs
