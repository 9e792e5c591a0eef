// Streaming FP32 operator kernels with four nodes per thread along y and
// paired-FP32 (f32x2) arithmetic.
//
// Same operator, fused modes and arithmetic as k_fine (fine.cu), node for
// node: the interior stencil in second-difference form, the boundary rows in
// first-difference form, the same operation order, so every output value is
// bit-identical to k_fine's.  What changes is the work per instruction.
// k_fine spends one scalar shared-memory load per neighbour value and one
// scalar FP32 instruction per operation and node (about 24 warp instructions
// per node on the 153M-DOF model, issue-bound).  Here a thread owns a quad of
// four consecutive y nodes: one 128-bit and one 64-bit shared-memory load
// bring a column of six values (y-1 .. y+4) of one component, which serves
// all four nodes, and the FP32 arithmetic runs on the node pairs (0,1) and
// (2,3) with the f32x2 add / sub / mul / fma instructions of sm_100-class
// GPUs (two FP32 results per instruction, each rounded as the scalar
// operation).
//
// A CTA owns 32 (y) x 16 (x) nodes: 8 quads x 16 rows, 128 threads; a warp
// covers 8 quads x 4 rows.  Each ring slot holds the three component planes
// of one z plane with a row pitch of 36 floats, y = -1 .. 32 at offsets
// 0 .. 33, so a quad's six-value column starts on a 16-byte boundary.  The
// ring, the halo staging, the z-chunking and the empty-tile skip follow
// k_fine.
#include "fine.cuh"

namespace gmgs {
namespace {

constexpr int QY = 8;                     // quads per row (32 nodes)
constexpr int TXQ = 16;                   // rows (x) per CTA
constexpr int NTQ = QY * TXQ;             // 128 threads
constexpr int PQ = 36;                    // row pitch (floats): y = -1 .. 32 at 0 .. 33
constexpr int PLQ = PQ * (TXQ + 2);       // one component plane
constexpr int SLQ = 3 * PLQ;              // one ring slot
constexpr int RINGQ = 4;                  // one barrier per plane (as k_fine)
constexpr int NHQ = 2 * QY;               // halo quads: rows -1 and 16
constexpr int NHP = 2 * (TXQ + 2);        // halo points: y = -1 and 32 of rows -1 .. 16
static_assert(NHQ + NHP <= NTQ, "one halo item per thread");
static_assert(PQ % 4 == 0, "16-byte aligned columns");

// two FP32 values in one 64-bit register pair, operands of the f32x2 instructions
typedef unsigned long long f2;
__device__ __forceinline__ f2 pk(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk(f2 v, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v)); }
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// the six values y-1 .. y+4 of one component column; i = ring offset of y-1
__device__ __forceinline__ void column(const float* __restrict__ P, int i, float v[6]) {
    constexpr long long R = SLQ;
    const float4 a = chk::ld4(P, i, R, chk::FINE_RING);
    const float2 b = chk::ld2(P, i + 4, R, chk::FINE_RING);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y;
}

// node pair p (nodes 2p, 2p+1 of the quad) at y offset o of a column
__device__ __forceinline__ f2 at(const float v[6], int p, int o) { return pk(v[2 * p + 1 + o], v[2 * p + 2 + o]); }

// interior stencil, second-difference form (as interior_s), for the four
// nodes of a quad: acc[a][p] = (y_a of node 2p, y_a of node 2p+1)
__device__ __forceinline__ void interior_q(const f2* __restrict__ sp, const float* __restrict__ P0,
                                           const float* __restrict__ P1, const float* __restrict__ P2, int ib,
                                           f2 acc[3][2]) {
    f2 cE[3][2];
    // k = 14: (dy, dx, dz) = (+1, 0, 0), up = y + 1 and down = y - 1 of the centre column
    {
        f2 d[3][2];
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            float v[6];
            column(P1 + b * PLQ, ib, v);
            cE[b][0] = at(v, 0, 0);
            cE[b][1] = at(v, 1, 0);
#pragma unroll
            for (int p = 0; p < 2; ++p) d[b][p] = add2(sub2(at(v, p, 1), cE[b][p]), sub2(at(v, p, -1), cE[b][p]));
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
#pragma unroll
            for (int p = 0; p < 2; ++p) acc[a][p] = 0ull;
#pragma unroll
            for (int b = 0; b < 3; ++b)
                if (s_nonzero(14, a, b)) {
                    const f2 s = sp[3 * a + b];
#pragma unroll
                    for (int p = 0; p < 2; ++p) acc[a][p] = fma2(s, d[b][p], acc[a][p]);
                }
        }
    }
    // the other 12 half offsets in four column groups (dx, dz), dy = -1, 0, +1:
    // k = (dz+1)*9 + (dx+1)*3 + (dy+1); up column (x+dx, z+dz), down column (x-dx, z-dz)
#pragma unroll
    for (int gi = 0; gi < 4; ++gi) {
        const int DX = gi == 0 ? 1 : (gi == 1 ? -1 : (gi == 2 ? 0 : 1));
        const int DZ = gi == 0 ? 0 : 1;
        const int KB = (DZ + 1) * 9 + (DX + 1) * 3;       // k of dy = -1
        const float* Pu = DZ > 0 ? P2 : P1;
        const float* Pd = DZ > 0 ? P0 : P1;
        f2 d[3][3][2];                                     // [dy + 1][b][pair]
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            float u[6], w[6];
            column(Pu + b * PLQ, ib + DX * PQ, u);
            column(Pd + b * PLQ, ib - DX * PQ, w);
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                for (int p = 0; p < 2; ++p)
                    d[dy + 1][b][p] = add2(sub2(at(u, p, dy), cE[b][p]), sub2(at(w, p, -dy), cE[b][p]));
        }
#pragma unroll
        for (int dy = 0; dy < 3; ++dy) {
            const int k = KB + dy;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b)
                    if (s_nonzero(k, a, b)) {
                        const f2 s = sp[(k - 14) * 9 + 3 * a + b];
#pragma unroll
                        for (int p = 0; p < 2; ++p) acc[a][p] = fma2(s, d[dy][b][p], acc[a][p]);
                    }
        }
    }
}

// the field (3 components) of a quad from the kernel's inputs, as field_at per node
template <int MODE>
__device__ __forceinline__ void field_q(const FineArgs& a, int S, int s, float beta, float alpha, float4 v[3]) {
    const long long n3 = 3ll * S;
    constexpr int F = chk::FINE_FIELD;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int i = s + c * S;
        if (MODE == FM_PLAIN) {
            v[c] = chk::ld4(a.v, i, n3, F);
        } else if (MODE == FM_VCYCLE_DOWN) {
            const float4 r = chk::ld4(a.r32, i, n3, F), w = chk::ld4(a.wdinv, i, n3, F);
            v[c] = make_float4(r.x * w.x, r.y * w.y, r.z * w.z, r.w * w.w);
        } else if (MODE == FM_CG_UPDATE_JACOBI) {
            const float4 r = chk::ld4(a.r32, i, n3, F), w = chk::ld4(a.wdinv, i, n3, F);
            float4 rm = r;
            if (!a.first) {
                const float4 q = chk::ld4(a.q32, i, n3, F);
                rm = make_float4(fmaf(-alpha, q.x, r.x), fmaf(-alpha, q.y, r.y), fmaf(-alpha, q.z, r.z),
                                 fmaf(-alpha, q.w, r.w));
            }
            v[c] = make_float4(rm.x * w.x, rm.y * w.y, rm.z * w.z, rm.w * w.w);
        } else {   // FM_CG_DIRECTION
            const float4 z = chk::ld4(a.z32, i, n3, F);
            v[c] = z;
            if (!a.first) {
                const float4 p = chk::ld4(a.pold, i, n3, F);
                v[c] = make_float4(fmaf(beta, p.x, z.x), fmaf(beta, p.y, z.y), fmaf(beta, p.z, z.z),
                                   fmaf(beta, p.w, z.w));
            }
        }
    }
}

__device__ __forceinline__ float comp4(const float4& v, int j) { return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w)); }

}  // namespace

// One CTA per 32 x 16 node column tile and z-chunk; modes as k_fine.
template <int MODE, int MINB>
__global__ void __launch_bounds__(NTQ, MINB) k_fine4(FineLevel L, const __grid_constant__ Coef32 cf, FineArgs a, int zc) {
    __shared__ __align__(16) float ring[RINGQ][SLQ];
    __shared__ __align__(16) f2 sp[13 * 9];    // (S, S) pairs of the half-offset blocks, k = 14 .. 26
    __shared__ double sh[32];
    const Grid& g = L.g;
    const int S = (int)g.slots;
    const int sz = g.py * g.px;
    const int tid = threadIdx.x;
    const int y0 = blockIdx.x * (4 * QY), x0 = blockIdx.y * TXQ;
    const int zb = blockIdx.z * zc;
    const int ze = min(zb + zc, g.nz + 1);        // node planes [zb, ze)
    if (L.tile_occ) {                             // the 8-wide column tiles of k_fine under this one
        const int ntx8 = (g.nx + 1 + 7) / 8;
        const int tx = 2 * blockIdx.y;
        int any = 0;
        for (int iz = zb; iz < ze; ++iz) {
            const int64_t row = (int64_t)iz * ntx8;
            any |= L.tile_occ[(row + tx) * gridDim.x + blockIdx.x];
            if (tx + 1 < ntx8) any |= L.tile_occ[(row + tx + 1) * gridDim.x + blockIdx.x];
        }
        if (!any) {
            if (MODE == FM_CG_DIRECTION || MODE == FM_CG_UPDATE_JACOBI) grid_dot_finish(0.0, a.dot, sh);
            return;
        }
    }
    if (tid < 13 * 9) {
        const float s = cf.S[14 * 9 + tid];
        sp[tid] = pk(s, s);
    }

    float beta = 0.f, alpha = 0.f;
    if (MODE == FM_CG_DIRECTION && !a.first) beta = (float)(a.scal[a.cur] / a.scal[a.cur ^ 1]);
    if (MODE == FM_CG_UPDATE_JACOBI && !a.first) alpha = (float)(a.scal[a.cur] / a.scal[2]);

    // this thread's quad: nodes (cy + j, cx), j = 0..3; ring offset ib of its column's y - 1
    const int q = tid & (QY - 1), r = tid / QY;
    const int cy = y0 + 4 * q, cx = x0 + r;
    const int ib = 4 * q + (r + 1) * PQ;
    // A quad starting at y <= ny + 1 lies inside its slot row (the row holds y up
    // to ny + 4); the values it stages beyond ny + 1 feed no owned node.
    const bool cload = cy <= g.ny + 1 && cx <= g.nx + 1;
    const int cbase = (cx + 1) * g.py + (cy + Grid::YOFF) + sz;   // slot(cy, cx, iz) = cbase + iz * sz
    // one halo item: tid < 16 a quad of row -1 or 16, 16 <= tid < 52 a point at y = -1 or 32
    int hoff = 0, hbase = 0;
    bool hload = false;
    if (tid < NHQ) {
        const int hr = tid < QY ? -1 : TXQ, hq = tid & (QY - 1);
        const int hy = y0 + 4 * hq, hx = x0 + hr;
        hload = hy <= g.ny + 1 && hx <= g.nx + 1;
        hoff = (4 * hq + 1) + (hr + 1) * PQ;
        hbase = (hx + 1) * g.py + (hy + Grid::YOFF) + sz;
    } else if (tid < NHQ + NHP) {
        const int k = tid - NHQ;
        const int hr = (k >> 1) - 1, hyl = (k & 1) ? 4 * QY : -1;
        const int hy = y0 + hyl, hx = x0 + hr;
        hload = hy <= g.ny + 1 && hx <= g.nx + 1;
        hoff = (hyl + 1) + (hr + 1) * PQ;
        hbase = (hx + 1) * g.py + (hy + Grid::YOFF) + sz;
    }
    auto fetch = [&](int iz, float4 vc[3], float4 vh[3]) {
#pragma unroll
        for (int c = 0; c < 3; ++c) vc[c] = vh[c] = make_float4(0.f, 0.f, 0.f, 0.f);
        const bool zok = iz >= -1 && iz <= g.nz + 1;
        if (zok && cload) field_q<MODE>(a, S, cbase + iz * sz, beta, alpha, vc);
        if (zok && hload) {
            if (tid < NHQ) {
                field_q<MODE>(a, S, hbase + iz * sz, beta, alpha, vh);
            } else {
                float v[3];
                field_at<MODE>(a, S, hbase + iz * sz, beta, alpha, v);
#pragma unroll
                for (int c = 0; c < 3; ++c) vh[c].x = v[c];
            }
        }
    };
    auto store = [&](float* R, const float4 vc[3], const float4 vh[3]) {
        constexpr long long RS = SLQ;
        constexpr int RG = chk::FINE_RING;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float* P = R + c * PLQ;
            chk::st(P, ib + 1, RS, RG, vc[c].x);
            chk::st2(P, ib + 2, RS, RG, make_float2(vc[c].y, vc[c].z));
            chk::st(P, ib + 4, RS, RG, vc[c].w);
            if (tid < NHQ) {
                chk::st(P, hoff, RS, RG, vh[c].x);
                chk::st2(P, hoff + 1, RS, RG, make_float2(vh[c].y, vh[c].z));
                chk::st(P, hoff + 3, RS, RG, vh[c].w);
            } else if (tid < NHQ + NHP) {
                chk::st(P, hoff, RS, RG, vh[c].x);
            }
        }
    };

    float4 vc[3], vh[3];
    fetch(zb - 1, vc, vh);
    store(ring[(zb - 1 + RINGQ) % RINGQ], vc, vh);
    fetch(zb, vc, vh);
    store(ring[zb % RINGQ], vc, vh);
    fetch(zb + 1, vc, vh);

    const bool own = cy <= g.ny && cx <= g.nx;
    uint32_t f_next = 0, e8_next = 0;
    if (own) {
        f_next = chk::ld_u8x4(L.nflag, cbase + zb * sz, g.slots, chk::FINE_FLAGS);
        e8_next = chk::ld_u8x4(L.emask8, cbase + zb * sz, g.slots, chk::FINE_FLAGS);
    }
    const long long n3 = 3ll * S;
    constexpr int O = chk::FINE_OUT;
    Kahan dot;
#pragma unroll 1
    for (int iz = zb; iz < ze; ++iz) {
        store(ring[(iz + 1) % RINGQ], vc, vh);
        __syncthreads();
        if (iz + 2 <= g.nz + 1) fetch(iz + 2, vc, vh);
        const uint32_t f4 = f_next, e84 = e8_next;
        if (own && iz + 1 < ze) {
            f_next = chk::ld_u8x4(L.nflag, cbase + (iz + 1) * sz, g.slots, chk::FINE_FLAGS);
            e8_next = chk::ld_u8x4(L.emask8, cbase + (iz + 1) * sz, g.slots, chk::FINE_FLAGS);
        }
        // nodes with a result: solid, not on the per-element path, y <= ny
        uint32_t act = 0, intr = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t f = (f4 >> (8 * j)) & 0xFFu;
            if (cy + j <= g.ny && (f & NF_SOLID) && !(f & NF_PEREL)) {
                act |= 1u << j;
                if (f & NF_INTERIOR) intr |= 1u << j;
            }
        }
        if (!act) continue;
        const float* P0 = ring[(iz - 1 + RINGQ) % RINGQ];
        const float* P1 = ring[iz % RINGQ];
        const float* P2 = ring[(iz + 1) % RINGQ];
        const int n0 = cbase + iz * sz;
        float4 er[3];
        if (MODE == FM_VCYCLE_DOWN) {       // in flight during the stencil arithmetic
#pragma unroll
            for (int c = 0; c < 3; ++c) er[c] = chk::ld4(a.r32, n0 + c * S, n3, chk::FINE_EPI);
        }
        float y[4][3];
        if (intr) {
            f2 acc[3][2];
            interior_q(sp, P0, P1, P2, ib, acc);
            const f2 ks = pk(L.kscale, L.kscale);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                upk(mul2(acc[c][0], ks), y[0][c], y[1][c]);
                upk(mul2(acc[c][1], ks), y[2][c], y[3][c]);
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (((act & ~intr) >> j) & 1u)
                boundary_s<PQ, PLQ>(L, cf, (e84 >> (8 * j)) & 0xFFu, n0 + j, P0, P1, P2, ib + 1 + j, y[j][0], y[j][1],
                                    y[j][2]);
            const uint32_t f = (f4 >> (8 * j)) & 0xFFu;
            if (f & NF_FIX_X) y[j][0] = 0.f;
            if (f & NF_FIX_Y) y[j][1] = 0.f;
            if (f & NF_FIX_Z) y[j][2] = 0.f;
        }
        // centre values (the staged field) for the modes that write or use it
        float4 vn[3];
        if (MODE == FM_CG_DIRECTION) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float v[6];
                column(P1 + c * PLQ, ib, v);
                vn[c] = make_float4(v[1], v[2], v[3], v[4]);
            }
        }
        if (act == 0xFu) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const int i = n0 + c * S;
                if (MODE == FM_PLAIN) {
                    chk::st4(a.out32, i, n3, O, make_float4(y[0][c], y[1][c], y[2][c], y[3][c]));
                } else if (MODE == FM_VCYCLE_DOWN) {
                    chk::st4(a.out32, i, n3, O,
                             make_float4(er[c].x - y[0][c], er[c].y - y[1][c], er[c].z - y[2][c], er[c].w - y[3][c]));
                } else if (MODE == FM_CG_DIRECTION) {
                    chk::st4(a.pout, i, n3, O, vn[c]);
                    chk::st4(a.out32, i, n3, O, make_float4(y[0][c], y[1][c], y[2][c], y[3][c]));
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (!((act >> j) & 1u)) continue;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const int i = n0 + j + c * S;
                    if (MODE == FM_PLAIN) {
                        chk::st(a.out32, i, n3, O, y[j][c]);
                    } else if (MODE == FM_VCYCLE_DOWN) {
                        chk::st(a.out32, i, n3, O, comp4(er[c], j) - y[j][c]);
                    } else if (MODE == FM_CG_DIRECTION) {
                        chk::st(a.pout, i, n3, O, comp4(vn[c], j));
                        chk::st(a.out32, i, n3, O, y[j][c]);
                    }
                }
            }
        }
        if (MODE == FM_CG_DIRECTION) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if ((act >> j) & 1u)
#pragma unroll
                    for (int c = 0; c < 3; ++c) dot.add(comp4(vn[c], j) * y[j][c]);
        }
    }
    if (MODE == FM_CG_DIRECTION || MODE == FM_CG_UPDATE_JACOBI) grid_dot_finish(dot.value(), a.dot, sh);
}

static int pick_zc4(const Grid& g, const Ctx& c) {
    const int64_t cols = (int64_t)((g.ny + 1 + 4 * QY - 1) / (4 * QY)) * ((g.nx + 1 + TXQ - 1) / TXQ);
    // about 16 waves of 4 resident CTAs per SM
    const int64_t want = (int64_t)c.num_sms * 4 * 16;
    int64_t zc = (cols * (g.nz + 1) + want - 1) / want;
    if (zc < 4) zc = 4;
    if (zc > 64) zc = 64;
    return (int)zc;
}

template <int MODE>
void launch_fine4(Ctx& c, const FineLevel& L, const Coef32& cf, const FineArgs& a) {
    static_assert(MODE != FM_CG_UPDATE_JACOBI, "the CG update runs on k_fine");
    const int zc = pick_zc4(L.g, c);
    dim3 grid((L.g.ny + 1 + 4 * QY - 1) / (4 * QY), (L.g.nx + 1 + TXQ - 1) / TXQ, (L.g.nz + 1 + zc - 1) / zc);
    const char* e = std::getenv("GMGS_QUAD");
    if (e && e[0] == '3') k_fine4<MODE, 3><<<grid, NTQ, 0, c.stream>>>(L, cf, a, zc);
    else k_fine4<MODE, 4><<<grid, NTQ, 0, c.stream>>>(L, cf, a, zc);
    GMGS_LAUNCHED(c);
}
template void launch_fine4<FM_PLAIN>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine4<FM_VCYCLE_DOWN>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine4<FM_CG_DIRECTION>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);

}  // namespace gmgs
