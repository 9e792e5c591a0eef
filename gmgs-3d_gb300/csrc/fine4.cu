// Finest-level streaming kernels with four y-adjacent nodes per thread.
//
// Same operator, modes and pipeline as k_fine (fine.cu), but each thread owns
// a quad of 4 consecutive y-nodes in one x column.  A stencil row (dx, dz) of
// the quad is then one 16-byte shared-memory load plus its two neighbours in
// y, instead of 12 scalar loads, and the index arithmetic is shared by four
// nodes.  A CTA of 256 threads covers 32 (y) x 32 (x) nodes; each warp covers
// 32 (y) x 4 (x).  The shared ring holds three planes of (32+2) x (32+2)
// points per component, rows padded to 40 floats so the quads are aligned.
#include "fine.cuh"

namespace gmgs {
namespace {

constexpr int QY = 8;                 // quads per column (32 y-nodes)
constexpr int TXC = 32;               // x columns per CTA
constexpr int NTH = QY * TXC;         // 256 threads
constexpr int RPQ = 40;               // row pitch: [3] = y0-1, [4..35] = y0..y0+31, [36] = y0+32
constexpr int HXQ = TXC + 2;          // rows x0-1 .. x0+32
constexpr int PLQ = RPQ * HXQ;        // floats per component plane
constexpr int RING = 3 * 3 * PLQ;     // three planes, three components
constexpr size_t SMEM = RING * sizeof(float) + 32 * sizeof(double);

struct Row {
    float m, q0, q1, q2, q3, p;       // values at quad-relative y = -1 .. 4
    __device__ __forceinline__ float at(int i) const {
        return i == -1 ? m : i == 0 ? q0 : i == 1 ? q1 : i == 2 ? q2 : i == 3 ? q3 : p;
    }
};

__device__ __forceinline__ Row load_row(const float* __restrict__ P, int off) {
    Row r;
    const float4 q = *reinterpret_cast<const float4*>(P + off);
    r.m = P[off - 1];
    r.q0 = q.x; r.q1 = q.y; r.q2 = q.z; r.q3 = q.w;
    r.p = P[off + 4];
    return r;
}

// one row pair (dx, dz) / (-dx, -dz) of the second-difference stencil for the
// quad; DY0..DY1 are the y offsets of the half-stencil served by this pair
template <int DX, int DZ, int DY0, int DY1>
__device__ __forceinline__ void quad_pair(const Coef32& cf, const float* __restrict__ P0,
                                          const float* __restrict__ P1, const float* __restrict__ P2, int pq,
                                          const float c[3][4], float acc[3][4]) {
    const float* up = DZ > 0 ? P2 : P1;
    const float* dn = DZ > 0 ? P0 : P1;
    // one input component at a time keeps only two rows live
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        const Row ru = load_row(up + b * PLQ, pq + DX * RPQ);
        const Row rd = load_row(dn + b * PLQ, pq - DX * RPQ);
#pragma unroll
        for (int dy = DY0; dy <= DY1; ++dy) {
            constexpr int kbase = (DZ + 1) * 9 + (DX + 1) * 3 + 1;
            const int k = kbase + dy;
            float d[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) d[i] = (ru.at(i + dy) - c[b][i]) + (rd.at(i - dy) - c[b][i]);
#pragma unroll
            for (int a = 0; a < 3; ++a)
                if (s_nonzero(k, a, b)) {
                    const float s = cf.S[k * 9 + 3 * a + b];
#pragma unroll
                    for (int i = 0; i < 4; ++i) acc[a][i] = fmaf(s, d[i], acc[a][i]);
                }
        }
    }
}

// the 13 half offsets k = 14..26, grouped by the row pair they read
__device__ __forceinline__ void quad_interior(const Coef32& cf, const float* __restrict__ P0,
                                              const float* __restrict__ P1, const float* __restrict__ P2, int pq,
                                              float acc[3][4]) {
    float c[3][4];
    Row rc[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        rc[b] = load_row(P1 + b * PLQ, pq);
        c[b][0] = rc[b].q0; c[b][1] = rc[b].q1; c[b][2] = rc[b].q2; c[b][3] = rc[b].q3;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int i = 0; i < 4; ++i) acc[a][i] = 0.f;
    // k = 14: (dy, dx, dz) = (+1, 0, 0), both ends on the centre row
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        float d[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) d[i] = (rc[b].at(i + 1) - c[b][i]) + (rc[b].at(i - 1) - c[b][i]);
#pragma unroll
        for (int a = 0; a < 3; ++a)
            if (s_nonzero(14, a, b)) {
                const float s = cf.S[14 * 9 + 3 * a + b];
#pragma unroll
                for (int i = 0; i < 4; ++i) acc[a][i] = fmaf(s, d[i], acc[a][i]);
            }
    }
    quad_pair<1, 0, -1, 1>(cf, P0, P1, P2, pq, c, acc);    // k = 15..17
    quad_pair<-1, 1, -1, 1>(cf, P0, P1, P2, pq, c, acc);   // k = 18..20
    quad_pair<0, 1, -1, 1>(cf, P0, P1, P2, pq, c, acc);    // k = 21..23
    quad_pair<1, 1, -1, 1>(cf, P0, P1, P2, pq, c, acc);    // k = 24..26
}

// the kernel's input field at a point (3 components) from its inputs
template <int MODE>
__device__ __forceinline__ float field1(const FineArgs& a, int i, float beta, float alpha) {
    if (MODE == FM_PLAIN) return a.v[i];
    if (MODE == FM_VCYCLE_DOWN) return a.r32[i] * a.wdinv[i];
    if (MODE == FM_CG_UPDATE_JACOBI) return (a.first ? a.r32[i] : fmaf(-alpha, a.q32[i], a.r32[i])) * a.wdinv[i];
    return a.first ? a.z32[i] : fmaf(beta, a.pold[i], a.z32[i]);
}

__device__ __forceinline__ float4 ld4(const float* p, int i) { return *reinterpret_cast<const float4*>(p + i); }

template <int MODE>
__device__ __forceinline__ float4 field4(const FineArgs& a, int i, float beta, float alpha) {
    if (MODE == FM_PLAIN) return ld4(a.v, i);
    if (MODE == FM_VCYCLE_DOWN) {
        const float4 r = ld4(a.r32, i), w = ld4(a.wdinv, i);
        return make_float4(r.x * w.x, r.y * w.y, r.z * w.z, r.w * w.w);
    }
    if (MODE == FM_CG_UPDATE_JACOBI) {
        const float4 r = ld4(a.r32, i), w = ld4(a.wdinv, i);
        if (a.first) return make_float4(r.x * w.x, r.y * w.y, r.z * w.z, r.w * w.w);
        const float4 q = ld4(a.q32, i);
        return make_float4(fmaf(-alpha, q.x, r.x) * w.x, fmaf(-alpha, q.y, r.y) * w.y, fmaf(-alpha, q.z, r.z) * w.z,
                           fmaf(-alpha, q.w, r.w) * w.w);
    }
    const float4 z = ld4(a.z32, i);
    if (a.first) return z;
    const float4 p = ld4(a.pold, i);
    return make_float4(fmaf(beta, p.x, z.x), fmaf(beta, p.y, z.y), fmaf(beta, p.z, z.z), fmaf(beta, p.w, z.w));
}

template <int MODE>
__global__ void __launch_bounds__(NTH, 2) k_fine4(FineLevel L, const __grid_constant__ Coef32 cf, FineArgs a, int zc) {
    extern __shared__ __align__(16) float smem[];
    float* ring = smem;
    double* sh = reinterpret_cast<double*>(smem + RING);
    const Grid& g = L.g;
    const int S = (int)g.slots;
    const int sz = g.py * g.px;
    const int y0 = blockIdx.x * (4 * QY), x0 = blockIdx.y * TXC;
    const int zb = blockIdx.z * zc;
    const int ze = min(zb + zc, g.nz + 1);
    const int tid = threadIdx.x;
    const int qy = tid & 7, xc = (tid >> 5) * 4 + ((tid >> 3) & 3);

    float beta = 0.f, alpha = 0.f;
    if (MODE == FM_CG_DIRECTION && !a.first) beta = (float)(a.scal[a.cur] / a.scal[a.cur ^ 1]);
    if (MODE == FM_CG_UPDATE_JACOBI && !a.first) alpha = (float)(a.scal[a.cur] / a.scal[2]);

    // own quad: nodes (y0 + 4 qy + i, x0 + xc), i = 0..3
    const int qy0 = y0 + 4 * qy, cx = x0 + xc;
    const int pq = (4 + 4 * qy) + (xc + 1) * RPQ;
    const bool qload = qy0 <= g.ny + 1 && cx <= g.nx + 1;       // quad inside the halo'd grid (float4-safe)
    const bool own = qy0 <= g.ny && cx <= g.nx;
    const int qbase = (cx + 1) * g.py + qy0 + Grid::YOFF + sz;  // slot(qy0, cx, iz) = qbase + iz * sz
    // halo: tid < 68 one y-halo point, 68 <= tid < 84 one x-halo quad
    int hkind = 0, hring = 0, hbase = 0;
    bool hok = false;
    if (tid < 68) {
        const int side = tid & 1, xr = tid >> 1;                 // xr = 0..33 -> x0-1 .. x0+32
        const int hy = side ? y0 + 4 * QY : y0 - 1, hx = x0 - 1 + xr;
        hkind = 1;
        hring = (side ? 4 + 4 * QY : 3) + xr * RPQ;
        hok = hy >= -1 && hy <= g.ny + 1 && hx >= -1 && hx <= g.nx + 1;
        hbase = (hx + 1) * g.py + hy + Grid::YOFF + sz;
    } else if (tid < 84) {
        const int k = tid - 68, side = k & 1, qq = k >> 1;
        const int hy = y0 + 4 * qq, hx = side ? x0 + TXC : x0 - 1;
        hkind = 2;
        hring = (4 + 4 * qq) + (side ? TXC + 1 : 0) * RPQ;
        hok = hy <= g.ny + 1 && hx >= -1 && hx <= g.nx + 1;
        hbase = (hx + 1) * g.py + hy + Grid::YOFF + sz;
    }

    float4 vq[3];
    float4 vh[3];
    auto fetch = [&](int iz) {
        const bool zok = iz >= -1 && iz <= g.nz + 1;
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            vq[b] = (zok && qload) ? field4<MODE>(a, qbase + iz * sz + b * S, beta, alpha) : make_float4(0, 0, 0, 0);
            if (hkind == 1) {
                vh[b].x = (zok && hok) ? field1<MODE>(a, hbase + iz * sz + b * S, beta, alpha) : 0.f;
            } else if (hkind == 2) {
                vh[b] = (zok && hok) ? field4<MODE>(a, hbase + iz * sz + b * S, beta, alpha) : make_float4(0, 0, 0, 0);
            }
        }
    };
    auto store = [&](float* r) {
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            *reinterpret_cast<float4*>(r + b * PLQ + pq) = vq[b];
            if (hkind == 1) r[b * PLQ + hring] = vh[b].x;
            else if (hkind == 2) *reinterpret_cast<float4*>(r + b * PLQ + hring) = vh[b];
        }
    };

    fetch(zb - 1);
    store(ring + ((zb + 2) % 3) * 3 * PLQ);
    fetch(zb);
    store(ring + (zb % 3) * 3 * PLQ);
    fetch(zb + 1);

    uint32_t f_next = 0, e_next = 0;
    if (own) {
        f_next = *reinterpret_cast<const uint32_t*>(L.nflag + qbase + zb * sz);
        e_next = *reinterpret_cast<const uint32_t*>(L.emask8 + qbase + zb * sz);
    }
    Kahan dot;
#pragma unroll 1
    for (int iz = zb; iz < ze; ++iz) {
        store(ring + ((iz + 1) % 3) * 3 * PLQ);
        __syncthreads();
        if (iz + 2 <= g.nz + 1) fetch(iz + 2);
        const uint32_t f4 = f_next, e4 = e_next;
        if (own && iz + 1 < ze) {
            f_next = *reinterpret_cast<const uint32_t*>(L.nflag + qbase + (iz + 1) * sz);
            e_next = *reinterpret_cast<const uint32_t*>(L.emask8 + qbase + (iz + 1) * sz);
        }
        const float* P0 = ring + ((iz + 2) % 3) * 3 * PLQ;
        const float* P1 = ring + (iz % 3) * 3 * PLQ;
        const float* P2 = ring + ((iz + 1) % 3) * 3 * PLQ;
        if (own && (f4 & 0x01010101u)) {
            const int n0 = qbase + iz * sz;
            // epilogue inputs, in flight during the stencil arithmetic
            float4 er[3], eq[3], ep[3];
            double2 el[3][2];
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                er[b] = eq[b] = ep[b] = make_float4(0.f, 0.f, 0.f, 0.f);
                el[b][0] = el[b][1] = make_double2(0.0, 0.0);
            }
            // the V-cycle residual is in flight during the stencil arithmetic
#pragma unroll
            for (int b = 0; b < 3; ++b)
                if (MODE == FM_VCYCLE_DOWN) er[b] = ld4(a.r32, n0 + b * S);
            float y[3][4];
            const uint32_t allint = (NF_INTERIOR) * 0x01010101u;
            if ((f4 & allint) == allint) {
                quad_interior(cf, P0, P1, P2, pq, y);
#pragma unroll
                for (int c = 0; c < 3; ++c)
#pragma unroll
                    for (int i = 0; i < 4; ++i) y[c][i] *= L.kscale;
            } else {
                // one node at a time (kept rolled: the boundary path is long)
#pragma unroll 1
                for (int i = 0; i < 4; ++i) {
                    const uint32_t fi = (f4 >> (8 * i)) & 0xffu;
                    y[0][i] = y[1][i] = y[2][i] = 0.f;
                    if (!(fi & NF_SOLID) || qy0 + i > g.ny) continue;
                    if (fi & NF_INTERIOR) {
                        interior_s<RPQ, PLQ>(cf, P0, P1, P2, pq + i, y[0][i], y[1][i], y[2][i]);
                        y[0][i] *= L.kscale; y[1][i] *= L.kscale; y[2][i] *= L.kscale;
                    } else {
                        boundary_s<RPQ, PLQ>(L, cf, (e4 >> (8 * i)) & 0xffu, n0 + i, P0, P1, P2, pq + i, y[0][i],
                                             y[1][i], y[2][i]);
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const uint32_t fi = (f4 >> (8 * i)) & 0xffu;
                if (fi & NF_FIX_X) y[0][i] = 0.f;
                if (fi & NF_FIX_Y) y[1][i] = 0.f;
                if (fi & NF_FIX_Z) y[2][i] = 0.f;
            }
            if (MODE == FM_CG_UPDATE_JACOBI) {
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    const int i = n0 + b * S;
                    er[b] = ld4(a.r32, i);
                    el[b][0] = *reinterpret_cast<const double2*>(a.r64 + i);
                    el[b][1] = *reinterpret_cast<const double2*>(a.r64 + i + 2);
                    if (!a.first) {
                        eq[b] = ld4(a.q32, i);
                        ep[b] = ld4(a.pold, i);
                    }
                }
            }
            // epilogue on the 4 nodes at once; non-solid nodes and halo slots
            // carry zeros in every input, so their outputs stay zero
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const int i = n0 + b * S;
                const float4 v = *reinterpret_cast<const float4*>(P1 + b * PLQ + pq);
                const float yv[4] = {y[b][0], y[b][1], y[b][2], y[b][3]};
                const float vv[4] = {v.x, v.y, v.z, v.w};
                if (MODE == FM_PLAIN) {
                    *reinterpret_cast<float4*>(a.out32 + i) = make_float4(yv[0], yv[1], yv[2], yv[3]);
                } else if (MODE == FM_VCYCLE_DOWN) {
                    *reinterpret_cast<float4*>(a.out32 + i) =
                        make_float4(er[b].x - yv[0], er[b].y - yv[1], er[b].z - yv[2], er[b].w - yv[3]);
                } else if (MODE == FM_CG_UPDATE_JACOBI) {
                    // previous iteration's update x += alpha p, r -= alpha q (CG_solver.m:32-33),
                    // then the Jacobi step x += dx, r -= A dx (CG_solver.m:18-19)
                    const float rr[4] = {er[b].x, er[b].y, er[b].z, er[b].w};
                    const float qq[4] = {eq[b].x, eq[b].y, eq[b].z, eq[b].w};
                    const float pp[4] = {ep[b].x, ep[b].y, ep[b].z, ep[b].w};
                    const double r64[4] = {el[b][0].x, el[b][0].y, el[b][1].x, el[b][1].y};
                    double xo[4], rn[4];
                    float r32n[4];
                    const double2 x01 = *reinterpret_cast<const double2*>(a.x64 + i);
                    const double2 x23 = *reinterpret_cast<const double2*>(a.x64 + i + 2);
                    const double xi[4] = {x01.x, x01.y, x23.x, x23.y};
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        float rinc = yv[j], rm32 = rr[j], xinc = vv[j];
                        if (!a.first) {
                            xinc = fmaf(alpha, pp[j], vv[j]);
                            rinc = fmaf(alpha, qq[j], rinc);
                            rm32 = fmaf(-alpha, qq[j], rm32);
                        }
                        xo[j] = xi[j] + (double)xinc;
                        rn[j] = r64[j] - (double)rinc;
                        r32n[j] = (float)rn[j];
                        dot.add(rm32 * rm32);
                    }
                    *reinterpret_cast<double2*>(a.x64 + i) = make_double2(xo[0], xo[1]);
                    *reinterpret_cast<double2*>(a.x64 + i + 2) = make_double2(xo[2], xo[3]);
                    *reinterpret_cast<double2*>(a.r64 + i) = make_double2(rn[0], rn[1]);
                    *reinterpret_cast<double2*>(a.r64 + i + 2) = make_double2(rn[2], rn[3]);
                    *reinterpret_cast<float4*>(a.r32out + i) = make_float4(r32n[0], r32n[1], r32n[2], r32n[3]);
                } else {
                    *reinterpret_cast<float4*>(a.pout + i) = v;
                    *reinterpret_cast<float4*>(a.out32 + i) = make_float4(yv[0], yv[1], yv[2], yv[3]);
#pragma unroll
                    for (int j = 0; j < 4; ++j) dot.add(vv[j] * yv[j]);
                }
            }
        }
        __syncthreads();
    }
    if (MODE == FM_CG_DIRECTION || MODE == FM_CG_UPDATE_JACOBI) grid_dot_finish(dot.value(), a.dot, sh);
}

int pick_zc4(const Grid& g, const Ctx& c) {
    const int64_t cols = (int64_t)((g.ny + 1 + 4 * QY - 1) / (4 * QY)) * ((g.nx + 1 + TXC - 1) / TXC);
    const int64_t want = (int64_t)c.num_sms * 2 * 6;     // ~6 waves of resident CTAs
    int64_t zc = (cols * (g.nz + 1) + want - 1) / want;
    if (zc < 4) zc = 4;
    if (zc > 128) zc = 128;
    return (int)zc;
}

template <int MODE>
void set_smem_attr() {
    // per function and device; cheap enough to set before every launch
    GMGS_CUDA(cudaFuncSetAttribute(k_fine4<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM));
}

}  // namespace

// the quad kernels need 16-byte aligned rows (Grid::YOFF = 4, py % 4 == 0)
bool fine4_supported(const Grid& g) { return g.py % 4 == 0 && Grid::YOFF % 4 == 0 && g.slots % 4 == 0; }

int fine4_grid_blocks(const Grid& g) {
    return ((g.ny + 1 + 4 * QY - 1) / (4 * QY)) * ((g.nx + 1 + TXC - 1) / TXC) * ((g.nz + 1 + 3) / 4);
}

template <int MODE>
void launch_fine4(Ctx& c, const FineLevel& L, const Coef32& cf, const FineArgs& a) {
    set_smem_attr<MODE>();
    const int zc = pick_zc4(L.g, c);
    dim3 grid((L.g.ny + 1 + 4 * QY - 1) / (4 * QY), (L.g.nx + 1 + TXC - 1) / TXC, (L.g.nz + 1 + zc - 1) / zc);
    k_fine4<MODE><<<grid, NTH, SMEM, c.stream>>>(L, cf, a, zc);
    GMGS_LAUNCHED(c);
}
template void launch_fine4<FM_PLAIN>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine4<FM_VCYCLE_DOWN>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine4<FM_CG_UPDATE_JACOBI>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);
template void launch_fine4<FM_CG_DIRECTION>(Ctx&, const FineLevel&, const Coef32&, const FineArgs&);

}  // namespace gmgs
