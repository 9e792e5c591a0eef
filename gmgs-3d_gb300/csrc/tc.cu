// Element-form operator on the tensor cores (tcgen05, kind::tf32) for the
// V-cycle down-sweep of the mixed path: out = r - A (omega D^-1 r) with fixed
// rows of A zeroed (src/kernel/Vcycle.m:14 with JacobiSmoother.m:5-9 and
// AtX.m:1-58, the element-by-element product y_e = Ks * x_e of AtX.m:11-16).
//
// One CTA owns a 31 x 7 column of nodes (y fastest) and walks it through z
// one element layer at a time.  The 32 x 8 elements of a layer that touch the
// owned nodes are one per thread.  Per layer:
//  1. every thread gathers its element's 24 nodal values of the field
//     v = omega D^-1 r from a three-plane ring in shared memory, as first
//     differences against the element's own origin node (Ke annihilates
//     rigid translations, so Ke v_e = Ke (v_e - v_origin); the differences
//     keep the operand small for smooth fields), and writes them to its row
//     of the A operand in tensor memory (128 rows per MMA, two MMAs per layer);
//  2. one thread issues D = A x Ke (M = 128, N = 32 with 24 used, K = 24 in
//     three K = 8 steps) for both halves, Ke in shared memory as TF32;
//  3. every thread reads its element's 24 outputs back (tcgen05.ld) into a
//     shared element-output buffer;
//  4. every owned node sums the contributions of its 4 elements in this
//     layer: the bottom corners finish the node plane of this layer, the top
//     corners start the next one (kept in registers).
// The next plane of the field is loaded into registers while the MMA runs.
//
// Precision: the tensor cores read the FP32 differences as TF32 (10-bit
// mantissa).  The down-sweep only feeds the preconditioner: its result is
// the fine residual r' = r - A v that the V-cycle restricts, and for smooth
// components |A v| << |r|, so the TF32 error of A v is small against r'.
// The outer CG's own products keep the FP32 second-difference kernels.
//
// Elements with their own stored matrix (coarse levels) and the nodes they
// touch (NF_PEREL) are left to k_perel_vdown; the element rows of such
// elements are zero here and PEREL nodes are not written.
#include <cstdlib>
#include <cstring>

#include "fine.cuh"
#include "tcgen05.cuh"

namespace gmgs {

namespace {

constexpr int EY = 32, EX = 8;            // element tile: 256 elements, one per thread
constexpr int NY = EY - 1, NX = EX - 1;   // owned node tile
constexpr int SY = EY + 1, SX = EX + 1;   // staged node region
constexpr int SPL = SY * SX;              // 297 points per component plane
constexpr int NTHR = EY * EX;
constexpr int EOS = 36;                   // floats per element in the output buffer (8 corners x 4 + 4):
                                          // 16-byte rows 144 bytes apart hit distinct bank groups
constexpr int TC_COLS = 128;              // tensor-memory columns per CTA: A and D of two MMA groups
constexpr int B_FLOATS = 32 * 24;
constexpr int RING_FLOATS = (3 * 3 * SPL + 3) / 4 * 4;   // 2,676 floats: the next buffer stays 16-byte aligned
constexpr size_t SMEM_BYTES = (size_t)(B_FLOATS + RING_FLOATS + NTHR * EOS) * 4 + 16;   // + mbarrier, TMEM address, stop flag
static_assert((B_FLOATS + RING_FLOATS) % 4 == 0, "element-output buffer must be 16-byte aligned");
static_assert((B_FLOATS + RING_FLOATS + NTHR * EOS) % 2 == 0, "the mbarrier must be 8-byte aligned");
constexpr uint32_t IDESC = tc::idesc_tf32(128, 32);

__device__ __forceinline__ int ring_slot(int z) { return (z + 3) % 3; }   // z >= -1

}  // namespace

// Ke (row = output DOF) in the tensor cores' K-major no-swizzle layout, rounded
// to TF32 (nearest, ties to even); output rows 24..31 are zero.
void make_tc_coef(const double* ke_rows, TcCoef& c) {
    for (int i = 0; i < B_FLOATS; ++i) c.B[i] = 0.f;
    for (int n = 0; n < 24; ++n)
        for (int k = 0; k < 24; ++k) {
            float f = (float)ke_rows[n * 24 + k];
            uint32_t u;
            std::memcpy(&u, &f, 4);
            u += 0x0FFFu + ((u >> 13) & 1u);
            u &= 0xFFFFE000u;
            std::memcpy(&f, &u, 4);
            c.B[((n / 8) * 6 + k / 4) * 32 + (n % 8) * 4 + (k % 4)] = f;
        }
}

// Raw inputs of one staged point, loaded a layer before they are combined
// into the field (so no thread waits on a load it has just issued).
struct RawPoint {
    float r[3], w[3];
};
// Raw data of this thread's element in one layer.
struct RawElem {
    uint32_t solid = 0;
    int32_t type = 0;
    float scale = 1.f;
};

template <int MINB>
__global__ void __launch_bounds__(NTHR, MINB) k_tc_vdown(FineLevel L, const __grid_constant__ TcCoef cf,
                                                     const float* __restrict__ r32, const float* __restrict__ wdinv,
                                                     float* __restrict__ out, int zc, int* __restrict__ err) {
    extern __shared__ __align__(16) float smem[];
    float* Bs = smem;
    float* ring = Bs + B_FLOATS;
    float* eout = ring + RING_FLOATS;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(eout + NTHR * EOS);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
    int& stop = *reinterpret_cast<int*>(tslot + 1);     // a tensor-core wait ran out: every thread leaves

    const Grid& g = L.g;
    const int S = (int)g.slots;
    const int sz = g.py * g.px;
    const int ny0 = blockIdx.x * NY, nx0 = blockIdx.y * NX;   // owned node tile origin
    const int ey0 = ny0 - 1, ex0 = nx0 - 1;                   // element tile origin = staged origin
    const int zb = blockIdx.z * zc;
    const int ze = min(zb + zc, g.nz + 1);                     // owned node planes [zb, ze)
    if (L.tile_occ) {
        int any = 0;
        for (int iz = zb; iz < ze; ++iz)
            any |= L.tile_occ[((int64_t)iz * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x];
        if (!any) return;
    }
    // an earlier CTA's tensor-core wait ran out: the result is void, leave at once
    if (*reinterpret_cast<volatile int*>(err)) return;
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;

    for (int i = t; i < B_FLOATS; i += NTHR) Bs[i] = cf.B[i];
    if (w == 0) {
        tc::tmem_alloc(tslot, TC_COLS);
        tc::tmem_relinquish();
    }
    if (t == 0) {
        tc::mbar_init(mbar, 1);
        tc::mbar_fence_init();
        stop = 0;
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tb = *tslot;
    const uint32_t lane_base = (uint32_t)((w & 3) * 32) << 16;
    const uint32_t a_col = (uint32_t)(w >> 2) * 64, d_col = a_col + 32;

    // staged points of this thread: p0 = t, p1 = t + NTHR (41 threads)
    const bool has_p1 = t + NTHR < SPL;
    auto point_slot = [&](int p, bool& ok) {
        const int gy = ey0 + p % SY, gx = ex0 + p / SY;
        ok = gy >= 0 && gx >= 0 && gy <= g.ny && gx <= g.nx;
        return (gx + 1) * g.py + gy + Grid::YOFF + sz;   // + iz * sz
    };
    bool ok0, ok1 = false;
    const int base0 = point_slot(t, ok0);
    const int base1 = has_p1 ? point_slot(t + NTHR, ok1) : 0;
    auto fetch = [&](int iz, RawPoint& p0, RawPoint& p1) {   // loads only
        const bool zok = iz >= 0 && iz <= g.nz;
        const long long n3 = 3ll * S;
        constexpr int F = chk::TC_FIELD;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            p0.r[c] = p0.w[c] = p1.r[c] = p1.w[c] = 0.f;
        }
        if (zok && ok0) {
            const int i = base0 + iz * sz;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                p0.r[c] = chk::ld(r32, i + c * S, n3, F);
                p0.w[c] = chk::ld(wdinv, i + c * S, n3, F);
            }
        }
        if (zok && ok1) {
            const int i = base1 + iz * sz;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                p1.r[c] = chk::ld(r32, i + c * S, n3, F);
                p1.w[c] = chk::ld(wdinv, i + c * S, n3, F);
            }
        }
    };
    auto store = [&](int iz, const RawPoint& p0, const RawPoint& p1) {   // the field v = omega D^-1 r
        const int rs = ring_slot(iz) * 3 * SPL;
        constexpr long long R = 3 * 3 * SPL;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            chk::st(ring, rs + c * SPL + t, R, chk::TC_RING, p0.r[c] * p0.w[c]);
            if (has_p1) chk::st(ring, rs + c * SPL + t + NTHR, R, chk::TC_RING, p1.r[c] * p1.w[c]);
        }
    };

    // this thread's element (lane, w) of the tile and its solid/type data
    const int egy = ey0 + lane, egx = ex0 + w;
    const bool ecol = egy >= 0 && egx >= 0 && egy < g.ny && egx < g.nx;
    const int eslot0 = (egx + 1) * g.py + egy + Grid::YOFF + sz;
    auto elem_fetch = [&](int ez) {            // loads only
        RawElem e;
        if (!ecol || ez < 0 || ez >= g.nz) return e;
        const int es = eslot0 + ez * sz;
        constexpr int E = chk::TC_ELEM;
        e.solid = chk::ld(L.emask, es, S, E);
        if (L.etype) e.type = chk::ld(L.etype, es, S, E);
        if (L.escale) e.scale = chk::ld(L.escale, es, S, E);
        return e;
    };
    // the element's row scale: 0 for void elements and for those with their own matrix
    auto elem_scale = [](const RawElem& e) { return (e.solid && e.type <= 0) ? e.scale : 0.f; };

    // first differences of this thread's element in the layer whose node
    // planes are in ring slots P0 (bottom) and P1 (top), times the row scale
    auto gather = [&](int ez, float s, float (&a)[24]) {
        const float* P0 = ring + ring_slot(ez) * 3 * SPL;
        const float* P1 = ring + ring_slot(ez + 1) * 3 * SPL;
        const int o = lane + w * SY;    // staged index of the element's origin node (dy = dx = 0)
        constexpr long long R = 3 * SPL;
        const float u[3] = {chk::ld(P0, o, R, chk::TC_RING), chk::ld(P0, SPL + o, R, chk::TC_RING),
                            chk::ld(P0, 2 * SPL + o, R, chk::TC_RING)};
#pragma unroll
        for (int k = 0; k < 24; ++k) {
            const int j = k / 3, b = k % 3;
            const float* P = corner_z(j) ? P1 : P0;
            a[k] = (chk::ld(P, b * SPL + o + corner_y(j) + corner_x(j) * SY, R, chk::TC_RING) - u[b]) * s;
        }
    };
    auto store_a = [&](const float (&a)[24]) {
#pragma unroll
        for (int kk = 0; kk < 3; ++kk) {
            float a8[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) a8[i] = a[8 * kk + i];
            tc::tmem_st8(tb + lane_base + a_col + 8 * kk, a8);
        }
    };

    // this thread's owned node (lane, w) for lane < 31, w < 7
    const int ngy = ny0 + lane, ngx = nx0 + w;
    const bool nown = lane < NY && w < NX && ngy <= g.ny && ngx <= g.nx;
    const int nslot0 = (ngx + 1) * g.py + ngy + Grid::YOFF + sz;
    // element-output rows of the node's 4 elements in a layer: element (lane + 1 - dy, w + 1 - dx)
    const int erow00 = (lane + 1 + (w + 1) * EY) * EOS;

    // prologue: node planes zb - 1 .. zb + 1 in the ring, plane zb + 2 loading,
    // layer zb - 1 in the A operand, layer zb's element data loading
    RawPoint p0, p1;
    fetch(zb - 1, p0, p1);
    store(zb - 1, p0, p1);
    fetch(zb, p0, p1);
    store(zb, p0, p1);
    fetch(zb + 1, p0, p1);
    store(zb + 1, p0, p1);
    fetch(zb + 2, p0, p1);
    RawElem en = elem_fetch(zb);
    {
        const float s = elem_scale(elem_fetch(zb - 1));
        __syncthreads();
        float a[24];
        gather(zb - 1, s, a);
        store_a(a);
    }
    float part[3] = {0.f, 0.f, 0.f};         // top-corner sums of the previous layer for the current plane
    uint32_t nf = 0;                         // flags and residual of the plane the next layer finishes
    float rn[3] = {0.f, 0.f, 0.f};           // (loaded one layer ahead; plane zb - 1 is not owned)

    uint32_t phase = 0;
#pragma unroll 1
    for (int ez = zb - 1; ez < ze; ++ez) {
        // A holds layer ez; the ring holds node planes ez .. ez + 2
        tc::tmem_wait_st();
        tc::fence_before_sync();
        __syncthreads();
        if (t == 0) {
            tc::fence_after_sync();
            const uint32_t bsa = tc::smem_u32(Bs);
#pragma unroll
            for (int gg = 0; gg < 2; ++gg)
#pragma unroll
                for (int kk = 0; kk < 3; ++kk)
                    tc::mma_tf32_ts(tb + gg * 64 + 32, tb + gg * 64 + 8 * kk, tc::smem_desc(bsa + kk * 256, 128, 768),
                                    IDESC, kk > 0);
            tc::mma_commit(mbar);
        }
        // while the MMA runs: the next layer's differences and element data
        const bool more = ez + 1 < ze;
        float a[24];
        if (more) gather(ez + 1, elem_scale(en), a);
        if (ez + 2 < ze) en = elem_fetch(ez + 2);
        // wait for the MMA, then the next layer's rows replace this one's in A
        bool ok = tc::mbar_wait_bounded(mbar, phase);
        if (!ok) {
            atomicExch(err, 1);
            stop = 1;
            ok = tc::mbar_wait_bounded(mbar, phase);   // its writes must end before TMEM is freed
        }
        ok = __all_sync(0xffffffffu, ok);               // tcgen05.ld/st are warp-collective
        if (t == 0 && *reinterpret_cast<volatile int*>(err)) stop = 1;   // another CTA gave up
        phase ^= 1u;
        tc::fence_after_sync();
        if (ok) {
            if (more) store_a(a);     // A is free once the MMA is done; storing first frees a's registers
            float d[3][8];
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) tc::tmem_ld8(tb + lane_base + d_col + 8 * kk, d[kk]);
            tc::tmem_wait_ld();
            float* eo = eout + t * EOS;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int c = corner_y(j) + 2 * corner_x(j) + 4 * corner_z(j);
                const float y0 = d[(3 * j) / 8][(3 * j) % 8];
                const float y1 = d[(3 * j + 1) / 8][(3 * j + 1) % 8];
                const float y2 = d[(3 * j + 2) / 8][(3 * j + 2) % 8];
                if (chk::ok(t * EOS + 4 * c + 3, NTHR * EOS, chk::TC_EOUT))
                    *reinterpret_cast<float4*>(eo + 4 * c) = make_float4(y0, y1, y2, 0.f);
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        if (stop) break;
        // owned node: finish plane ez with this layer's bottom corners, start plane ez + 1
        if (nown) {
            float yb[3] = {part[0], part[1], part[2]};
            float yt[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int dy = 0; dy < 2; ++dy)
#pragma unroll
                for (int dx = 0; dx < 2; ++dx) {
                    const int eb = erow00 - (dy + dx * EY) * EOS;
                    const float* eo = eout + eb;
                    float4 b = make_float4(0.f, 0.f, 0.f, 0.f), tp = b;
                    if (chk::ok(eb, NTHR * EOS - 32, chk::TC_EOUT)) {
                        b = *reinterpret_cast<const float4*>(eo + 4 * (dy + 2 * dx));
                        tp = *reinterpret_cast<const float4*>(eo + 4 * (dy + 2 * dx + 4));
                    }
                    yb[0] += b.x; yb[1] += b.y; yb[2] += b.z;
                    yt[0] += tp.x; yt[1] += tp.y; yt[2] += tp.z;
                }
            if (ez >= zb && (nf & NF_SOLID) && !(nf & NF_PEREL)) {
                const int n = nslot0 + ez * sz;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float y = (nf & (NF_FIX_X << c)) ? 0.f : yb[c] * L.kscale;
                    chk::st(out, n + c * S, 3ll * S, chk::TC_OUT, rn[c] - y);
                }
            }
            part[0] = yt[0]; part[1] = yt[1]; part[2] = yt[2];
            // node data of plane ez + 1 for the next layer
            if (ez + 1 < ze && ez + 1 >= 0) {
                const int n = nslot0 + (ez + 1) * sz;
                nf = chk::ld(L.nflag, n, S, chk::TC_NODE);
#pragma unroll
                for (int c = 0; c < 3; ++c) rn[c] = chk::ld(r32, n + c * S, 3ll * S, chk::TC_NODE);
            }
        }
        // node plane ez + 3 into the ring slot of plane ez (no longer read),
        // and the loads of plane ez + 4
        if (ez + 2 < ze) {
            store(ez + 3, p0, p1);
            fetch(ez + 4, p0, p1);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (w == 0) tc::tmem_dealloc(tb, TC_COLS);
}

int tc_grid_blocks(const Grid& g, int zc) {
    return ((g.ny + 1 + NY - 1) / NY) * ((g.nx + 1 + NX - 1) / NX) * ((g.nz + 1 + zc - 1) / zc);
}

static int tc_zc(const Grid& g, const Ctx& c, int minb) {
    const int64_t cols = (int64_t)((g.ny + 1 + NY - 1) / NY) * ((g.nx + 1 + NX - 1) / NX);
    const int64_t want = (int64_t)c.num_sms * minb * 12;   // ~12 waves of the resident CTAs
    int64_t zc = (cols * (g.nz + 1) + want - 1) / want;
    return (int)std::min<int64_t>(64, std::max<int64_t>(8, zc));
}

template <int MINB>
static void launch_tc_vdown_t(Ctx& c, const FineLevel& L, const TcCoef& cf, const float* r32, const float* wdinv,
                              float* out, int* err) {
    static bool attr_set = false;    // per process; the attribute is a property of the function
    if (!attr_set) {
        GMGS_CUDA(cudaFuncSetAttribute(k_tc_vdown<MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
        attr_set = true;
    }
    const int zc = tc_zc(L.g, c, MINB);
    const dim3 grid((L.g.ny + 1 + NY - 1) / NY, (L.g.nx + 1 + NX - 1) / NX, (L.g.nz + 1 + zc - 1) / zc);
    k_tc_vdown<MINB><<<grid, NTHR, SMEM_BYTES, c.stream>>>(L, cf, r32, wdinv, out, zc, err);
    GMGS_LAUNCHED(c);
}

void launch_tc_vdown(Ctx& c, const FineLevel& L, const TcCoef& cf, const float* r32, const float* wdinv, float* out,
                     int* err) {
    const char* e = std::getenv("GMGS_TC_MINB");
    if (e && e[0] == '2') launch_tc_vdown_t<2>(c, L, cf, r32, wdinv, out, err);
    else launch_tc_vdown_t<3>(c, L, cf, r32, wdinv, out, err);
}

// occupancy of the element-form kernel's 31 x 7 node tiles per z plane
__global__ void k_tc_tile_occ(Grid g, const uint8_t* __restrict__ nflag, uint8_t* __restrict__ occ) {
    const int ty = threadIdx.x & 31, tx = threadIdx.x >> 5;
    const int iy = blockIdx.x * NY + ty, ix = blockIdx.y * NX + tx, iz = blockIdx.z;
    const bool solid = ty < NY && tx < NX && iy <= g.ny && ix <= g.nx && (nflag[g.slot(iy, ix, iz)] & NF_SOLID);
    const int any = __syncthreads_or(solid);
    if (threadIdx.x == 0) occ[((int64_t)iz * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = any ? 1 : 0;
}
size_t tc_tile_occ_bytes(const Grid& g) {
    return (size_t)((g.ny + 1 + NY - 1) / NY) * ((g.nx + 1 + NX - 1) / NX) * (g.nz + 1);
}
void launch_tc_tile_occ(Ctx& c, const Grid& g, const uint8_t* nflag, uint8_t* occ) {
    const dim3 grid((g.ny + 1 + NY - 1) / NY, (g.nx + 1 + NX - 1) / NX, g.nz + 1);
    k_tc_tile_occ<<<grid, NTHR, 0, c.stream>>>(g, nflag, occ);
    GMGS_LAUNCHED(c);
}

}  // namespace gmgs
