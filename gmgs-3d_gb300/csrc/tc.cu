// Element-form operator on the tensor cores (tcgen05, kind::tf32) for the
// V-cycle down-sweep of the mixed path: out = r - A (omega D^-1 r) with fixed
// rows of A zeroed (src/kernel/Vcycle.m:14 with JacobiSmoother.m:5-9 and
// AtX.m:1-58, the element-by-element product y_e = Ks * x_e of AtX.m:11-16).
//
// One CTA owns a 31 x 7 column of nodes (y fastest) and walks it through z
// one element layer at a time.  The 32 x 8 elements of a layer that touch the
// owned nodes belong to 256 worker threads, one element each; a ninth warp
// issues the MMAs.  Two stages of the A and D operands live in tensor memory,
// so the tensor cores multiply layer k while the workers reduce layer k - 1
// and gather layer k + 1:
//  * gather: each worker forms its element's 24 nodal values of the field
//    v = omega D^-1 r as first differences against the element's origin node
//    (Ke annihilates rigid translations, so Ke v_e = Ke (v_e - v_origin); the
//    differences keep the operand small for smooth fields), reading a
//    three-plane ring of the field in shared memory, and stores them as its
//    row of A (128 rows per MMA group, two groups per layer); one arrival per
//    worker on the stage's "A full" mbarrier;
//  * MMA warp: waits for "A full" (and, two layers on, for the workers to
//    have read the stage's D), issues D = A x Ke for both groups (M = 128,
//    N = 32 with 24 used, K = 24 in three K = 8 steps; Ke in shared memory as
//    TF32) and commits to the stage's "D full" mbarrier;
//  * reduce: each worker reads its element's 24 outputs (tcgen05.ld), arrives
//    on "D empty" and writes them to a double-buffered element-output buffer;
//    after a barrier among the workers every owned node adds the corners of
//    its 4 elements of the layer: the bottom corners finish the node plane of
//    the layer, the top corners start the next one (kept in registers).
// The field planes are loaded two planes ahead into registers and combined
// (r times omega / diag) only when they are stored, so no thread waits on a
// load it has just issued.
//
// Precision: the tensor cores read the FP32 differences as TF32 (10-bit
// mantissa, truncated).  The down-sweep only feeds the preconditioner: its
// result is the fine residual r' = r - A v that the V-cycle restricts, and for
// smooth components |A v| << |r|, so the TF32 error of A v is small against
// r'.  The outer CG's own products keep the FP32 second-difference kernels.
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

constexpr int EY = 32, EX = 8;            // element tile: 256 elements, one per worker thread
constexpr int NY = EY - 1, NX = EX - 1;   // owned node tile
constexpr int SY = EY + 1, SX = EX + 1;   // staged node region
constexpr int SPL = SY * SX;              // 297 points per component plane
constexpr int NWORK = EY * EX;            // worker threads (warps 0-7)
constexpr int NTHR = NWORK + 32;          // + the MMA warp (warp 8)
constexpr int EOS = 36;                   // floats per element in the output buffer (8 corners x 4 + 4):
                                          // 16-byte rows 144 bytes apart hit distinct bank groups
constexpr int TC_COLS = 256;              // tensor-memory columns: A and D of 2 stages x 2 groups, 32 each
constexpr int B_FLOATS = 32 * 24;
constexpr int RING = 4;                   // node planes in the ring (see the loop for why four)
constexpr int RING_FLOATS = (RING * 3 * SPL + 3) / 4 * 4;   // the next buffer stays 16-byte aligned
constexpr int EOUT_FLOATS = NWORK * EOS;
constexpr int NBAR = 6;                   // mbarriers: A full, D full, D empty for 2 stages
constexpr size_t SMEM_BYTES = (size_t)(B_FLOATS + RING_FLOATS + 2 * EOUT_FLOATS) * 4 + NBAR * 8 + 16;   // + TMEM address, flags
static_assert((B_FLOATS + RING_FLOATS) % 4 == 0, "element-output buffers must be 16-byte aligned");
static_assert((B_FLOATS + RING_FLOATS + 2 * EOUT_FLOATS) % 2 == 0, "the mbarriers must be 8-byte aligned");
constexpr uint32_t IDESC = tc::idesc_tf32(128, 32);
constexpr uint32_t WORKER_BAR = 1;        // named barrier of the 256 worker threads

__device__ __forceinline__ int ring_slot(int z) { return (z + RING) % RING; }   // z >= -1
__device__ __forceinline__ uint32_t a_col(int stage, int group) { return (uint32_t)(2 * stage + group) * 32; }
__device__ __forceinline__ uint32_t d_col(int stage, int group) { return 128u + (uint32_t)(2 * stage + group) * 32; }

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

// Raw inputs of one staged point, loaded two planes before they are combined
// into the field.
struct RawPoint {
    float r[3], w[3];
};
// Raw data of a worker's element in one layer.
struct RawElem {
    uint32_t solid = 0;
    int32_t type = 0;
    float scale = 1.f;
};

__global__ void __launch_bounds__(NTHR, 2) k_tc_vdown(FineLevel L, const __grid_constant__ TcCoef cf,
                                                     const float* __restrict__ r32, const float* __restrict__ wdinv,
                                                     float* __restrict__ out, int zc, int* __restrict__ err) {
    extern __shared__ __align__(16) float smem[];
    float* Bs = smem;
    float* ring = Bs + B_FLOATS;
    float* eout = ring + RING_FLOATS;                                    // [2][NWORK * EOS]
    uint64_t* bars = reinterpret_cast<uint64_t*>(eout + 2 * EOUT_FLOATS);
    uint64_t* a_full = bars;          // [2]: one arrival per worker warp
    uint64_t* d_full = bars + 2;      // [2]: the MMA commit
    uint64_t* d_empty = bars + 4;     // [2]: one arrival per worker warp after reading D
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + NBAR);
    // flags[0]: the error flag was already set when this CTA started (read once, by thread 0);
    // flags[1 + (li & 1)]: a worker's wait in layer li ran out (written before that layer's worker
    // barrier, read after it, so every worker leaves the loop in the same layer)
    int* flags = reinterpret_cast<int*>(tslot + 1);

    const Grid& g = L.g;
    const int S = (int)g.slots;
    const int sz = g.py * g.px;
    const int ny0 = blockIdx.x * NY, nx0 = blockIdx.y * NX;   // owned node tile origin
    const int ey0 = ny0 - 1, ex0 = nx0 - 1;                   // element tile origin = staged origin
    const int zb = blockIdx.z * zc;
    const int ze = min(zb + zc, g.nz + 1);                     // owned node planes [zb, ze)
    const int nl = ze - zb + 1;                                // element layers zb - 1 .. ze - 1
    if (L.tile_occ) {
        int any = 0;
        for (int iz = zb; iz < ze; ++iz)
            any |= L.tile_occ[((int64_t)iz * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x];
        if (!any) return;
    }
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    const bool worker = w < NWORK / 32;

    for (int i = t; i < B_FLOATS; i += NTHR) Bs[i] = cf.B[i];
    if (w == NWORK / 32) {
        tc::tmem_alloc(tslot, TC_COLS);
        tc::tmem_relinquish();
    }
    if (t == 0) {
        for (int s = 0; s < 2; ++s) {
            tc::mbar_init(a_full + s, NWORK / 32);    // one arrival per worker warp
            tc::mbar_init(d_full + s, 1);
            tc::mbar_init(d_empty + s, NWORK / 32);
        }
        tc::mbar_fence_init();
        // an earlier CTA's tensor-core wait ran out: the result is void, skip the work
        flags[0] = *reinterpret_cast<volatile int*>(err);
        flags[1] = flags[2] = 0;
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tb = *tslot;
    const bool skip = flags[0] != 0;

    if (skip) {
        // nothing issued: free the tensor memory below
    } else if (!worker) {
        // ------------------------------------------------------------ MMA warp
        if (lane == 0) {
            const uint32_t bsa = tc::smem_u32(Bs);
            for (int li = 0; li < nl; ++li) {
                const int s = li & 1;
                const uint32_t par = (uint32_t)(li >> 1) & 1u;
                bool ok = tc::mbar_wait_bounded(a_full + s, par);
                if (ok && li >= 2) ok = tc::mbar_wait_bounded(d_empty + s, par ^ 1u);
                if (!ok) {             // the workers stopped (or never arrived): issue no more
                    atomicExch(err, 1);
                    break;
                }
                tc::fence_after_sync();
#pragma unroll
                for (int gg = 0; gg < 2; ++gg)
#pragma unroll
                    for (int kk = 0; kk < 3; ++kk)
                        tc::mma_tf32_ts(tb + d_col(s, gg), tb + a_col(s, gg) + 8 * kk,
                                        tc::smem_desc(bsa + kk * 256, 128, 768), IDESC, kk > 0);
                tc::mma_commit(d_full + s);
            }
        }
    } else {
        // ------------------------------------------------------------ workers
        const int grp = w >> 2;
        const uint32_t lane_base = (uint32_t)((w & 3) * 32) << 16;

        // staged points of this thread: p0 = t, p1 = t + NWORK (41 threads)
        const bool has_p1 = t + NWORK < SPL;
        auto point_slot = [&](int p, bool& ok) {
            const int gy = ey0 + p % SY, gx = ex0 + p / SY;
            ok = gy >= 0 && gx >= 0 && gy <= g.ny && gx <= g.nx;
            return (gx + 1) * g.py + gy + Grid::YOFF + sz;   // + iz * sz
        };
        bool ok0, ok1 = false;
        const int base0 = point_slot(t, ok0);
        const int base1 = has_p1 ? point_slot(t + NWORK, ok1) : 0;
        auto fetch = [&](int iz, RawPoint& p0, RawPoint& p1) {   // loads only
            const bool zok = iz >= 0 && iz <= g.nz;
            const long long n3 = 3ll * S;
            constexpr int F = chk::TC_FIELD;
#pragma unroll
            for (int c = 0; c < 3; ++c) p0.r[c] = p0.w[c] = p1.r[c] = p1.w[c] = 0.f;
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
            constexpr long long R = RING * 3 * SPL;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                chk::st(ring, rs + c * SPL + t, R, chk::TC_RING, p0.r[c] * p0.w[c]);
                if (has_p1) chk::st(ring, rs + c * SPL + t + NWORK, R, chk::TC_RING, p1.r[c] * p1.w[c]);
            }
        };

        // this thread's element (lane, w) of the tile
        const int egy = ey0 + lane, egx = ex0 + w;
        const bool ecol = egy >= 0 && egx >= 0 && egy < g.ny && egx < g.nx;
        const int eslot0 = (egx + 1) * g.py + egy + Grid::YOFF + sz;
        auto elem_fetch = [&](int ez) {   // loads only
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

        // first differences of this element in layer ez (node planes ez, ez + 1
        // in the ring) times the row scale, stored as its row of A in stage s
        auto gather_store = [&](int ez, float sc, int s) {
            const float* P0 = ring + ring_slot(ez) * 3 * SPL;
            const float* P1 = ring + ring_slot(ez + 1) * 3 * SPL;
            const int o = lane + w * SY;    // staged index of the element's origin node (dy = dx = 0)
            constexpr long long R = 3 * SPL;
            const float u[3] = {chk::ld(P0, o, R, chk::TC_RING), chk::ld(P0, SPL + o, R, chk::TC_RING),
                                chk::ld(P0, 2 * SPL + o, R, chk::TC_RING)};
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
                float a8[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int k = 8 * kk + i, j = k / 3, b = k % 3;
                    const float* P = corner_z(j) ? P1 : P0;
                    a8[i] = (chk::ld(P, b * SPL + o + corner_y(j) + corner_x(j) * SY, R, chk::TC_RING) - u[b]) * sc;
                }
                tc::tmem_st8(tb + lane_base + a_col(s, grp) + 8 * kk, a8);
            }
            tc::tmem_wait_st();
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(a_full + s);
        };

        // this thread's owned node (lane, w) for lane < 31, w < 7
        const int ngy = ny0 + lane, ngx = nx0 + w;
        const bool nown = lane < NY && w < NX && ngy <= g.ny && ngx <= g.nx;
        const int nslot0 = (ngx + 1) * g.py + ngy + Grid::YOFF + sz;
        // element-output rows of the node's 4 elements in a layer: element (lane + 1 - dy, w + 1 - dx)
        const int erow00 = (lane + 1 + (w + 1) * EY) * EOS;

        // prologue: node planes zb - 1 .. zb + 1 in the ring, plane zb + 2
        // loading, layer zb - 1 (local 0) in stage 0, layer zb's element data loading.
        // Ring slots: the loop stores plane ez + 3 in layer ez into the slot of
        // plane ez - 1, whose last reader (the gather of layer ez - 1, in the
        // previous layer or the prologue) finished before the previous worker
        // barrier; with three slots the prologue's gather would race with the
        // first layer's store.
        RawPoint p0, p1;
        fetch(zb - 1, p0, p1);
        store(zb - 1, p0, p1);
        fetch(zb, p0, p1);
        store(zb, p0, p1);
        fetch(zb + 1, p0, p1);
        store(zb + 1, p0, p1);
        fetch(zb + 2, p0, p1);
        const float sc0 = elem_scale(elem_fetch(zb - 1));
        RawElem en = elem_fetch(zb);
        tc::named_sync(WORKER_BAR, NWORK);
        gather_store(zb - 1, sc0, 0);

        float part[3] = {0.f, 0.f, 0.f};    // top-corner sums of the previous layer for the current plane
        uint32_t nf = 0;                    // flags and residual of the plane the next layer finishes
        float rn[3] = {0.f, 0.f, 0.f};      // (loaded one layer ahead; plane zb - 1 is not owned)
#pragma unroll 1
        for (int li = 0; li < nl; ++li) {
            const int ez = zb - 1 + li;
            const int s = li & 1;
            // 1. the next layer into the other stage, while the MMA of this one runs;
            //    that stage's previous MMA (layer li - 1) completed before its D was read
            if (li + 1 < nl) {
                gather_store(ez + 1, elem_scale(en), s ^ 1);
                if (li + 2 < nl) en = elem_fetch(ez + 2);
            }
            // 2. this layer's outputs
            bool ok = tc::mbar_wait_bounded(d_full + s, (uint32_t)(li >> 1) & 1u);
            if (!ok) {
                atomicExch(err, 1);
                flags[1 + s] = 1;
            }
            ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld is warp-collective
            tc::fence_after_sync();
            float* eo = eout + s * EOUT_FLOATS + t * EOS;
            if (ok) {
                float d[3][8];
#pragma unroll
                for (int kk = 0; kk < 3; ++kk) tc::tmem_ld8(tb + lane_base + d_col(s, grp) + 8 * kk, d[kk]);
                tc::tmem_wait_ld();
                tc::fence_before_sync();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(d_empty + s);
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int c = corner_y(j) + 2 * corner_x(j) + 4 * corner_z(j);
                    const float y0 = d[(3 * j) / 8][(3 * j) % 8];
                    const float y1 = d[(3 * j + 1) / 8][(3 * j + 1) % 8];
                    const float y2 = d[(3 * j + 2) / 8][(3 * j + 2) % 8];
                    if (chk::ok(s * EOUT_FLOATS + t * EOS + 4 * c + 3, 2 * EOUT_FLOATS, chk::TC_EOUT))
                        *reinterpret_cast<float4*>(eo + 4 * c) = make_float4(y0, y1, y2, 0.f);
                }
            }
            // 3. node plane ez + 3 into the ring slot of plane ez - 1, and the loads of plane ez + 4
            if (li + 2 < nl) {
                store(ez + 3, p0, p1);
                fetch(ez + 4, p0, p1);
            }
            tc::named_sync(WORKER_BAR, NWORK);
            if (*reinterpret_cast<volatile int*>(flags + 1 + s)) break;
            // 4. owned node: finish plane ez with this layer's bottom corners, start plane ez + 1
            if (nown) {
                const float* eb0 = eout + s * EOUT_FLOATS;
                float yb[3] = {part[0], part[1], part[2]};
                float yt[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int dy = 0; dy < 2; ++dy)
#pragma unroll
                    for (int dx = 0; dx < 2; ++dx) {
                        const int eb = erow00 - (dy + dx * EY) * EOS;
                        float4 b = make_float4(0.f, 0.f, 0.f, 0.f), tp = b;
                        if (chk::ok(eb, EOUT_FLOATS - 32, chk::TC_EOUT)) {
                            b = *reinterpret_cast<const float4*>(eb0 + eb + 4 * (dy + 2 * dx));
                            tp = *reinterpret_cast<const float4*>(eb0 + eb + 4 * (dy + 2 * dx + 4));
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
        }
    }
    // every MMA this CTA issued has completed (the workers waited for each
    // layer's D, or the MMA warp stopped issuing) before the memory is freed
    tc::fence_before_sync();
    __syncthreads();
    if (w == NWORK / 32) tc::tmem_dealloc(tb, TC_COLS);
}

int tc_grid_blocks(const Grid& g, int zc) {
    return ((g.ny + 1 + NY - 1) / NY) * ((g.nx + 1 + NX - 1) / NX) * ((g.nz + 1 + zc - 1) / zc);
}

static int tc_zc(const Grid& g, const Ctx& c) {
    const int64_t cols = (int64_t)((g.ny + 1 + NY - 1) / NY) * ((g.nx + 1 + NX - 1) / NX);
    const int64_t want = (int64_t)c.num_sms * 2 * 8;       // ~8 waves of 2 resident CTAs per SM
    int64_t zc = (cols * (g.nz + 1) + want - 1) / want;
    return (int)std::min<int64_t>(128, std::max<int64_t>(8, zc));
}

void launch_tc_vdown(Ctx& c, const FineLevel& L, const TcCoef& cf, const float* r32, const float* wdinv, float* out,
                     int* err) {
    static bool attr_set = false;    // per process; the attribute is a property of the function
    if (!attr_set) {
        GMGS_CUDA(cudaFuncSetAttribute(k_tc_vdown, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
        attr_set = true;
    }
    const int zc = tc_zc(L.g, c);
    const dim3 grid((L.g.ny + 1 + NY - 1) / NY, (L.g.nx + 1 + NX - 1) / NX, (L.g.nz + 1 + zc - 1) / zc);
    k_tc_vdown<<<grid, NTHR, SMEM_BYTES, c.stream>>>(L, cf, r32, wdinv, out, zc, err);
    GMGS_LAUNCHED(c);
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
    k_tc_tile_occ<<<grid, NWORK, 0, c.stream>>>(g, nflag, occ);
    GMGS_LAUNCHED(c);
}

}  // namespace gmgs
