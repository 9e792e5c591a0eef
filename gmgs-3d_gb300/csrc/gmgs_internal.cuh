// Internal definitions of libgmgs: dense per-level node grids on the GPU.
//
// Layout in HBM.  Level l has ny x nx x nz (padded) elements and
// (ny+1) x (nx+1) x (nz+1) nodes.  Nodes live in a dense slot grid with a
// zero halo on every side, y fastest (the reference's column-major (y, x, z)
// order, src/common/DiscretizeDesignDomain.m:76):
//     slot(iy, ix, iz) = ((iz + 1) * px + (ix + 1)) * py + (iy + YOFF)
// The y halo is YOFF = 4 wide so that node rows start on 16-byte boundaries
// (groups of 4 y-nodes load as one float4); x and z halos are one node.
// An element (ey, ex, ez) shares the slot of its lowest-index node, so the 8
// elements around node n are the slots n - {0,1} * {1, py, py*px}.
// Vectors are stored as three component planes of `slots` entries (SoA).
// Every vector is zero on halo and non-solid slots, so stencils need no
// bounds checks.
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "gmgs.h"

namespace gmgs {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define GMGS_CUDA(call)                                                              \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            throw ::gmgs::Error(e_ == cudaErrorMemoryAllocation ? GMGS_ERR_OUT_OF_MEMORY \
                                                                : GMGS_ERR_CUDA,     \
                                std::string(#call) + ": " + cudaGetErrorString(e_)); \
        }                                                                            \
    } while (0)

// Record a kernel launch: check the launch error and count it.
#define GMGS_LAUNCHED(ctx)                                                           \
    do {                                                                             \
        cudaError_t e_ = cudaGetLastError();                                         \
        if (e_ != cudaSuccess)                                                       \
            throw ::gmgs::Error(GMGS_ERR_CUDA, std::string("kernel launch: ") +      \
                                                   cudaGetErrorString(e_));          \
        ++(ctx).launches;                                                            \
    } while (0)

// ---------------------------------------------------------------------------
// checked accesses (build.py --debug compiles with GMGS_CHECKED)
// ---------------------------------------------------------------------------
// chk::ld / chk::st wrap the gathers, scatters and shared-memory staging of
// the solver kernels.  In a checked build each one tests its index against the
// extent of the buffer it touches; an index outside is not accessed (a load
// gives 0) and is recorded: the number of such accesses and the first one's
// site and index, in device words of the translation unit.  Every C-ABI call
// of a checked build then reads those words and fails with GMGS_ERR_CUDA
// naming the site.  Release builds compile the plain access.
namespace chk {
enum Site : int {
    FINE_FIELD = 1, FINE_EPI, FINE_FLAGS, FINE_ELEM, FINE_KS, FINE_RING, FINE_OUT,
    UP_FINE, UP_COARSE, UP_OUT, PEREL_NODE, PEREL_ELEM, PEREL_VEC, PEREL_KS, PEREL_OUT,
    TC_FIELD, TC_ELEM, TC_NODE, TC_RING, TC_EOUT, TC_OUT,
    MV_X, MV_ELEM, MV_Y, RESTRICT, PROLONG, STRESS_U, STRESS_OUT, GRAD,
    SITE_COUNT
};
const char* site_name(int site);
#ifdef GMGS_CHECKED
static __device__ unsigned long long g_first = 0;   // (site << 48) | (index & 2^48-1) of the first violation
static __device__ unsigned int g_count = 0;
__device__ __forceinline__ bool ok(long long i, long long n, int site) {
    if (i >= 0 && i < n) return true;
    atomicAdd(&g_count, 1u);
    atomicCAS(&g_first, 0ull, ((unsigned long long)site << 48) | ((unsigned long long)i & 0xFFFFFFFFFFFFull));
    return false;
}
template <typename T, typename I>
__device__ __forceinline__ T ld(const T* p, I i, long long n, int site) {
    return ok((long long)i, n, site) ? p[i] : T(0);
}
template <typename T, typename I, typename V>
__device__ __forceinline__ void st(T* p, I i, long long n, int site, V v) {
    if (ok((long long)i, n, site)) p[i] = (T)v;
}
// host: each translation unit registers a reader of its own device words
using Reader = bool (*)(std::string& msg);
void add_reader(Reader r);
bool report(std::string& msg);   // true (and msg) when any kernel recorded a violation
static bool read_this_unit(std::string& msg) {
    unsigned long long first = 0;
    unsigned int count = 0;
    if (cudaMemcpyFromSymbol(&first, g_first, sizeof(first)) != cudaSuccess ||
        cudaMemcpyFromSymbol(&count, g_count, sizeof(count)) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (!count) return false;
    const unsigned long long zero = 0;
    const unsigned int zc = 0;
    cudaMemcpyToSymbol(g_first, &zero, sizeof(zero));
    cudaMemcpyToSymbol(g_count, &zc, sizeof(zc));
    const int site = (int)(first >> 48);
    long long idx = (long long)(first & 0xFFFFFFFFFFFFull);
    if (idx & 0x800000000000ll) idx -= 0x1000000000000ll;   // negative indices
    msg = "checked build: " + std::to_string(count) + " out-of-range access(es), first at " + site_name(site) +
          " index " + std::to_string(idx);
    return true;
}
static const bool g_reader_added = (add_reader(&read_this_unit), true);
#else
// the index keeps the caller's type: 32-bit indices stay 32-bit address arithmetic
__device__ __forceinline__ bool ok(long long, long long, int) { return true; }
template <typename T, typename I>
__device__ __forceinline__ T ld(const T* p, I i, long long, int) { return p[i]; }
template <typename T, typename I, typename V>
__device__ __forceinline__ void st(T* p, I i, long long, int, V v) { p[i] = (T)v; }
#endif
}  // namespace chk

// ---------------------------------------------------------------------------
// FP32 <-> FP64 without the FP64 pipe, and double-float sums
// ---------------------------------------------------------------------------
// GB300 runs FP64 adds and FP32<->FP64 conversions at about 2 lanes per clock
// per SM, 1/64 of its FP32 rate.  float -> double and double -> float (round
// to nearest even) with integer operations, equal to the hardware conversions
// bit for bit; values outside the normal float range, zero, infinities and NaN
// take the hardware path.
__device__ __forceinline__ double f2d_int(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xFFu;
    if (e == 0u || e == 0xFFu) return (double)f;
    const uint32_t hi = (u & 0x80000000u) | (((u & 0x7FFFFFFFu) >> 3) + 0x38000000u);
    return __hiloint2double((int)hi, (int)(u << 29));
}
__device__ __forceinline__ float d2f_int(double d) {
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
    const uint32_t e = (hi >> 20) & 0x7FFu;
    if (e < 897u || e > 1150u) return (float)d;
    uint32_t t = ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const uint32_t half = (lo >> 28) & 1u, rest = (lo & 0x0FFFFFFFu) != 0u;
    t += half & (rest | (t & 1u));
    return __uint_as_float((hi & 0x80000000u) | t);
}

// (hi, lo) += a for a double-float hi + lo (|lo| <= ulp(hi) / 2): Knuth's
// branch-free two-sum of hi + a (exact: s + e = hi + a), the low parts added,
// then Dekker's fast two-sum renormalises.  The sum keeps about 48 significant
// bits (relative error ~2^-47 per update), all on the FP32 pipe.
__device__ __forceinline__ void df_add(float& hi, float& lo, float a) {
    const float s = __fadd_rn(hi, a);
    const float bv = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bv)), __fsub_rn(a, bv));
    const float t = __fadd_rn(e, lo);
    const float h = __fadd_rn(s, t);
    lo = __fsub_rn(t, __fsub_rn(h, s));
    hi = h;
}

// ---------------------------------------------------------------------------
// grid geometry
// ---------------------------------------------------------------------------
struct Grid {
    static constexpr int YOFF = 4;
    int ny = 0, nx = 0, nz = 0;   // elements (padded)
    int py = 0, px = 0, pz = 0;   // slot pitches, halo included
    int64_t slots = 0;

    static Grid make(int ny, int nx, int nz) {
        Grid g;
        g.ny = ny; g.nx = nx; g.nz = nz;
        g.py = ((ny + 1 + 2 * YOFF) + 7) / 8 * 8;     // rows start on 32-byte boundaries
        g.px = nx + 3;
        g.pz = nz + 3;
        g.slots = (int64_t)g.py * g.px * g.pz;
        return g;
    }
    __host__ __device__ __forceinline__ int64_t slot(int iy, int ix, int iz) const {
        return ((int64_t)(iz + 1) * px + (ix + 1)) * py + (iy + YOFF);
    }
    // inverse of slot(); halo slots give indices outside [0, n]
    __host__ __device__ __forceinline__ void coords(int64_t s, int& iy, int& ix, int& iz) const {
        iy = (int)(s % py) - YOFF;
        const int64_t r = s / py;
        ix = (int)(r % px) - 1;
        iz = (int)(r / px) - 1;
    }
    __host__ __device__ __forceinline__ int64_t sx() const { return py; }
    __host__ __device__ __forceinline__ int64_t sz() const { return (int64_t)py * px; }
};

// Local node k of an element sits at (iy + CY[k], ix + CX[k], iz + CZ[k]) from the
// element's lowest-index node: node 1 = (iy+1, ix, iz), 2 = (iy+1, ix+1, iz),
// 3 = (iy, ix+1, iz), 4 = (iy, ix, iz), 5..8 the same at iz+1
// (src/common/DiscretizeDesignDomain.m:80).
__host__ __device__ constexpr int corner_y(int k) { return (k & 3) < 2 ? 1 : 0; }
__host__ __device__ constexpr int corner_x(int k) { return ((k & 3) == 1 || (k & 3) == 2) ? 1 : 0; }
__host__ __device__ constexpr int corner_z(int k) { return k >> 2; }
__host__ __device__ constexpr int corner_of(int dy, int dx, int dz) {
    return (dy ? (dx ? 1 : 0) : (dx ? 2 : 3)) + 4 * dz;
}

// node flag bits
enum : uint8_t { NF_SOLID = 1, NF_FIX_X = 2, NF_FIX_Y = 4, NF_FIX_Z = 8 };
constexpr uint8_t NF_INTERIOR = 16;  // all 8 surrounding elements carry the level's kscale * Ke0

// ---------------------------------------------------------------------------
// device-side views passed to kernels by value
// ---------------------------------------------------------------------------
template <typename T>
struct LevelView {
    Grid g;
    const uint8_t* emask;    // element solid / non-empty
    const uint8_t* nflag;    // node flags
    const int32_t* etype;    // -1 void, 0 universal (Kc), k>0 -> Ks[k-1]; null = all universal
    const T* Ks;             // per-element matrices, 576 each, row = output DOF
    int64_t nK;              // matrices held in Ks
    const T* escale;         // finest-level element scale (density extension) or null
    const T* diag;           // 3 planes
    T omega;
};

// ---------------------------------------------------------------------------
// host-side level storage
// ---------------------------------------------------------------------------
// Device bytes held by every DevBuf in the process, and the high-water mark.
inline std::atomic<int64_t> g_dev_bytes{0}, g_dev_peak{0};
inline void count_alloc(int64_t b) {
    const int64_t now = g_dev_bytes.fetch_add(b) + b;
    int64_t pk = g_dev_peak.load();
    while (now > pk && !g_dev_peak.compare_exchange_weak(pk, now)) {
    }
}

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void release() {
        if (p) { cudaFree(p); g_dev_bytes.fetch_sub((int64_t)bytes); }
        p = nullptr;
        bytes = 0;
    }
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

struct Level {
    Grid g;
    int64_t n_elem = 0, n_node = 0;
    int state = 0;            // reference storingState: 0 uniform, 1 per element, 2 unique + universal
    int64_t nK = 0;           // per-element matrices held
    double kscale = 1.0;      // universal matrix = Ke0 * kscale (SetupSolver.m:37)
    DevBuf emask, nflag, etype, escale64, escale32;
    DevBuf Ks64, Ks32;
    DevBuf kslot;             // slot of the coarse element owning Ks[k]
    DevBuf diag64, diag32;
    DevBuf node_slot;         // compact node id -> slot (int32), reference nodMapBack order
    DevBuf elem_slot;         // compact element id -> slot (int32), eleMapBack order
    // V-cycle work vectors (3 planes each), precision of the V-cycle
    DevBuf vr, vrp, vdx, vx, vy;
    DevBuf tile_occ;          // mixed path: per 32x8 node tile and z plane, 1 if it holds a solid node
    DevBuf wdinv32;           // mixed path: omega / diag in FP32
    DevBuf emask8;            // mixed path: per-node mask of the 8 surrounding solid elements
    DevBuf perel_nodes;       // slots of nodes touching an element with its own stored matrix
    DevBuf tc_occ;            // mixed path: per 31x7 node tile (tensor-core kernels) and z plane, 1 if solid
    int64_t n_perel = 0;
};

// Per-launch CUDA-event timing of selected kernels (diagnostics; off by default).
enum ProfKernel {
    PK_FINE_MATVEC = 0,   // every finest-level stencil launch
    PK_VCYCLE = 1,        // whole V-cycles
    PK_CG_ITER = 2,       // whole CG iterations
    PK_UPDATE_JACOBI = 3, // finest fused CG update + Jacobi step
    PK_VDOWN0 = 4,        // finest V-cycle down-sweep
    PK_DIRECTION = 5,     // finest CG direction + q = A p
    PK_UP0 = 6,           // finest prolongation + post-smooth + r.z
    PK_COARSE = 7,        // everything on levels 2..L of a V-cycle
    PK_COUNT = 8
};

struct ProfSlot {
    std::vector<cudaEvent_t> ev;   // start/stop pairs
    int used = 0;                  // events in use (2 per launch)
    double bytes = 0;              // algorithmic bytes of the recorded launches
};

struct Ctx {
    cudaStream_t stream = nullptr;
    int64_t launches = 0;
    int num_sms = 148;
    bool prof = false;
    ProfSlot prof_slot[PK_COUNT];
    // Setup/solve phase trace on stderr (environment GMGS_TRACE=1): each
    // point waits for the stream and prints the wall time since the last one.
    bool trace = false;
    std::chrono::steady_clock::time_point t_trace{};
    void trace_point(const char* what) {
        if (!trace) return;
        cudaStreamSynchronize(stream);
        const auto now = std::chrono::steady_clock::now();
        if (t_trace.time_since_epoch().count())
            std::fprintf(stderr, "[gmgs] %-34s %9.3f ms\n", what,
                         std::chrono::duration<double, std::milli>(now - t_trace).count());
        t_trace = now;
    }
    // record a start (stop=false) or stop event for kernel k
    void mark(int k, bool stop, double bytes = 0) {
        if (!prof) return;
        ProfSlot& s = prof_slot[k];
        if ((int)s.ev.size() <= s.used) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return;
            s.ev.push_back(e);
        }
        cudaEventRecord(s.ev[s.used++], stream);
        if (stop) s.bytes += bytes;
    }
};

// ---------------------------------------------------------------------------
// kernels and launchers (operators.cu, setup.cu, post.cu)
// ---------------------------------------------------------------------------
constexpr int KE = 576;

// uniform element matrices in constant memory: [0] = Ke0 (FP64), [1] = Ke0 (FP32)
// Element matrix Ke0 (row = output DOF) and the assembled 27-point interior
// stencil (3x3 block per offset k, offsets (k%3-1, k/3%3-1, k/9-1) in (y,x,z)),
// passed to the operator kernels as a __grid_constant__ parameter so that
// every handle carries its own material and voxel size.
template <typename T>
struct MatCoef {
    T K[KE];
    T S[243];
};
void make_mat_coef(const double* ke_rows, MatCoef<double>& c64, MatCoef<float>& c32);

template <typename T> LevelView<T> view(const Level& L, double omega);

// y = K_l x, fixed rows zeroed (AtX.m:1-58).  Tin/Tout let the mixed path read
// FP64 CG vectors and compute in FP32.
template <typename Tc, typename Tin, typename Tout>
void launch_matvec(Ctx& c, const LevelView<Tc>& lv, const MatCoef<Tc>& cf, const Tin* x, Tout* y, double kscale);

// dx = (omega r) / d  (JacobiSmoother.m:5)
template <typename Tr, typename Td, typename Tx>
void launch_jacobi_dx(Ctx& c, const Grid& g, const Td* diag, double omega, const Tr* r, Tx* dx);
// x += dx (elementwise over 3 planes)
template <typename T, typename U>
void launch_add(Ctx& c, int64_t n, T* x, const U* dx);
// r -= y
template <typename T, typename U>
void launch_sub(Ctx& c, int64_t n, T* r, const U* y);
// out = a (conversion copy)
template <typename T, typename U>
void launch_copy(Ctx& c, int64_t n, T* out, const U* a);
// out = a - b
template <typename T>
void launch_diff(Ctx& c, int64_t n, T* out, const T* a, const T* b);

// restriction r_c = P^T r_f (RestrictResidual.m) and prolongation with the
// post-smoothing term x_f = (dx + P x_c) + (omega r') / d (Vcycle.m:29-32)
template <typename T>
void launch_restrict(Ctx& c, const Grid& gf, const Grid& gc, const uint8_t* nflag_c,
                     const T* rf, T* rc);
template <typename T>
void launch_prolong_post(Ctx& c, const Grid& gf, const Grid& gc, const uint8_t* nflag_f,
                         const T* diag_f, double omega, const T* xc, const T* dx,
                         const T* rp, T* xf, bool zero_fixed);

// deterministic dot product: out[0] = sum a*b over n entries (FP64 accumulate)
struct DotScratch { double* partials; unsigned int* ticket; int blocks; };
template <typename Ta, typename Tb>
void launch_dot(Ctx& c, const DotScratch& s, int64_t n, const Ta* a, const Tb* b, double* out);

// CG updates.  scal: device scalars (see solver.cu)
// cur_first = (r.z slot) | (first iteration << 1)
template <typename Tz>
void launch_p_update(Ctx& c, int64_t n, const Tz* z, double* p, const double* scal, int cur_first);
template <typename Tq>
void launch_xr_update(Ctx& c, int64_t n, double* x, double* r, const double* p, const Tq* q,
                      const double* scal, int cur);

// coarsest level: gather free DOFs, dense GEMV with the inverse, scatter back
template <typename T>
void launch_gather(Ctx& c, int64_t n, const int32_t* idx, const T* src, double* dst);
template <typename T>
void launch_scatter(Ctx& c, int64_t n, const int32_t* idx, const double* src, T* dst);
// coarsest level: block-tridiagonal LDL^T of the free-DOF matrix, factored
// from both ends towards the middle block (coarse.cu)
struct CoarseBlocks {
    int n = 0;        // free DOFs
    int B = 0;        // block order: a multiple of 64, at least the half bandwidth
    int nb = 0;       // blocks; rows n..nb*B-1 are identity padding
    DevBuf sinv;      // nb x (B x B) column-major: A_ii on entry, D_i^-1 after factor_coarse
    DevBuf g;         // nb x (B x B): A_(i,i-1) on entry, the coupling G_i or H_(i-1) after
    DevBuf partial;   // max(nb, 4) x (B/64) x B partial sums of the block matrix-vector products
    DevBuf ticket;    // max(nb, 4) arrival counters (zero between launches)
};
int coarse_block_order(int n, int half_bandwidth);
// overlap: host work run while the two halves factor on their own streams
// (it may enqueue on c.stream); may be empty
void factor_coarse(Ctx& c, CoarseBlocks& cb, const std::function<void()>& overlap);
// x = A^-1 r: r in cvec (overwritten), both nb*B long with zero padding
void launch_coarse_solve(Ctx& c, const CoarseBlocks& cb, double* cvec, double* x);

// compact <-> dense (interleaved 3-vectors)
template <typename T>
void launch_compact_to_dense(Ctx& c, int64_t nn, int64_t slots, const int32_t* node_slot,
                             const double* src, T* dst);
template <typename T>
void launch_dense_to_compact(Ctx& c, int64_t nn, int64_t slots, const int32_t* node_slot,
                             const T* src, double* dst);

}  // namespace gmgs
