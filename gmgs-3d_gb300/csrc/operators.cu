// Per-level operators of the V-cycle PCG: matrix-free K*x, damped Jacobi,
// trilinear restriction / prolongation, deterministic dot products and the
// CG vector updates.  All kernels work on the dense slot grids described in
// gmgs_internal.cuh and are free of atomics on data (reruns are bitwise equal).
#include "gmgs_internal.cuh"

namespace gmgs {

// stencil offsets of the assembled interior operator (k = 0..26)
__host__ __device__ constexpr int st_y(int k) { return k % 3 - 1; }
__host__ __device__ constexpr int st_x(int k) { return (k / 3) % 3 - 1; }
__host__ __device__ constexpr int st_z(int k) { return k / 9 - 1; }
__host__ __device__ constexpr int st_c(int k, int a) { return a == 0 ? st_x(k) : (a == 1 ? st_y(k) : st_z(k)); }
// structural non-zeros of block S(k)[a][b] (reflection symmetry of the box element)
__host__ __device__ constexpr bool st_nz(int k, int a, int b) { return a == b || (st_c(k, a) != 0 && st_c(k, b) != 0); }

void make_mat_coef(const double* ke_rows, MatCoef<double>& c64, MatCoef<float>& c32) {
    double S[27][9] = {};
    for (int k = 0; k < 27; ++k) {
        const int dy = st_y(k), dx = st_x(k), dz = st_z(k);
        for (int e = 0; e < 8; ++e) {
            const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;     // node = element origin + (A, B, C)
            const int my = A + dy, mx = B + dx, mz = C + dz;       // neighbour relative to the origin
            if (my < 0 || my > 1 || mx < 0 || mx > 1 || mz < 0 || mz > 1) continue;
            const int cn = corner_of(A, B, C), cm = corner_of(my, mx, mz);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) S[k][3 * a + b] += ke_rows[(3 * cn + a) * 24 + 3 * cm + b];
        }
    }
    for (int i = 0; i < KE; ++i) {
        c64.K[i] = ke_rows[i];
        c32.K[i] = (float)ke_rows[i];
    }
    for (int k = 0; k < 27; ++k)
        for (int i = 0; i < 9; ++i) {
            c64.S[k * 9 + i] = S[k][i];
            c32.S[k * 9 + i] = (float)S[k][i];
        }
}

template <typename T>
LevelView<T> view(const Level& L, double omega) {
    LevelView<T> v;
    v.g = L.g;
    v.emask = L.emask.as<uint8_t>();
    v.nflag = L.nflag.as<uint8_t>();
    v.etype = L.etype.as<int32_t>();
    if constexpr (sizeof(T) == 8) {
        v.Ks = L.Ks64.as<T>();
        v.escale = L.escale64.as<T>();
        v.diag = L.diag64.as<T>();
    } else {
        v.Ks = L.Ks32.as<T>();
        v.escale = L.escale32.as<T>();
        v.diag = L.diag32.as<T>();
    }
    v.omega = (T)omega;
    v.nK = v.Ks ? L.nK : 0;
    return v;
}
template LevelView<double> view<double>(const Level&, double);
template LevelView<float> view<float>(const Level&, double);

// ---------------------------------------------------------------------------
// matrix-free K*x, node-centric element-by-element (AtX.m:1-58)
//
// Each thread owns one node and sums the rows of that node over its (up to)
// 8 solid elements: y_n += K_e[3c+a, :] . x_e, c = the node's corner in e.
// Element matrices are stored with row = output DOF (the reference computes
// V = U * Ks, i.e. output column j of Ks; the transposed storage keeps the
// 72 coefficients of one node contiguous).
// ---------------------------------------------------------------------------
template <typename Tc, typename Tin, int C>
__device__ __forceinline__ void elem_rows_const(const MatCoef<Tc>& cf, const Tin* __restrict__ x, int64_t es,
                                                int64_t S, int64_t sx, int64_t sz, Tc s, Tc& a0, Tc& a1, Tc& a2) {
    Tc b0 = 0, b1 = 0, b2 = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int64_t ns = es + corner_y(j) + corner_x(j) * sx + corner_z(j) * sz;
        const Tc x0 = (Tc)chk::ld(x, ns, 3 * S, chk::MV_X), x1 = (Tc)chk::ld(x, ns + S, 3 * S, chk::MV_X),
                 x2 = (Tc)chk::ld(x, ns + 2 * S, 3 * S, chk::MV_X);
        b0 += cf.K[(3 * C + 0) * 24 + 3 * j + 0] * x0 + cf.K[(3 * C + 0) * 24 + 3 * j + 1] * x1 +
              cf.K[(3 * C + 0) * 24 + 3 * j + 2] * x2;
        b1 += cf.K[(3 * C + 1) * 24 + 3 * j + 0] * x0 + cf.K[(3 * C + 1) * 24 + 3 * j + 1] * x1 +
              cf.K[(3 * C + 1) * 24 + 3 * j + 2] * x2;
        b2 += cf.K[(3 * C + 2) * 24 + 3 * j + 0] * x0 + cf.K[(3 * C + 2) * 24 + 3 * j + 1] * x1 +
              cf.K[(3 * C + 2) * 24 + 3 * j + 2] * x2;
    }
    a0 += s * b0; a1 += s * b1; a2 += s * b2;
}

template <typename Tc, typename Tin>
__device__ __forceinline__ void elem_rows_mat(const Tin* __restrict__ x, int64_t es, int64_t S,
                                              int64_t sx, int64_t sz, const Tc* __restrict__ K, int c,
                                              Tc& a0, Tc& a1, Tc& a2) {
    const Tc* k0 = K + (3 * c) * 24;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int64_t ns = es + corner_y(j) + corner_x(j) * sx + corner_z(j) * sz;
        const Tc x0 = (Tc)chk::ld(x, ns, 3 * S, chk::MV_X), x1 = (Tc)chk::ld(x, ns + S, 3 * S, chk::MV_X),
                 x2 = (Tc)chk::ld(x, ns + 2 * S, 3 * S, chk::MV_X);
        a0 += k0[3 * j] * x0 + k0[3 * j + 1] * x1 + k0[3 * j + 2] * x2;
        a1 += k0[24 + 3 * j] * x0 + k0[24 + 3 * j + 1] * x1 + k0[24 + 3 * j + 2] * x2;
        a2 += k0[48 + 3 * j] * x0 + k0[48 + 3 * j + 1] * x1 + k0[48 + 3 * j + 2] * x2;
    }
}

template <typename Tc, typename Tin, int E>
__device__ __forceinline__ void elem_contrib(const LevelView<Tc>& lv, const MatCoef<Tc>& cf, Tc kscale,
                                             const Tin* __restrict__ x,
                                             int64_t n, int64_t S, int64_t sx, int64_t sz,
                                             Tc& a0, Tc& a1, Tc& a2) {
    constexpr int A = E & 1, B = (E >> 1) & 1, Cz = E >> 2;
    constexpr int C = corner_of(A, B, Cz);     // node = element origin + (A, B, Cz)
    const int64_t es = n - A - B * sx - Cz * sz;
    if (!chk::ld(lv.emask, es, S, chk::MV_ELEM)) return;
    if (lv.etype) {
        const int t = chk::ld(lv.etype, es, S, chk::MV_ELEM);
        if (t > 0) {
            if (chk::ok(t - 1, lv.nK, chk::MV_ELEM))
                elem_rows_mat<Tc, Tin>(x, es, S, sx, sz, lv.Ks + (int64_t)(t - 1) * KE, C, a0, a1, a2);
            return;
        }
    }
    Tc s = kscale;
    if (lv.escale) s *= chk::ld(lv.escale, es, S, chk::MV_ELEM);
    elem_rows_const<Tc, Tin, C>(cf, x, es, S, sx, sz, s, a0, a1, a2);
}

// interior node of a uniform level: kscale * (S(0) x(n) + sum over the 13 half
// offsets d of S(d) (x(n+d) + x(n-d))), S(-d) = S(d) on the uniform grid;
// about 117 arithmetic operations instead of the 576 FMAs of the element form
template <typename Tc, typename Tin>
__device__ __forceinline__ void interior_pairs(const MatCoef<Tc>& cf, const Tin* __restrict__ x, int64_t n,
                                               int64_t S, int64_t sx, int64_t sz, Tc& a0, Tc& a1, Tc& a2) {
    Tc acc[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) acc[a] = cf.S[13 * 9 + 4 * a] * (Tc)chk::ld(x, n + a * S, 3 * S, chk::MV_X);   // S(0) is diagonal
#pragma unroll
    for (int k = 14; k < 27; ++k) {
        const int64_t o = st_y(k) + st_x(k) * sx + st_z(k) * sz;
        Tc p[3];
#pragma unroll
        for (int b = 0; b < 3; ++b)
            p[b] = (Tc)chk::ld(x, n + o + b * S, 3 * S, chk::MV_X) + (Tc)chk::ld(x, n - o + b * S, 3 * S, chk::MV_X);
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
                if (st_nz(k, a, b)) acc[a] += cf.S[k * 9 + 3 * a + b] * p[b];
    }
    a0 = acc[0]; a1 = acc[1]; a2 = acc[2];
}

// the void-element complement applies when the level has no per-element
// scale, every solid element around the node carries the uniform matrix and
// at least four of the eight are solid
template <typename Tc>
__device__ __forceinline__ bool complement_ok(const LevelView<Tc>& lv, int64_t n, int64_t sx, int64_t sz) {
    if (lv.escale) return false;
    int solid = 0;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int64_t es = n - (e & 1) - ((e >> 1) & 1) * sx - (e >> 2) * sz;
        if (chk::ld(lv.emask, es, lv.g.slots, chk::MV_ELEM)) {
            ++solid;
            if (lv.etype && chk::ld(lv.etype, es, lv.g.slots, chk::MV_ELEM) > 0) return false;
        }
    }
    return solid >= 6;
}

// rows of corner c of the uniform element at es, times s (run-time corner)
template <typename Tc, typename Tin>
__device__ __noinline__ void elem_rows_rt(const MatCoef<Tc>& cf, const Tin* __restrict__ x, int64_t es, int64_t S,
                                          int64_t sx, int64_t sz, int c, Tc s, Tc& a0, Tc& a1, Tc& a2) {
    Tc b0 = 0, b1 = 0, b2 = 0;
#pragma unroll 1
    for (int j = 0; j < 8; ++j) {
        const int64_t ns = es + corner_y(j) + corner_x(j) * sx + corner_z(j) * sz;
        const Tc x0 = (Tc)chk::ld(x, ns, 3 * S, chk::MV_X), x1 = (Tc)chk::ld(x, ns + S, 3 * S, chk::MV_X),
                 x2 = (Tc)chk::ld(x, ns + 2 * S, 3 * S, chk::MV_X);
        const Tc* k = cf.K + (3 * c) * 24 + 3 * j;
        b0 += k[0] * x0 + k[1] * x1 + k[2] * x2;
        b1 += k[24] * x0 + k[25] * x1 + k[26] * x2;
        b2 += k[48] * x0 + k[49] * x1 + k[50] * x2;
    }
    a0 += s * b0; a1 += s * b1; a2 += s * b2;
}

template <typename Tc, typename Tin, typename Tout>
__global__ void __launch_bounds__(128) k_matvec(LevelView<Tc> lv, const __grid_constant__ MatCoef<Tc> cf, Tc kscale,
                                                const Tin* __restrict__ x, Tout* __restrict__ y) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y * blockDim.y + threadIdx.y;
    const int iz = blockIdx.z;
    const Grid& g = lv.g;
    if (iy > g.ny || ix > g.nx) return;
    const int64_t n = g.slot(iy, ix, iz);
    const int64_t S = g.slots, sx = g.sx(), sz = g.sz();
    const uint8_t f = chk::ld(lv.nflag, n, S, chk::MV_ELEM);
    Tc a0 = 0, a1 = 0, a2 = 0;
    if (f & NF_INTERIOR) {
        interior_pairs<Tc, Tin>(cf, x, n, S, sx, sz, a0, a1, a2);
        a0 *= kscale; a1 *= kscale; a2 *= kscale;
    } else if ((f & NF_SOLID) && complement_ok(lv, n, sx, sz)) {
        // all solid elements uniform, at most two void: the assembled stencil
        // (≈160 FMA) minus the void elements' rows (72 each) costs fewer
        // operations than the solid elements' rows (AtX.m:34-56 sums the
        // latter, 72 each); with three or four void elements it does not
        interior_pairs<Tc, Tin>(cf, x, n, S, sx, sz, a0, a1, a2);
        a0 *= kscale; a1 *= kscale; a2 *= kscale;
#pragma unroll 1
        for (int e = 0; e < 8; ++e) {
            const int A = e & 1, B = (e >> 1) & 1, Cz = e >> 2;
            const int64_t es = n - A - B * sx - Cz * sz;
            if (chk::ld(lv.emask, es, S, chk::MV_ELEM)) continue;
            elem_rows_rt<Tc, Tin>(cf, x, es, S, sx, sz, corner_of(A, B, Cz), -kscale, a0, a1, a2);
        }
    } else if (f & NF_SOLID) {
        elem_contrib<Tc, Tin, 0>(lv, cf, kscale, x, n, S, sx, sz, a0, a1, a2);
        elem_contrib<Tc, Tin, 1>(lv, cf, kscale, x, n, S, sx, sz, a0, a1, a2);
        elem_contrib<Tc, Tin, 2>(lv, cf, kscale, x, n, S, sx, sz, a0, a1, a2);
        elem_contrib<Tc, Tin, 3>(lv, cf, kscale, x, n, S, sx, sz, a0, a1, a2);
        elem_contrib<Tc, Tin, 4>(lv, cf, kscale, x, n, S, sx, sz, a0, a1, a2);
        elem_contrib<Tc, Tin, 5>(lv, cf, kscale, x, n, S, sx, sz, a0, a1, a2);
        elem_contrib<Tc, Tin, 6>(lv, cf, kscale, x, n, S, sx, sz, a0, a1, a2);
        elem_contrib<Tc, Tin, 7>(lv, cf, kscale, x, n, S, sx, sz, a0, a1, a2);
    }
    if (f & NF_FIX_X) a0 = 0;
    if (f & NF_FIX_Y) a1 = 0;
    if (f & NF_FIX_Z) a2 = 0;
    chk::st(y, n, 3 * S, chk::MV_Y, a0);
    chk::st(y, n + S, 3 * S, chk::MV_Y, a1);
    chk::st(y, n + 2 * S, 3 * S, chk::MV_Y, a2);
}

static dim3 node_grid(const Grid& g, dim3 blk) {
    return dim3((g.ny + 1 + blk.x - 1) / blk.x, (g.nx + 1 + blk.y - 1) / blk.y, g.nz + 1);
}

template <typename Tc, typename Tin, typename Tout>
void launch_matvec(Ctx& c, const LevelView<Tc>& lv, const MatCoef<Tc>& cf, const Tin* x, Tout* y, double kscale) {
    dim3 blk(32, 4, 1);
    k_matvec<Tc, Tin, Tout><<<node_grid(lv.g, blk), blk, 0, c.stream>>>(lv, cf, (Tc)kscale, x, y);
    GMGS_LAUNCHED(c);
}
template void launch_matvec<double, double, double>(Ctx&, const LevelView<double>&, const MatCoef<double>&,
                                                    const double*, double*, double);
template void launch_matvec<float, float, float>(Ctx&, const LevelView<float>&, const MatCoef<float>&, const float*,
                                                 float*, double);
template void launch_matvec<float, double, float>(Ctx&, const LevelView<float>&, const MatCoef<float>&,
                                                  const double*, float*, double);

// ---------------------------------------------------------------------------
// elementwise helpers
// ---------------------------------------------------------------------------
template <typename Tr, typename Td, typename Tx>
__global__ void k_jacobi_dx(int64_t S, const Td* __restrict__ d, double omega, const Tr* __restrict__ r,
                            Tx* __restrict__ dx) {
    using Tc = Td;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 3 * S;
         i += (int64_t)gridDim.x * blockDim.x) {
        const Tc dd = d[i];
        dx[i] = dd != (Tc)0 ? (Tx)(((Tc)omega * (Tc)r[i]) / dd) : (Tx)0;
    }
}

static int ew_blocks(const Ctx& c, int64_t n) {
    int64_t b = (n + 255) / 256;
    int64_t cap = (int64_t)c.num_sms * 16;
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

template <typename Tr, typename Td, typename Tx>
void launch_jacobi_dx(Ctx& c, const Grid& g, const Td* diag, double omega, const Tr* r, Tx* dx) {
    k_jacobi_dx<Tr, Td, Tx><<<ew_blocks(c, 3 * g.slots), 256, 0, c.stream>>>(g.slots, diag, omega, r, dx);
    GMGS_LAUNCHED(c);
}
template void launch_jacobi_dx<double, double, double>(Ctx&, const Grid&, const double*, double, const double*, double*);
template void launch_jacobi_dx<float, float, float>(Ctx&, const Grid&, const float*, double, const float*, float*);

template <typename T, typename U>
__global__ void k_add(int64_t n, T* __restrict__ x, const U* __restrict__ dx) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = x[i] + (T)dx[i];
}
template <typename T, typename U>
__global__ void k_sub(int64_t n, T* __restrict__ x, const U* __restrict__ dx) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = x[i] - (T)dx[i];
}
template <typename T, typename U>
__global__ void k_copy(int64_t n, T* __restrict__ x, const U* __restrict__ a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = (T)a[i];
}
template <typename T, typename U>
void launch_add(Ctx& c, int64_t n, T* x, const U* dx) {
    k_add<T, U><<<ew_blocks(c, n), 256, 0, c.stream>>>(n, x, dx);
    GMGS_LAUNCHED(c);
}
template <typename T, typename U>
void launch_sub(Ctx& c, int64_t n, T* x, const U* y) {
    k_sub<T, U><<<ew_blocks(c, n), 256, 0, c.stream>>>(n, x, y);
    GMGS_LAUNCHED(c);
}
template <typename T, typename U>
void launch_copy(Ctx& c, int64_t n, T* x, const U* a) {
    k_copy<T, U><<<ew_blocks(c, n), 256, 0, c.stream>>>(n, x, a);
    GMGS_LAUNCHED(c);
}
template <typename T>
__global__ void k_diff(int64_t n, T* __restrict__ out, const T* __restrict__ a, const T* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = a[i] - b[i];
}
template <typename T>
void launch_diff(Ctx& c, int64_t n, T* out, const T* a, const T* b) {
    k_diff<T><<<ew_blocks(c, n), 256, 0, c.stream>>>(n, out, a, b);
    GMGS_LAUNCHED(c);
}
template void launch_diff<double>(Ctx&, int64_t, double*, const double*, const double*);
template void launch_diff<float>(Ctx&, int64_t, float*, const float*, const float*);
template void launch_add<double, double>(Ctx&, int64_t, double*, const double*);
template void launch_sub<double, double>(Ctx&, int64_t, double*, const double*);
template void launch_sub<double, float>(Ctx&, int64_t, double*, const float*);
template void launch_sub<float, float>(Ctx&, int64_t, float*, const float*);
template void launch_copy<float, double>(Ctx&, int64_t, float*, const double*);
template void launch_copy<double, float>(Ctx&, int64_t, double*, const float*);
template void launch_copy<double, double>(Ctx&, int64_t, double*, const double*);

// ---------------------------------------------------------------------------
// trilinear transfers (RestrictResidual.m, InterpolationDeviation.m)
//
// With zero values on non-solid fine nodes, the reference's restriction
// (divide by the multiplicity, gather 27 nodes per non-empty coarse element,
// weight by RI, scatter to 8 corners) equals sum_k w(k - 2C) r_f(k) over the
// 27 fine nodes around coarse node C, w = prod(1 - |d|/2); its interpolation
// equals the trilinear interpolant restricted to solid fine nodes.
// ---------------------------------------------------------------------------
// one line of the restriction stencil, (w/2 a + b) + w/2 c with w = 1, and one
// weighted accumulation (weight 1 when `centre`, else 1/2); the roundings are
// explicit so that every kernel summing in this order gives the same bits
__device__ __forceinline__ float restrict_line(float a, float b, float c) {
    return __fmaf_rn(0.5f, c, __fmaf_rn(0.5f, a, b));
}
__device__ __forceinline__ double restrict_line(double a, double b, double c) {
    return __fma_rn(0.5, c, __fma_rn(0.5, a, b));
}
__device__ __forceinline__ float restrict_acc(float acc, float v, bool centre) {
    return centre ? __fadd_rn(acc, v) : __fmaf_rn(0.5f, v, acc);
}
__device__ __forceinline__ double restrict_acc(double acc, double v, bool centre) {
    return centre ? __dadd_rn(acc, v) : __fma_rn(0.5, v, acc);
}

template <typename T>
__global__ void k_restrict(Grid gf, Grid gc, const uint8_t* __restrict__ nflag_c, const T* __restrict__ rf,
                           T* __restrict__ rc) {
    const int Iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int Ix = blockIdx.y * blockDim.y + threadIdx.y;
    const int Iz = blockIdx.z;
    if (Iy > gc.ny || Ix > gc.nx) return;
    const int64_t cs = gc.slot(Iy, Ix, Iz);
    const int64_t Sf = gf.slots, Sc = gc.slots, sx = gf.sx(), sz = gf.sz();
    constexpr int R = chk::RESTRICT;
    if (!(chk::ld(nflag_c, cs, Sc, R) & NF_SOLID)) {
        chk::st(rc, cs, 3 * Sc, R, 0);
        chk::st(rc, cs + Sc, 3 * Sc, R, 0);
        chk::st(rc, cs + 2 * Sc, 3 * Sc, R, 0);
        return;
    }
    const int64_t f0 = gf.slot(2 * Iy, 2 * Ix, 2 * Iz);
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
        T accz = 0;
#pragma unroll
        for (int c = -1; c <= 1; ++c) {
            T accx = 0;
#pragma unroll
            for (int b = -1; b <= 1; ++b) {
                const int64_t s = comp * Sf + f0 + b * sx + c * sz;
                const T line = restrict_line(chk::ld(rf, s - 1, 3 * Sf, R), chk::ld(rf, s, 3 * Sf, R),
                                             chk::ld(rf, s + 1, 3 * Sf, R));
                accx = restrict_acc(accx, line, b == 0);
            }
            accz = restrict_acc(accz, accx, c == 0);
        }
        chk::st(rc, cs + comp * Sc, 3 * Sc, R, accz);
    }
}

template <typename T>
void launch_restrict(Ctx& c, const Grid& gf, const Grid& gc, const uint8_t* nflag_c, const T* rf, T* rc) {
    dim3 blk(32, 4, 1);
    k_restrict<T><<<node_grid(gc, blk), blk, 0, c.stream>>>(gf, gc, nflag_c, rf, rc);
    GMGS_LAUNCHED(c);
}
template void launch_restrict<double>(Ctx&, const Grid&, const Grid&, const uint8_t*, const double*, double*);
template void launch_restrict<float>(Ctx&, const Grid&, const Grid&, const uint8_t*, const float*, float*);

template <typename T>
__global__ void k_prolong_post(Grid gf, Grid gc, const uint8_t* __restrict__ nflag_f, const T* __restrict__ d,
                               T omega, const T* __restrict__ xc, const T* __restrict__ dx,
                               const T* __restrict__ rp, T* __restrict__ xf, int zero_fixed) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y * blockDim.y + threadIdx.y;
    const int iz = blockIdx.z;
    if (iy > gf.ny || ix > gf.nx) return;
    const int64_t fs = gf.slot(iy, ix, iz);
    const int64_t Sf = gf.slots, Sc = gc.slots;
    constexpr int P = chk::PROLONG;
    const uint8_t fl = chk::ld(nflag_f, fs, Sf, P);
    if (!(fl & NF_SOLID)) {
        chk::st(xf, fs, 3 * Sf, P, 0);
        chk::st(xf, fs + Sf, 3 * Sf, P, 0);
        chk::st(xf, fs + 2 * Sf, 3 * Sf, P, 0);
        return;
    }
    const int Iy = iy >> 1, Ix = ix >> 1, Iz = iz >> 1;
    const int oy = iy & 1, ox = ix & 1, oz = iz & 1;
    const int64_t c0 = gc.slot(Iy, Ix, Iz);
    const int64_t csx = gc.sx(), csz = gc.sz();
    const T wy = oy ? (T)0.5 : (T)1, wx = ox ? (T)0.5 : (T)1, wz = oz ? (T)0.5 : (T)1;
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
        T v = 0;
        for (int c = 0; c <= oz; ++c)
            for (int b = 0; b <= ox; ++b)
                for (int a = 0; a <= oy; ++a)
                    v += wy * wx * wz * chk::ld(xc, comp * Sc + c0 + a + b * csx + c * csz, 3 * Sc, P);
        const int64_t i = fs + comp * Sf;
        const T dd = chk::ld(d, i, 3 * Sf, P);
        T out = (chk::ld(dx, i, 3 * Sf, P) + v) + (dd != (T)0 ? (omega * chk::ld(rp, i, 3 * Sf, P)) / dd : (T)0);
        if (zero_fixed && (fl & (NF_FIX_X << comp))) out = 0;
        chk::st(xf, i, 3 * Sf, P, out);
    }
}

template <typename T>
void launch_prolong_post(Ctx& c, const Grid& gf, const Grid& gc, const uint8_t* nflag_f, const T* diag_f,
                         double omega, const T* xc, const T* dx, const T* rp, T* xf, bool zero_fixed) {
    dim3 blk(32, 4, 1);
    k_prolong_post<T><<<node_grid(gf, blk), blk, 0, c.stream>>>(gf, gc, nflag_f, diag_f, (T)omega, xc, dx, rp, xf,
                                                                 zero_fixed ? 1 : 0);
    GMGS_LAUNCHED(c);
}
template void launch_prolong_post<double>(Ctx&, const Grid&, const Grid&, const uint8_t*, const double*, double,
                                          const double*, const double*, const double*, double*, bool);
template void launch_prolong_post<float>(Ctx&, const Grid&, const Grid&, const uint8_t*, const float*, double,
                                         const float*, const float*, const float*, float*, bool);

// ---------------------------------------------------------------------------
// deterministic dot product: fixed grid-stride partition, fixed-order block
// reduction, and the last block to finish sums the partials in index order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    v = 0;
    if (w == 0) {
        v = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;   // valid in thread 0
}

template <typename Ta, typename Tb>
__global__ void __launch_bounds__(256) k_dot(int64_t n, const Ta* __restrict__ a, const Tb* __restrict__ b,
                                             double* __restrict__ partials, unsigned int* ticket,
                                             double* __restrict__ out) {
    __shared__ double sh[32];
    __shared__ bool last;
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += (double)a[i] * (double)b[i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = s;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) {
        __threadfence();
        double t = 0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) t += ((volatile double*)partials)[i];
        t = block_sum(t, sh);
        if (threadIdx.x == 0) {
            *out = t;
            *ticket = 0;
        }
    }
}

template <typename Ta, typename Tb>
void launch_dot(Ctx& c, const DotScratch& s, int64_t n, const Ta* a, const Tb* b, double* out) {
    k_dot<Ta, Tb><<<s.blocks, 256, 0, c.stream>>>(n, a, b, s.partials, s.ticket, out);
    GMGS_LAUNCHED(c);
}
template void launch_dot<double, double>(Ctx&, const DotScratch&, int64_t, const double*, const double*, double*);
template void launch_dot<double, float>(Ctx&, const DotScratch&, int64_t, const double*, const float*, double*);

// ---------------------------------------------------------------------------
// CG updates (CG_solver.m:23-33).  scal layout: [0],[1] r.z of even/odd
// iterations, [2] p.q, [3] r.r, [4] b.b
// ---------------------------------------------------------------------------
template <typename Tz>
__global__ void k_p_update(int64_t n, const Tz* __restrict__ z, double* __restrict__ p,
                           const double* __restrict__ scal, int cur, int first) {
    const double beta = first ? 0.0 : scal[cur] / scal[cur ^ 1];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = first ? (double)z[i] : (double)z[i] + beta * p[i];
}
template <typename Tz>
void launch_p_update(Ctx& c, int64_t n, const Tz* z, double* p, const double* scal, int cur_first) {
    const int cur = cur_first & 1, first = cur_first >> 1;
    k_p_update<Tz><<<ew_blocks(c, n), 256, 0, c.stream>>>(n, z, p, scal, cur, first);
    GMGS_LAUNCHED(c);
}
template void launch_p_update<double>(Ctx&, int64_t, const double*, double*, const double*, int);
template void launch_p_update<float>(Ctx&, int64_t, const float*, double*, const double*, int);

template <typename Tq>
__global__ void k_xr_update(int64_t n, double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                            const Tq* __restrict__ q, const double* __restrict__ scal, int cur) {
    const double alpha = scal[cur] / scal[2];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = x[i] + alpha * p[i];
        r[i] = r[i] - alpha * (double)q[i];
    }
}
template <typename Tq>
void launch_xr_update(Ctx& c, int64_t n, double* x, double* r, const double* p, const Tq* q, const double* scal,
                      int cur) {
    k_xr_update<Tq><<<ew_blocks(c, n), 256, 0, c.stream>>>(n, x, r, p, q, scal, cur);
    GMGS_LAUNCHED(c);
}
template void launch_xr_update<double>(Ctx&, int64_t, double*, double*, const double*, const double*, const double*, int);
template void launch_xr_update<float>(Ctx&, int64_t, double*, double*, const double*, const float*, const double*, int);

// ---------------------------------------------------------------------------
// coarsest level: free-DOF gather, dense GEMV with K^-1, scatter
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_gather(int64_t n, const int32_t* __restrict__ idx, const T* __restrict__ src,
                         double* __restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (double)src[idx[i]];
}
template <typename T>
__global__ void k_scatter(int64_t n, const int32_t* __restrict__ idx, const double* __restrict__ src,
                          T* __restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[idx[i]] = (T)src[i];
}
template <typename T>
void launch_gather(Ctx& c, int64_t n, const int32_t* idx, const T* src, double* dst) {
    k_gather<T><<<ew_blocks(c, n), 256, 0, c.stream>>>(n, idx, src, dst);
    GMGS_LAUNCHED(c);
}
template <typename T>
void launch_scatter(Ctx& c, int64_t n, const int32_t* idx, const double* src, T* dst) {
    k_scatter<T><<<ew_blocks(c, n), 256, 0, c.stream>>>(n, idx, src, dst);
    GMGS_LAUNCHED(c);
}
template void launch_gather<double>(Ctx&, int64_t, const int32_t*, const double*, double*);
template void launch_gather<float>(Ctx&, int64_t, const int32_t*, const float*, double*);
template void launch_scatter<double>(Ctx&, int64_t, const int32_t*, const double*, double*);
template void launch_scatter<float>(Ctx&, int64_t, const int32_t*, const double*, float*);

// ---------------------------------------------------------------------------
// compact interleaved <-> dense planes
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_c2d(int64_t nn, int64_t S, const int32_t* __restrict__ ns, const double* __restrict__ src,
                      T* __restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = ns[i];
        dst[s] = (T)src[3 * i];
        dst[s + S] = (T)src[3 * i + 1];
        dst[s + 2 * S] = (T)src[3 * i + 2];
    }
}
template <typename T>
__global__ void k_d2c(int64_t nn, int64_t S, const int32_t* __restrict__ ns, const T* __restrict__ src,
                      double* __restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = ns[i];
        dst[3 * i] = (double)src[s];
        dst[3 * i + 1] = (double)src[s + S];
        dst[3 * i + 2] = (double)src[s + 2 * S];
    }
}
template <typename T>
void launch_compact_to_dense(Ctx& c, int64_t nn, int64_t S, const int32_t* ns, const double* src, T* dst) {
    k_c2d<T><<<ew_blocks(c, nn), 256, 0, c.stream>>>(nn, S, ns, src, dst);
    GMGS_LAUNCHED(c);
}
template <typename T>
void launch_dense_to_compact(Ctx& c, int64_t nn, int64_t S, const int32_t* ns, const T* src, double* dst) {
    k_d2c<T><<<ew_blocks(c, nn), 256, 0, c.stream>>>(nn, S, ns, src, dst);
    GMGS_LAUNCHED(c);
}
template void launch_compact_to_dense<double>(Ctx&, int64_t, int64_t, const int32_t*, const double*, double*);
template void launch_compact_to_dense<float>(Ctx&, int64_t, int64_t, const int32_t*, const double*, float*);
template void launch_dense_to_compact<double>(Ctx&, int64_t, int64_t, const int32_t*, const double*, double*);
template void launch_dense_to_compact<float>(Ctx&, int64_t, int64_t, const int32_t*, const float*, double*);

}  // namespace gmgs
