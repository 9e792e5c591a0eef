// Coarsest-level direct solve (SetupSolver.m:257-259, Vcycle.m:22-23): the
// reference factors the assembled free-DOF matrix with a sparse Cholesky and
// applies two triangular solves per V-cycle.  Here the free DOFs are numbered
// node by node in slot order, so the matrix is banded; with blocks of order
// B >= the half bandwidth it is block tridiagonal,
//     A = tridiag(A_(i,i-1), A_ii, A_(i,i-1)^T),   i = 0..nb-1.
// It is factored from both ends towards a middle block k ("twisted" block
// LDL^T): from the top
//     S_0 = A_00,  G_i = A_(i,i-1) S_(i-1)^-1,  S_i = A_ii - G_i A_(i,i-1)^T   (i < k)
// from the bottom
//     T_(nb-1) = A_(nb-1,nb-1),  H_i = A_(i+1,i)^T T_(i+1)^-1,
//     T_i = A_ii - H_i A_(i+1,i)                                             (i > k)
// and in the middle M = A_kk - G_k A_(k,k-1)^T - H_k A_(k+1,k).  A x = r is
//     c_i = r_i - G_i c_(i-1) (i = 1..k-1),  c_i = r_i - H_i c_(i+1) (i = nb-2..k+1)
//     c_k = r_k - G_k c_(k-1) - H_k c_(k+1)
//     x_i = D_i^-1 c_i for every block (D = S, T or M)
//     x_i -= G_(i+1)^T x_(i+1) (i = k-1..0),  x_i -= H_(i-1)^T x_(i-1) (i = k+1..nb-1)
// so both sequential sweeps run as two independent chains of about nb/2
// steps, and the two halves of the factorisation run on two streams.  The
// factors take 2 nb B^2 doubles (the D_i^-1 and the couplings G_i / H_i)
// instead of the n^2 of a dense inverse factor.  Each D_i^-1 comes from a
// recursive blocked Cholesky that also forms L^-1 (no pivoting: every D_i is
// SPD), then D^-1 = L^-T L^-1.
//
// Everything runs in FP64 in this file's own kernels, launched in stream
// order: a tiled DGEMM with triangle-aware k-ranges, a one-CTA Cholesky +
// inverse of 32 x 32 diagonal tiles, and block matrix-vector products whose
// last CTA per output block (arrival ticket, no spinning) sums the
// reduction-tile partial sums in a fixed order.
#include "setup.cuh"

namespace gmgs {

namespace {

constexpr int GT = 16;       // DGEMM output tile (one output per thread)
constexpr int MT = 64;       // block matrix-vector tile

enum : int { TRI_A_LOWER = 1, TRI_A_UPPER = 2, TRI_B_LOWER = 4, TRI_B_UPPER = 8 };

// C = alpha op(A) op(B) + beta C, column-major, m, n, k multiples of 16.
// TRI marks operands known to be triangular so the k-loop skips their zero
// tiles (the skipped products are exact zeros); LOWER_OUT skips output tiles
// strictly above the diagonal (their values are never read).
template <bool TA, bool TB, int TRI, bool LOWER_OUT>
__global__ void __launch_bounds__(256) k_dgemm(int k, double alpha, const double* __restrict__ A, int lda,
                                               const double* __restrict__ B, int ldb, double beta,
                                               double* __restrict__ C, int ldc) {
    const int r0 = blockIdx.x * GT, c0 = blockIdx.y * GT;
    if (LOWER_OUT && r0 + GT <= c0) return;
    __shared__ double As[GT][GT + 1];   // As[l][i] = op(A)(r0 + i, k0 + l)
    __shared__ double Bs[GT][GT + 1];   // Bs[l][j] = op(B)(k0 + l, c0 + j)
    const int tx = threadIdx.x & (GT - 1), ty = threadIdx.x / GT;
    int kb = 0, ke = k;
    if (TRI & TRI_A_LOWER) ke = min(ke, r0 + GT);
    if (TRI & TRI_A_UPPER) kb = max(kb, r0);
    if (TRI & TRI_B_LOWER) kb = max(kb, c0);
    if (TRI & TRI_B_UPPER) ke = min(ke, c0 + GT);
    double acc = 0.0;
    for (int k0 = kb; k0 < ke; k0 += GT) {
        if (!TA) As[ty][tx] = A[(int64_t)(k0 + ty) * lda + r0 + tx];
        else     As[tx][ty] = A[(int64_t)(r0 + ty) * lda + k0 + tx];
        if (!TB) Bs[tx][ty] = B[(int64_t)(c0 + ty) * ldb + k0 + tx];
        else     Bs[ty][tx] = B[(int64_t)(k0 + ty) * ldb + c0 + tx];
        __syncthreads();
#pragma unroll
        for (int l = 0; l < GT; ++l) acc = fma(As[l][tx], Bs[l][ty], acc);
        __syncthreads();
    }
    double* cp = C + (int64_t)(c0 + ty) * ldc + r0 + tx;
    *cp = beta == 0.0 ? alpha * acc : fma(alpha, acc, beta * *cp);
}

enum class Op { N, T };

struct Gemm {
    Op ta = Op::N, tb = Op::N;
    int tri = 0;
    bool lower_out = false;
};

template <bool TA, bool TB, int TRI, bool LO>
void run_gemm(Ctx& c, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
              double beta, double* C, int ldc) {
    const dim3 grid(m / GT, n / GT);
    k_dgemm<TA, TB, TRI, LO><<<grid, GT * GT, 0, c.stream>>>(k, alpha, A, lda, B, ldb, beta, C, ldc);
    GMGS_LAUNCHED(c);
}

// the operand forms the factorisation uses
void gemm(Ctx& c, const Gemm& g, int m, int n, int k, double alpha, const double* A, int lda, const double* B,
          int ldb, double beta, double* C, int ldc) {
    if (m <= 0 || n <= 0) return;
    if (g.ta == Op::N && g.tb == Op::T && g.tri == TRI_B_UPPER && !g.lower_out)
        run_gemm<false, true, TRI_B_UPPER, false>(c, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (g.ta == Op::N && g.tb == Op::T && g.tri == 0 && g.lower_out)
        run_gemm<false, true, 0, true>(c, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (g.ta == Op::N && g.tb == Op::N && g.tri == TRI_B_LOWER && !g.lower_out)
        run_gemm<false, false, TRI_B_LOWER, false>(c, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (g.ta == Op::N && g.tb == Op::N && g.tri == TRI_A_LOWER && !g.lower_out)
        run_gemm<false, false, TRI_A_LOWER, false>(c, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (g.ta == Op::T && g.tb == Op::N && g.tri == (TRI_A_UPPER | TRI_B_LOWER) && !g.lower_out)
        run_gemm<true, false, TRI_A_UPPER | TRI_B_LOWER, false>(c, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (g.ta == Op::N && g.tb == Op::N && g.tri == 0 && !g.lower_out)
        run_gemm<false, false, 0, false>(c, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (g.ta == Op::N && g.tb == Op::N && g.tri == 0 && g.lower_out)
        run_gemm<false, false, 0, true>(c, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else if (g.ta == Op::T && g.tb == Op::N && g.tri == 0 && !g.lower_out)
        run_gemm<true, false, 0, false>(c, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else
        throw Error(GMGS_ERR_CUDA, "internal: unsupported DGEMM form");
}

// Cholesky of a 32 x 32 SPD tile (lower triangle of A, in place) and the
// inverse of its factor into Li (zeros above the diagonal), one column per
// step: the pivot's square root and reciprocal, column j of L, row j of L^-1
// (forward substitution of L X = I carried along: X(j, c) is final once
// scaled by 1/L(j,j)), then the rank-1 updates of the trailing part of A and
// of the rows of X below j.  A pivot that is not positive sets *info and is
// replaced by 1 so the arithmetic stays finite.
__global__ void __launch_bounds__(256) k_chol_inv32(double* __restrict__ A, int lda, double* __restrict__ Li,
                                                    int ldl, int* __restrict__ info) {
    __shared__ double a[32][33];   // a[c][r] = A(r, c), becomes L
    __shared__ double x[32][33];   // x[c][r] = X(r, c), becomes L^-1
    __shared__ double dinv;
    const int t = threadIdx.x;
    for (int e = t; e < 1024; e += 256) {
        const int cc = e >> 5, r = e & 31;
        a[cc][r] = A[(int64_t)cc * lda + r];
        x[cc][r] = r == cc ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int j = 0; j < 32; ++j) {
        if (t == 0) {
            const double d = a[j][j];
            const bool ok = d > 0.0 && d < INFINITY;
            if (!ok) atomicExch(info, 1);
            const double piv = ok ? sqrt(d) : 1.0;
            a[j][j] = piv;
            dinv = 1.0 / piv;
        }
        __syncthreads();
        if (t > j && t < 32) a[j][t] *= dinv;                  // L(t, j)
        if (t >= 32 && t - 32 <= j) x[t - 32][j] *= dinv;      // X(j, c), c <= j
        __syncthreads();
        // only rows r > j change: (31 - j) rows x 32 columns, column cc of row r
        // of A (j < cc <= r) or of X (cc <= j); the same update per element as a
        // full sweep, in the same column order
        for (int e = t; e < 32 * (31 - j); e += 256) {
            const int r = j + 1 + (e >> 5), cc = e & 31;
            if (cc > j) {
                if (r >= cc) a[cc][r] = fma(-a[j][r], a[j][cc], a[cc][r]);
            } else {
                x[cc][r] = fma(-a[j][r], x[cc][j], x[cc][r]);
            }
        }
        __syncthreads();
    }
    for (int e = t; e < 1024; e += 256) {
        const int cc = e >> 5, r = e & 31;
        if (r >= cc) A[(int64_t)cc * lda + r] = a[cc][r];
        Li[(int64_t)cc * ldl + r] = x[cc][r];
    }
}

// L (in place of the lower triangle of A) and L^-1 (into Li, whose part above
// the diagonal must be zero on entry) of an n x n SPD matrix, n a multiple of
// 32, by halves:  L11 = chol(A11), L21 = A21 L11^-T, L22 = chol(A22 - L21 L21^T),
// L^-1_21 = -L22^-1 L21 L11^-1.  T: scratch of at least n * n / 2 doubles.
void chol_inv(Ctx& c, double* A, double* Li, int n, int ld, double* T, int* info) {
    if (n == 32) {
        k_chol_inv32<<<1, 256, 0, c.stream>>>(A, ld, Li, ld, info);
        GMGS_LAUNCHED(c);
        return;
    }
    const int n1 = 32 * ((n / 32) / 2), n2 = n - n1;
    double* A21 = A + n1;
    double* A22 = A + (int64_t)n1 * ld + n1;
    const double* Li11 = Li;
    double* Li21 = Li + n1;
    double* Li22 = Li + (int64_t)n1 * ld + n1;
    chol_inv(c, A, Li, n1, ld, T, info);
    gemm(c, {Op::N, Op::T, TRI_B_UPPER, false}, n2, n1, n1, 1.0, A21, ld, Li11, ld, 0.0, T, n2);   // L21
    GMGS_CUDA(cudaMemcpy2DAsync(A21, (size_t)ld * sizeof(double), T, (size_t)n2 * sizeof(double),
                                (size_t)n2 * sizeof(double), n1, cudaMemcpyDeviceToDevice, c.stream));
    gemm(c, {Op::N, Op::T, 0, true}, n2, n2, n1, -1.0, A21, ld, A21, ld, 1.0, A22, ld);         // A22 - L21 L21^T
    chol_inv(c, A22, Li22, n2, ld, T, info);
    gemm(c, {Op::N, Op::N, TRI_B_LOWER, false}, n2, n1, n1, 1.0, A21, ld, Li11, ld, 0.0, T, n2);   // L21 L11^-1
    gemm(c, {Op::N, Op::N, TRI_A_LOWER, false}, n2, n1, n2, -1.0, Li22, ld, T, n2, 0.0, Li21, ld);
}

// one 64 x 64 tile of op(M) times v: the tile into shared memory, 64 partial
// sums (4 threads per output, 16 terms each, fixed order) returned in the
// threads with (t & 3) == 0
__device__ __forceinline__ double tile_mv(int Bn, const double* __restrict__ M, bool trans, int r0, int c0,
                                          const double* v, double (*tile)[MT + 1], double* vs, bool wait_first) {
    const int t = threadIdx.x;
    constexpr int PER = MT * MT / 256;
    double reg[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int e = t + j * 256;
        reg[j] = M[(int64_t)(c0 + e / MT) * Bn + r0 + e % MT];
    }
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int e = t + j * 256;
        tile[e / MT][e % MT] = reg[j];
    }
    if (wait_first) asm volatile("griddepcontrol.wait;" ::: "memory");
    if (t < MT) vs[t] = v[(trans ? r0 : c0) + t];
    __syncthreads();
    const int o = t >> 2, q = t & 3;
    double s = 0.0;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        const int w = q * 16 + u;
        s = fma(trans ? tile[o][w] : tile[w][o], vs[w], s);
    }
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    return s;
}

// Partial sums of one output block are stored, and the last CTA of that
// output block to arrive adds them up in reduction-tile order:
// y[i] = base[i] - sum (or the sum alone when base is null).
__device__ __forceinline__ void finish_partials(int Bn, int nred, int rt, int out0, double s, double* partial,
                                                unsigned int* ticket, const double* base, double* y) {
    __shared__ bool last;
    const int t = threadIdx.x;
    if ((t & 3) == 0) partial[(int64_t)rt * Bn + out0 + (t >> 2)] = s;
    __threadfence();
    __syncthreads();
    if (t == 0) last = atomicAdd(ticket, 1u) == (unsigned)(nred * (Bn / MT) - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int i = t; i < Bn; i += 256) {
        double acc = 0.0;
        int k = 0;
        for (; k + 8 <= nred; k += 8) {
            double p[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) p[j] = __ldcg(partial + (int64_t)(k + j) * Bn + i);
#pragma unroll
            for (int j = 0; j < 8; ++j) acc += p[j];
        }
        for (; k < nred; ++k) acc += __ldcg(partial + (int64_t)k * Bn + i);
        y[i] = base ? base[i] - acc : acc;
    }
    if (t == 0) *ticket = 0;
}

// y_b = M_b v_b for the blocks b of the grid's z dimension (M_b: Bn x Bn,
// column-major, stride sM; vectors stride Bn)
__global__ void __launch_bounds__(256) k_blk_mv(int Bn, const double* __restrict__ M, int64_t sM, const double* v,
                                                double* y, double* partial, unsigned int* ticket) {
    __shared__ double tile[MT][MT + 1];
    __shared__ double vs[MT];
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int b = blockIdx.z, ntiles = Bn / MT;
    const double s = tile_mv(Bn, M + b * sM, false, blockIdx.x * MT, blockIdx.y * MT, v + (int64_t)b * Bn, tile, vs,
                             true);
    finish_partials(Bn, ntiles, blockIdx.y, blockIdx.x * MT, s, partial + (int64_t)b * ntiles * Bn, ticket + b,
                    nullptr, y + (int64_t)b * Bn);
}

// up to two independent jobs (grid z), each y = base - sum_s op(M_s) v_s over
// one or two segments s; grid y runs over (segment, reduction tile)
struct StepJob {
    const double* M[2];
    const double* v[2];
    int trans[2];
    const double* base;
    double* y;
};
struct StepJobs {
    StepJob j[2];
    int nseg;
};

__global__ void __launch_bounds__(256) k_blk_step(int Bn, const __grid_constant__ StepJobs jobs, double* partial,
                                                  unsigned int* ticket) {
    __shared__ double tile[MT][MT + 1];
    __shared__ double vs[MT];
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const StepJob& J = jobs.j[blockIdx.z];
    const int ntiles = Bn / MT;
    const int seg = blockIdx.y / ntiles, red = blockIdx.y % ntiles;
    const bool tr = J.trans[seg] != 0;
    const int r0 = (tr ? red : blockIdx.x) * MT, c0 = (tr ? blockIdx.x : red) * MT;
    const double s = tile_mv(Bn, J.M[seg], tr, r0, c0, J.v[seg], tile, vs, true);
    const int nred = jobs.nseg * ntiles;
    finish_partials(Bn, nred, blockIdx.y, blockIdx.x * MT, s, partial + (int64_t)blockIdx.z * nred * Bn,
                    ticket + blockIdx.z, J.base, J.y);
}

// launched as a programmatic dependent of the previous kernel in the stream:
// its CTAs load their matrix tiles while that kernel finishes, then wait
// (griddepcontrol.wait, the hardware grid dependency) before they read the
// vector it writes and touch the shared partial sums and arrival counters
void launch_step(Ctx& c, int B, const StepJobs& jobs, int njobs, double* part, unsigned int* tk) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(B / MT, jobs.nseg * (B / MT), njobs);
    cfg.blockDim = dim3(256, 1, 1);
    cfg.stream = c.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GMGS_CUDA(cudaLaunchKernelEx(&cfg, k_blk_step, B, jobs, part, tk));
    GMGS_LAUNCHED(c);
}

// D^-1 of the SPD block D (in place): Cholesky + inverse factor, L^-T L^-1
void inv_spd(Ctx& c, double* D, int B, double* li, double* t, int* info) {
    const int64_t B2 = (int64_t)B * B;
    GMGS_CUDA(cudaMemsetAsync(li, 0, B2 * sizeof(double), c.stream));
    chol_inv(c, D, li, B, B, t, info);
    gemm(c, {Op::T, Op::N, TRI_A_UPPER | TRI_B_LOWER, false}, B, B, B, 1.0, li, B, li, B, 0.0, D, B);
}

}  // namespace

int coarse_block_order(int n, int half_bandwidth) {
    const int want = std::max(half_bandwidth, 1);
    return std::max(MT, (std::min(want, n) + MT - 1) / MT * MT);
}

int coarse_middle(int nb) { return (nb - 1) / 2; }

void factor_coarse(Ctx& c, CoarseBlocks& cb, const std::function<void()>& overlap) {
    const int B = cb.B, nb = cb.nb, k = coarse_middle(nb);
    const int64_t B2 = (int64_t)B * B;
    double* D = cb.sinv.as<double>();   // A_ii on entry
    double* E = cb.g.as<double>();      // E_i = A_(i,i-1) on entry (i >= 1)
    auto Db = [&](int i) { return D + i * B2; };
    auto Eb = [&](int i) { return E + i * B2; };
    // the two halves run on their own streams, forked from and joined to c.stream
    cudaStream_t st[2] = {nullptr, nullptr};
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    struct Res {
        cudaStream_t* s; cudaEvent_t* e;
        ~Res() {
            for (int i = 0; i < 2; ++i) if (s[i]) cudaStreamDestroy(s[i]);
            for (int i = 0; i < 3; ++i) if (e[i]) cudaEventDestroy(e[i]);
        }
    } res{st, ev};
    for (int i = 0; i < 2; ++i) GMGS_CUDA(cudaStreamCreateWithFlags(&st[i], cudaStreamNonBlocking));
    for (int i = 0; i < 3; ++i) GMGS_CUDA(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
    DevBuf info = dalloc(2 * sizeof(int));
    GMGS_CUDA(cudaMemsetAsync(info.p, 0, 2 * sizeof(int), c.stream));
    DevBuf li[2], tt[2], t2[2];
    for (int h = 0; h < 2; ++h) {
        li[h] = dalloc(B2 * sizeof(double));
        tt[h] = dalloc(B2 * sizeof(double));
        t2[h] = dalloc(B2 * sizeof(double));
    }
    GMGS_CUDA(cudaEventRecord(ev[0], c.stream));
    Ctx half[2] = {c, c};
    for (int h = 0; h < 2; ++h) {
        half[h].stream = st[h];
        half[h].prof = false;
        half[h].trace = false;
        half[h].launches = 0;
        GMGS_CUDA(cudaStreamWaitEvent(st[h], ev[0], 0));
    }
    int* inf = info.as<int>();
    {   // top: S_i^-1 (i < k), G_i (i = 1..k-1), and G_k into t2[0]
        Ctx& h = half[0];
        for (int i = 0; i < k; ++i) {
            if (i > 0) {
                gemm(h, {Op::N, Op::N, 0, false}, B, B, B, 1.0, Eb(i), B, Db(i - 1), B, 0.0, t2[0].as<double>(), B);
                gemm(h, {Op::N, Op::T, 0, true}, B, B, B, -1.0, t2[0].as<double>(), B, Eb(i), B, 1.0, Db(i), B);
                GMGS_CUDA(cudaMemcpyAsync(Eb(i), t2[0].p, B2 * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
            }
            inv_spd(h, Db(i), B, li[0].as<double>(), tt[0].as<double>(), inf);
        }
        if (k >= 1)
            gemm(h, {Op::N, Op::N, 0, false}, B, B, B, 1.0, Eb(k), B, Db(k - 1), B, 0.0, t2[0].as<double>(), B);
    }
    {   // bottom: T_i^-1 (i > k), H_i = E_(i+1) (i = k+1..nb-2), and H_k into t2[1]
        Ctx& h = half[1];
        for (int i = nb - 1; i > k; --i) {
            if (i < nb - 1) {
                gemm(h, {Op::T, Op::N, 0, false}, B, B, B, 1.0, Eb(i + 1), B, Db(i + 1), B, 0.0, t2[1].as<double>(), B);
                gemm(h, {Op::N, Op::N, 0, true}, B, B, B, -1.0, t2[1].as<double>(), B, Eb(i + 1), B, 1.0, Db(i), B);
                GMGS_CUDA(cudaMemcpyAsync(Eb(i + 1), t2[1].p, B2 * sizeof(double), cudaMemcpyDeviceToDevice, h.stream));
            }
            inv_spd(h, Db(i), B, li[1].as<double>(), tt[1].as<double>(), inf + 1);
        }
        if (k + 1 <= nb - 1)
            gemm(h, {Op::T, Op::N, 0, false}, B, B, B, 1.0, Eb(k + 1), B, Db(k + 1), B, 0.0, t2[1].as<double>(), B);
    }
    if (overlap) overlap();
    c.trace_point("bc: work buffers (beside the factorisation)");
    for (int h = 0; h < 2; ++h) {
        GMGS_CUDA(cudaEventRecord(ev[1 + h], st[h]));
        GMGS_CUDA(cudaStreamWaitEvent(c.stream, ev[1 + h], 0));
        c.launches += half[h].launches;
    }
    // the middle block: M = A_kk - G_k A_(k,k-1)^T - H_k A_(k+1,k), then M^-1
    if (k >= 1) {
        gemm(c, {Op::N, Op::T, 0, true}, B, B, B, -1.0, t2[0].as<double>(), B, Eb(k), B, 1.0, Db(k), B);
        GMGS_CUDA(cudaMemcpyAsync(Eb(k), t2[0].p, B2 * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    }
    if (k + 1 <= nb - 1) {
        gemm(c, {Op::N, Op::N, 0, true}, B, B, B, -1.0, t2[1].as<double>(), B, Eb(k + 1), B, 1.0, Db(k), B);
        GMGS_CUDA(cudaMemcpyAsync(Eb(k + 1), t2[1].p, B2 * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    }
    inv_spd(c, Db(k), B, li[0].as<double>(), tt[0].as<double>(), inf);
    c.trace_point("bc: coarsest block LDL^T");
    int h_info[2] = {0, 0};
    GMGS_CUDA(cudaMemcpyAsync(h_info, info.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    GMGS_CUDA(cudaStreamSynchronize(c.stream));
    if (h_info[0] || h_info[1]) throw Error(GMGS_ERR_NOT_SPD, "coarsest-level matrix is not positive definite");
    const int nslot = std::max(nb, 4);
    cb.partial = dalloc((size_t)nslot * (B / MT) * B * sizeof(double));
    cb.ticket = dalloc((size_t)nslot * sizeof(unsigned int));
    GMGS_CUDA(cudaMemsetAsync(cb.ticket.p, 0, (size_t)nslot * sizeof(unsigned int), c.stream));
    GMGS_CUDA(cudaStreamSynchronize(c.stream));
}

void launch_coarse_solve(Ctx& c, const CoarseBlocks& cb, double* cvec, double* x) {
    const int B = cb.B, nb = cb.nb, k = coarse_middle(nb);
    if (nb <= 0) return;
    const int64_t B2 = (int64_t)B * B;
    const double* D = cb.sinv.as<double>();
    const double* E = cb.g.as<double>();
    double* part = cb.partial.as<double>();
    unsigned int* tk = cb.ticket.as<unsigned int>();
    auto Eb = [&](int i) { return E + i * B2; };
    auto vb = [&](double* v, int i) { return v + (int64_t)i * B; };
    // forward chains, in place on cvec: top i = 1..k-1, bottom i = nb-2..k+1
    const int top_steps = std::max(0, k - 1), bot_steps = std::max(0, nb - 2 - k);
    for (int s = 0; s < std::max(top_steps, bot_steps); ++s) {
        StepJobs J = {};
        J.nseg = 1;
        int nj = 0;
        if (s < top_steps) {
            const int i = 1 + s;
            J.j[nj++] = {{Eb(i), nullptr}, {vb(cvec, i - 1), nullptr}, {0, 0}, vb(cvec, i), vb(cvec, i)};
        }
        if (s < bot_steps) {
            const int i = nb - 2 - s;
            J.j[nj++] = {{Eb(i + 1), nullptr}, {vb(cvec, i + 1), nullptr}, {0, 0}, vb(cvec, i), vb(cvec, i)};
        }
        launch_step(c, B, J, nj, part, tk);
    }
    {   // the middle block's right-hand side
        StepJobs J = {};
        int ns = 0;
        StepJob& m = J.j[0];
        if (k >= 1) { m.M[ns] = Eb(k); m.v[ns] = vb(cvec, k - 1); m.trans[ns] = 0; ++ns; }
        if (k + 1 <= nb - 1) { m.M[ns] = Eb(k + 1); m.v[ns] = vb(cvec, k + 1); m.trans[ns] = 0; ++ns; }
        if (ns > 0) {
            m.base = vb(cvec, k);
            m.y = vb(cvec, k);
            J.nseg = ns;
            launch_step(c, B, J, 1, part, tk);
        }
    }
    // x_i = D_i^-1 c_i for all blocks
    k_blk_mv<<<dim3(B / MT, B / MT, nb), 256, 0, c.stream>>>(B, D, B2, cvec, x, part, tk);
    GMGS_LAUNCHED(c);
    // backward chains, in place on x: top i = k-1..0, bottom i = k+1..nb-1
    const int tb = k, bb = nb - 1 - k;
    for (int s = 0; s < std::max(tb, bb); ++s) {
        StepJobs J = {};
        J.nseg = 1;
        int nj = 0;
        if (s < tb) {
            const int i = k - 1 - s;
            J.j[nj++] = {{Eb(i + 1), nullptr}, {vb(x, i + 1), nullptr}, {1, 0}, vb(x, i), vb(x, i)};
        }
        if (s < bb) {
            const int i = k + 1 + s;
            J.j[nj++] = {{Eb(i), nullptr}, {vb(x, i - 1), nullptr}, {1, 0}, vb(x, i), vb(x, i)};
        }
        launch_step(c, B, J, nj, part, tk);
    }
}

}  // namespace gmgs
