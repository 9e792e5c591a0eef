// V-cycle preconditioner and the outer PCG (src/kernel/Vcycle.m:1-36,
// src/kernel/CG_solver.m:1-56, src/kernel/JacobiSmoother.m:1-10).
//
// The FP64 path runs every vector and operator in double precision.  The
// mixed path keeps x, r, p, the dot products and the coarsest solve in FP64
// and runs the V-cycle (smoothers, transfers, level matvecs) in FP32; the
// CG's own matvecs read FP64 vectors and compute in FP32.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>

#include "setup.cuh"

namespace gmgs {

enum { SC_RZ0 = 0, SC_RZ1 = 1, SC_PQ = 2, SC_RR = 3, SC_BB = 4, SC_TC = 5, SC_N = 8 };   // SC_TC: host copy of the device wait-error flag

static void zalloc(Ctx& c, DevBuf& b, size_t bytes) {
    if (b.bytes < bytes) b = dalloc(bytes);
    GMGS_CUDA(cudaMemsetAsync(b.p, 0, bytes, c.stream));
}

// level-0 matvec with optional event timing; algorithmic bytes: read x and
// write y at every solid node, one mask byte per solid element and node
template <typename Tc, typename Tin, typename Tout>
static void fine_matvec(Model& M, const Tin* x, Tout* y) {
    Level& l0 = M.levels[0];
    const double bytes = (double)l0.n_node * (3.0 * sizeof(Tin) + 3.0 * sizeof(Tout) + 1.0) + (double)l0.n_elem;
    M.ctx.mark(PK_FINE_MATVEC, false);
    launch_matvec<Tc, Tin, Tout>(M.ctx, view<Tc>(l0, M.prm.omega), mat_coef<Tc>(M), x, y, l0.kscale);
    M.ctx.mark(PK_FINE_MATVEC, true, bytes);
}

void alloc_work(Model& M) {
    Ctx& c = M.ctx;
    ++M.gen;   // buffers and operators may move: captured graphs are stale
    const bool mixed = M.prm.precision == GMGS_MIXED;
    const size_t T = mixed ? sizeof(float) : sizeof(double);
    const int L = M.num_levels;
    for (int l = 0; l < L; ++l) {
        Level& lv = M.levels[l];
        const size_t n3 = 3 * (size_t)lv.g.slots;
        if (l > 0) zalloc(c, lv.vr, n3 * T);
        if (l > 0 || !mixed) zalloc(c, lv.vx, n3 * T);
        if (l < L - 1) {
            zalloc(c, lv.vrp, n3 * T);
            if (!mixed) {
                zalloc(c, lv.vdx, n3 * T);
                zalloc(c, lv.vy, n3 * T);
            } else {
                if (lv.wdinv32.bytes < n3 * 4) lv.wdinv32 = dalloc(n3 * 4);
                launch_wdinv(c, (int64_t)n3, lv.diag64.as<double>(), M.prm.omega, lv.wdinv32.as<float>());
                if (lv.emask8.bytes < (size_t)lv.g.slots) lv.emask8 = dalloc(lv.g.slots);
                launch_emask8(c, lv.g, lv.emask.as<uint8_t>(), lv.emask8.as<uint8_t>());
                if (lv.tile_occ.bytes < tile_occ_bytes(lv.g)) lv.tile_occ = dalloc(tile_occ_bytes(lv.g));
                launch_tile_occ(c, lv.g, lv.nflag.as<uint8_t>(), lv.tile_occ.as<uint8_t>());
                if (lv.tc_occ.bytes < tc_tile_occ_bytes(lv.g)) lv.tc_occ = dalloc(tc_tile_occ_bytes(lv.g));
                launch_tc_tile_occ(c, lv.g, lv.nflag.as<uint8_t>(), lv.tc_occ.as<uint8_t>());
            }
        }
    }
    const size_t n3 = 3 * (size_t)M.levels[0].g.slots;
    zalloc(c, M.cg_x, n3 * 8);
    zalloc(c, M.cg_r, n3 * 8);
    if (mixed) {
        zalloc(c, M.cg_r32b, n3 * 4);
        zalloc(c, M.cg_pa, n3 * 4);
        zalloc(c, M.cg_pb, n3 * 4);
        zalloc(c, M.cg_q32, n3 * 4);
        zalloc(c, M.cg_z32, n3 * 4);
        zalloc(c, M.cg_r32, n3 * 4);
    } else {
        zalloc(c, M.cg_p, n3 * 8);
        zalloc(c, M.cg_dx, n3 * 8);
        zalloc(c, M.cg_q64, n3 * 8);
        zalloc(c, M.cg_y64, n3 * 8);
        zalloc(c, M.cg_z64, n3 * 8);
    }
    zalloc(c, M.scal, SC_N * sizeof(double));
    if (mixed) zalloc(c, M.tc_err, sizeof(int));
    M.dot_blocks = M.ctx.num_sms * 4;
    const int maxb = std::max({M.dot_blocks, fine_grid_blocks(M.levels[0].g), up32_grid_blocks(M.levels[0].g)});
    zalloc(c, M.dot_partials, (size_t)maxb * sizeof(double));
    zalloc(c, M.dot_ticket, sizeof(unsigned int));
    if (!M.scal_host) GMGS_CUDA(cudaMallocHost(&M.scal_host, SC_N * sizeof(double)));
    GMGS_CUDA(cudaStreamSynchronize(c.stream));
}

static DotScratch dots(Model& M) {
    return DotScratch{M.dot_partials.as<double>(), M.dot_ticket.as<unsigned int>(), M.dot_blocks};
}

// V-cycle down-sweeps on the tensor cores when the environment sets GMGS_TC=1
static bool tc_enabled() {
    const char* e = std::getenv("GMGS_TC");
    return e && e[0] == '1';
}

// A kernel whose bounded wait ran out (a tensor-core kernel waiting for its
// MMA, or the CG update waiting for its TMA-staged operands) sets the device
// flag; the solve reports it instead of returning a result computed without
// the data it waited for.
static void check_tc(Model& M) {
    if (!M.tc_err.p) return;
    int flag = 0;
    GMGS_CUDA(cudaMemcpyAsync(&flag, M.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, M.ctx.stream));
    GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
    if (flag) {
        GMGS_CUDA(cudaMemsetAsync(M.tc_err.p, 0, sizeof(int), M.ctx.stream));
        throw Error(GMGS_ERR_CUDA, "a kernel's bounded wait for its tensor-core MMA or staged operands timed out");
    }
}

// One V(1,1) cycle, Vcycle.m:1-36: down-sweep Jacobi with residual update and
// restriction, coarsest direct solve, up-sweep prolongation + Jacobi with the
// pre-smoothing residual, fixed DOFs of the finest level zeroed.
template <typename T>
static void vcycle(Model& M, const T* r0, T* z) {
    Ctx& c = M.ctx;
    c.mark(PK_VCYCLE, false);
    const int L = M.num_levels;
    const double om = M.prm.omega;
    for (int l = 0; l < L - 1; ++l) {
        Level& lv = M.levels[l];
        Level& lc = M.levels[l + 1];
        const T* r = l == 0 ? r0 : lv.vr.as<T>();
        const LevelView<T> v = view<T>(lv, om);
        const int64_t n3 = 3 * lv.g.slots;
        launch_jacobi_dx<T, T, T>(c, lv.g, v.diag, om, r, lv.vdx.as<T>());
        if (l == 0) fine_matvec<T, T, T>(M, lv.vdx.as<T>(), lv.vy.as<T>());
        else launch_matvec<T, T, T>(c, v, mat_coef<T>(M), lv.vdx.as<T>(), lv.vy.as<T>(), lv.kscale);
        launch_diff<T>(c, n3, lv.vrp.as<T>(), r, lv.vy.as<T>());
        launch_restrict<T>(c, lv.g, lc.g, lc.nflag.as<uint8_t>(), lv.vrp.as<T>(), lc.vr.as<T>());
    }
    Level& lc = M.levels[L - 1];
    launch_gather<T>(c, M.nfree, M.free_idx.as<int32_t>(), lc.vr.as<T>(), M.cvec_in.as<double>());
    launch_coarse_solve(c, M.cb, M.cvec_in.as<double>(), M.cvec_out.as<double>());
    launch_scatter<T>(c, M.nfree, M.free_idx.as<int32_t>(), M.cvec_out.as<double>(), lc.vx.as<T>());
    for (int l = L - 2; l >= 0; --l) {
        Level& lv = M.levels[l];
        T* out = l == 0 ? z : lv.vx.as<T>();
        const LevelView<T> v = view<T>(lv, om);
        launch_prolong_post<T>(c, lv.g, M.levels[l + 1].g, lv.nflag.as<uint8_t>(), v.diag, om,
                               M.levels[l + 1].vx.as<T>(), lv.vdx.as<T>(), lv.vrp.as<T>(), out, l == 0);
    }
    c.mark(PK_VCYCLE, true);
}

static void vcycle32(Model& M, const float* r32, float* z, bool with_dot, int dot_slot);

void vcycle_apply(Model& M, const double* r, double* z) {
    const int64_t n3 = 3 * M.levels[0].g.slots;
    if (M.prm.precision == GMGS_MIXED) {
        M.use_tc = tc_enabled();
        launch_copy<float, double>(M.ctx, n3, M.cg_r32.as<float>(), r);
        vcycle32(M, M.cg_r32.as<float>(), M.cg_z32.as<float>(), false, 0);
        launch_copy<double, float>(M.ctx, n3, z, M.cg_z32.as<float>());
        check_tc(M);
    } else {
        vcycle<double>(M, r, z);
    }
}

void vcycle_apply_fp64(Model& M, const double* r, double* z) { vcycle_apply(M, r, z); }

void apply_operator_dense(Model& M, int level, const double* x, double* y) {
    Level& lv = M.levels[level];
    launch_matvec<double, double, double>(M.ctx, view<double>(lv, M.prm.omega), M.mc64, x, y, lv.kscale);
}


// ---------------------------------------------------------------------------
// mixed path: FP32 V-cycle on the fused tiled kernels
// ---------------------------------------------------------------------------
static FineLevel fine_level(const Level& lv) {
    FineLevel f;
    f.g = lv.g;
    f.emask = lv.emask.as<uint8_t>();
    f.nflag = lv.nflag.as<uint8_t>();
    f.emask8 = lv.emask8.as<uint8_t>();
    f.etype = lv.etype.as<int32_t>();
    f.Ks = lv.Ks32.as<float>();
    f.nK = lv.Ks32.p ? lv.nK : 0;
    f.escale = lv.escale32.as<float>();
    f.kscale = (float)lv.kscale;
    f.tile_occ = lv.tile_occ.as<uint8_t>();
    return f;
}

template <int MODE>
static void launch_l0(Model& M, const FineLevel& f, const FineArgs& a) {
    launch_fine<MODE>(M.ctx, f, M.coef, a);
}

static DotOut dot_out(Model& M, int slot) {
    DotOut d;
    d.partials = M.dot_partials.as<double>();
    d.ticket = M.dot_ticket.as<unsigned int>();
    d.out = M.scal.as<double>() + slot;
    return d;
}

// z = V(r32); the level-1 up-sweep also accumulates r32 . z into scal[dot_slot]
static void vcycle32(Model& M, const float* r32, float* z, bool with_dot, int dot_slot) {
    Ctx& c = M.ctx;
    const int L = M.num_levels;
    c.mark(PK_VCYCLE, false);
    for (int l = 0; l < L - 1; ++l) {
        Level& lv = M.levels[l];
        Level& lc = M.levels[l + 1];
        FineArgs a;
        a.r32 = l == 0 ? r32 : lv.vr.as<float>();
        a.wdinv = lv.wdinv32.as<float>();
        a.out32 = lv.vrp.as<float>();
        // r, omega/diag, r' per node; element masks
        const double bytes = (double)lv.n_node * 3 * 12 + (double)lv.n_elem;
        if (l == 0) {
            c.mark(PK_FINE_MATVEC, false);
            c.mark(PK_VDOWN0, false);
        }
        if (l == 1) c.mark(PK_COARSE, false);
        const FineLevel fl = fine_level(lv);
        if (M.use_tc && lv.n_perel < lv.n_node) {
            FineLevel ft = fl;
            ft.tile_occ = lv.tc_occ.as<uint8_t>();
            launch_tc_vdown(c, ft, M.tcoef, a.r32, a.wdinv, a.out32, M.tc_err.as<int>());
        } else if (l == 0) {
            launch_l0<FM_VCYCLE_DOWN>(M, fl, a);
        } else if (lv.n_perel < lv.n_node) {
            launch_fine<FM_VCYCLE_DOWN>(c, fl, M.coef, a);
        }
        if (lv.n_perel > 0)
            launch_perel_vdown(c, fl, M.coef, lv.perel_nodes.as<int32_t>(), (int)lv.n_perel, a.r32, a.wdinv,
                               a.out32);
        if (l == 0) {
            c.mark(PK_FINE_MATVEC, true, bytes);
            c.mark(PK_VDOWN0, true, bytes);
        }
        launch_restrict<float>(c, lv.g, lc.g, lc.nflag.as<uint8_t>(), lv.vrp.as<float>(), lc.vr.as<float>());
    }
    if (L == 2) c.mark(PK_COARSE, false);
    Level& lc = M.levels[L - 1];
    launch_gather<float>(c, M.nfree, M.free_idx.as<int32_t>(), lc.vr.as<float>(), M.cvec_in.as<double>());
    launch_coarse_solve(c, M.cb, M.cvec_in.as<double>(), M.cvec_out.as<double>());
    launch_scatter<float>(c, M.nfree, M.free_idx.as<int32_t>(), M.cvec_out.as<double>(), lc.vx.as<float>());
    for (int l = L - 2; l >= 0; --l) {
        Level& lv = M.levels[l];
        const DotOut d = dot_out(M, dot_slot);
        if (l == 0) {
            c.mark(PK_COARSE, true);
            c.mark(PK_UP0, false);
        }
        launch_up32(c, lv.g, M.levels[l + 1].g, lv.nflag.as<uint8_t>(), lv.tile_occ.as<uint8_t>(),
                    lv.wdinv32.as<float>(),
                    l == 0 ? r32 : lv.vr.as<float>(), lv.vrp.as<float>(), M.levels[l + 1].vx.as<float>(),
                    l == 0 ? z : lv.vx.as<float>(), l == 0, (l == 0 && with_dot) ? &d : nullptr);
        if (l == 0) c.mark(PK_UP0, true, (double)lv.n_node * 3 * 20);
    }
    c.mark(PK_VCYCLE, true);
}

static bool graphs_enabled() {
    const char* e = std::getenv("GMGS_GRAPH");
    return e && e[0] && e[0] != '0';
}

void reset_graphs(Model& M) {
    for (auto& g : M.cg_graph) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
    M.cg_graph_x = nullptr;
}

// Capture the iteration body for both parities (its = 2 and 3) without
// running it.  Returns false (nothing captured) when capture or
// instantiation fails; the caller restores its pointer state and launches
// eagerly.
template <class Body>
static bool capture_iteration_graphs(Model& M, Body& body) {
    Ctx& c = M.ctx;
    reset_graphs(M);
    for (int k = 0; k < 2; ++k) {
        const int its = 2 + k;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            reset_graphs(M);
            return false;
        }
        bool ok = true;
        const int64_t l0 = c.launches;
        try {
            body(its);
        } catch (const Error&) {
            ok = false;
        }
        M.cg_graph_kernels[its & 1] = c.launches - l0;   // recorded, not run
        c.launches = l0;
        const cudaError_t e = cudaStreamEndCapture(c.stream, &g);
        cudaGraphExec_t ex = nullptr;
        if (ok && e == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) M.cg_graph[its & 1] = ex;
        else ok = false;
        cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        if (!ok) {
            reset_graphs(M);
            return false;
        }
    }
    return true;
}

static int pcg_mixed(Model& M, const double* b, double* x, int32_t* iters_out, double* relres_out, double* hist) {
    Ctx& c = M.ctx;
    M.use_tc = tc_enabled();
    Level& l0 = M.levels[0];
    const int64_t n3 = 3 * l0.g.slots;
    double* scal = M.scal.as<double>();
    const DotScratch ds = dots(M);
    // double-float state: x = x_hi + x_lo in the two halves of cg_x, r = r32 + r_lo
    // (the high part double-buffered, the low part in the first half of cg_r)
    float* x_hi = M.cg_x.as<float>();
    float* x_lo = x_hi + n3;
    float* r_lo = M.cg_r.as<float>();
    float* r32a = M.cg_r32.as<float>();
    float* r32b = M.cg_r32b.as<float>();
    float* pa = M.cg_pa.as<float>();
    float* pb = M.cg_pb.as<float>();
    float* q = M.cg_q32.as<float>();
    const FineLevel f0 = fine_level(l0);

    launch_dot<double, double>(c, ds, n3, b, b, scal + SC_BB);
    GMGS_CUDA(cudaMemcpyAsync(M.scal_host + SC_BB, scal + SC_BB, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    GMGS_CUDA(cudaMemsetAsync(x_hi, 0, 2 * n3 * sizeof(float), c.stream));
    launch_df_split(c, n3, b, r32a, r_lo);     // r = b - A*0
    GMGS_CUDA(cudaStreamSynchronize(c.stream));
    const double normB = std::sqrt(M.scal_host[SC_BB]);
    if (normB == 0.0) {
        GMGS_CUDA(cudaMemsetAsync(x, 0, n3 * sizeof(double), c.stream));
        GMGS_CUDA(cudaStreamSynchronize(c.stream));
        if (iters_out) *iters_out = 0;
        if (relres_out) *relres_out = 0;
        M.last_iters = 0;
        M.last_relres = 0;
        return GMGS_OK;
    }
    if (!std::isfinite(normB)) throw Error(GMGS_ERR_NONFINITE, "non-finite load vector");
    // algorithmic bytes per node: r (high part read + write, low part rw), q, p, wdinv, x (both parts rw)
    const double jbytes = (double)l0.n_node * 3 * (8 + 8 + 4 + 4 + 4 + 16) + 2.0 * (double)l0.n_node;
    const double pbytes = (double)l0.n_node * 3 * (4 + 4 + 4 + 4) + 2.0 * (double)l0.n_node;

    // Fused kernel: the previous iteration's update (x += alpha p, r -= alpha q,
    // |r|^2 for its convergence test) followed by the next iteration's Jacobi
    // step (x += dx, r -= A dx).  When the solve stops, the last dx (which
    // belongs to an iteration that does not run) is removed from x again.
    auto update_jacobi = [&](int first, int cur) {
        FineArgs a;
        a.r32 = r32a;
        a.r_lo = r_lo;
        a.q32 = q;
        a.pold = pa;
        a.wdinv = l0.wdinv32.as<float>();
        a.x_hi = x_hi;
        a.x_lo = x_lo;
        a.r32out = r32b;
        a.scal = scal;
        a.cur = cur;
        a.first = first;
        a.dot = dot_out(M, SC_RR);
        a.err = M.tc_err.as<int>();
        c.mark(PK_FINE_MATVEC, false);
        c.mark(PK_UPDATE_JACOBI, false);
        launch_l0<FM_CG_UPDATE_JACOBI>(M, f0, a);
        c.mark(PK_FINE_MATVEC, true, jbytes);
        c.mark(PK_UPDATE_JACOBI, true, jbytes);
        std::swap(r32a, r32b);
    };

    // one PCG iteration: V-cycle, direction + A p, update + next Jacobi step;
    // the double buffers swap, so the launches repeat with period two
    auto body = [&](int its) {
        const int cur = its & 1;
        vcycle32(M, r32a, M.cg_z32.as<float>(), true, cur);     // z2 = PtV(r1), r1'z2   (CG_solver.m:21,26)
        {   // p2 = z2 + beta p1; q = A p2; p2'q   (CG_solver.m:23-31)
            FineArgs a;
            a.z32 = M.cg_z32.as<float>();
            a.pold = pa;
            a.pout = pb;
            a.scal = scal;
            a.cur = cur;
            a.first = its == 1;
            a.out32 = q;
            a.dot = dot_out(M, SC_PQ);
            c.mark(PK_FINE_MATVEC, false);
            c.mark(PK_DIRECTION, false);
            launch_l0<FM_CG_DIRECTION>(M, f0, a);
            c.mark(PK_FINE_MATVEC, true, pbytes);
            c.mark(PK_DIRECTION, true, pbytes);
            std::swap(pa, pb);
        }
        update_jacobi(0, cur);     // x += alpha p2; r2 = r1 - alpha q; |r2|; next Jacobi step
    };
    // With GMGS_GRAPH=1 the body is replayed from the second iteration on as
    // a CUDA graph (one per parity, captured once per model and solution
    // buffer): one launch per iteration instead of ~50.  Measured on the
    // 153M-DOF model it gives the same solve time as eager launches (the host
    // enqueues far ahead of the GPU and the in-iteration gaps are short) and
    // its capture + instantiation costs ~55 ms on the first solve, so eager
    // launches are the default.  Profiled runs always launch eagerly.
    const bool use_graph = !c.prof && graphs_enabled();
    bool graphs_ok = use_graph && M.cg_graph[0] && M.cg_graph[1] && M.cg_graph_x == x && M.cg_graph_gen == M.gen;

    const auto t0 = std::chrono::steady_clock::now();
    int its = 0, nhist = 0;
    double resnorm = INFINITY;
    int status = GMGS_ERR_MAX_ITERATIONS;
    update_jacobi(1, 0);          // [x, r1] = JacobiSmoother(var) of the first iteration (CG_solver.m:18-19)
    while (its <= M.prm.max_it) {
        c.mark(PK_CG_ITER, false);
        ++its;
        if (its >= 2 && use_graph && !graphs_ok) {
            float *sa = r32a, *sb = r32b, *qa = pa, *qb = pb;
            graphs_ok = capture_iteration_graphs(M, body);
            r32a = sa; r32b = sb; pa = qa; pb = qb;
            if (graphs_ok) {
                M.cg_graph_x = x;
                M.cg_graph_gen = M.gen;
            }
        }
        if (its >= 2 && graphs_ok) {
            GMGS_CUDA(cudaGraphLaunch(M.cg_graph[its & 1], c.stream));
            c.launches += M.cg_graph_kernels[its & 1];
            std::swap(pa, pb);     // the swaps the replayed body made
            std::swap(r32a, r32b);
        } else {
            body(its);
        }
        c.mark(PK_CG_ITER, true);
        GMGS_CUDA(cudaMemcpyAsync(M.scal_host + SC_RR, scal + SC_RR, sizeof(double), cudaMemcpyDeviceToHost,
                                  c.stream));
        GMGS_CUDA(cudaMemcpyAsync(M.scal_host + SC_TC, M.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        GMGS_CUDA(cudaStreamSynchronize(c.stream));
        if (*reinterpret_cast<const int*>(M.scal_host + SC_TC)) break;   // check_tc reports it
        resnorm = std::sqrt(M.scal_host[SC_RR]) / normB;
        if (M.prm.verbose) std::printf(" It.: %4d Res.: %16.6e\n", its, resnorm);
        if (!std::isfinite(resnorm)) {
            status = GMGS_ERR_NONFINITE;
            break;
        }
        if (resnorm < M.prm.tol) {
            status = GMGS_OK;
            if (M.prm.verbose)
                std::printf("CG solver converged at iteration%5d to a solution with relative residual%16.6e\n", its,
                            resnorm);
            break;
        }
        if (hist) {
            const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            hist[3 * nhist + 0] = its;
            hist[3 * nhist + 1] = t;
            hist[3 * nhist + 2] = resnorm;
        }
        ++nhist;
    }
    // the last fused launch already applied the Jacobi step of an iteration
    // that does not run; its inputs (r32 it read, q, alpha) are still in place
    launch_drop_last_dx(c, n3, x, x_hi, x_lo, r32b, q, l0.wdinv32.as<float>(), scal, its & 1, 0);
    GMGS_CUDA(cudaStreamSynchronize(c.stream));
    check_tc(M);
    if (status == GMGS_ERR_MAX_ITERATIONS && M.prm.verbose) std::printf("Exceed the maximum iterate numbers\n");
    if (iters_out) *iters_out = its;
    if (relres_out) *relres_out = resnorm;
    M.last_iters = its;
    M.last_relres = resnorm;
    return status;
}

// CG_solver.m:1-56 with the Jacobi step before each preconditioner call.
int pcg_solve(Model& M, const double* b, double* x, int32_t* iters_out, double* relres_out, double* hist) {
    if (M.prm.precision == GMGS_MIXED) return pcg_mixed(M, b, x, iters_out, relres_out, hist);
    Ctx& c = M.ctx;
    Level& l0 = M.levels[0];
    const int64_t n3 = 3 * l0.g.slots;
    const bool mixed = M.prm.precision == GMGS_MIXED;
    const double om = M.prm.omega;
    double* scal = M.scal.as<double>();
    const DotScratch ds = dots(M);
    double* r = M.cg_r.as<double>();
    double* p = M.cg_p.as<double>();
    double* dx = M.cg_dx.as<double>();

    launch_dot<double, double>(c, ds, n3, b, b, scal + SC_BB);
    GMGS_CUDA(cudaMemcpyAsync(M.scal_host + SC_BB, scal + SC_BB, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    GMGS_CUDA(cudaMemsetAsync(x, 0, n3 * sizeof(double), c.stream));
    GMGS_CUDA(cudaMemcpyAsync(r, b, n3 * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));  // r = b - A*0
    GMGS_CUDA(cudaStreamSynchronize(c.stream));
    const double normB = std::sqrt(M.scal_host[SC_BB]);
    if (normB == 0.0) {
        // zero load: the reference would divide 0/0; the solution is zero
        if (iters_out) *iters_out = 0;
        if (relres_out) *relres_out = 0;
        M.last_iters = 0;
        M.last_relres = 0;
        return GMGS_OK;
    }
    if (!std::isfinite(normB)) throw Error(GMGS_ERR_NONFINITE, "non-finite load vector");

    const auto t0 = std::chrono::steady_clock::now();
    int its = 0;
    double resnorm = INFINITY;
    int status = GMGS_ERR_MAX_ITERATIONS;
    const int max_it = M.prm.max_it;
    int nhist = 0;
    while (its <= max_it) {
        c.mark(PK_CG_ITER, false);
        // [x, r1] = JacobiSmoother(var)   (CG_solver.m:18-19)
        launch_jacobi_dx<double, double, double>(c, l0.g, l0.diag64.as<double>(), om, r, dx);
        launch_add<double, double>(c, n3, x, dx);
        if (mixed) {
            fine_matvec<float, double, float>(M, dx, M.cg_y32.as<float>());
            launch_sub<double, float>(c, n3, r, M.cg_y32.as<float>());
            launch_copy<float, double>(c, n3, M.cg_r32.as<float>(), r);
            vcycle<float>(M, M.cg_r32.as<float>(), M.cg_z32.as<float>());
        } else {
            fine_matvec<double, double, double>(M, dx, M.cg_y64.as<double>());
            launch_sub<double, double>(c, n3, r, M.cg_y64.as<double>());
            vcycle<double>(M, r, M.cg_z64.as<double>());
        }
        ++its;
        const int cur = its & 1;
        if (mixed) {
            launch_dot<double, float>(c, ds, n3, r, M.cg_z32.as<float>(), scal + cur);
            launch_p_update<float>(c, n3, M.cg_z32.as<float>(), p, scal, cur | ((its == 1) << 1));
            fine_matvec<float, double, float>(M, p, M.cg_q32.as<float>());
            launch_dot<double, float>(c, ds, n3, p, M.cg_q32.as<float>(), scal + SC_PQ);
            launch_xr_update<float>(c, n3, x, r, p, M.cg_q32.as<float>(), scal, cur);
        } else {
            launch_dot<double, double>(c, ds, n3, r, M.cg_z64.as<double>(), scal + cur);
            launch_p_update<double>(c, n3, M.cg_z64.as<double>(), p, scal, cur | ((its == 1) << 1));
            fine_matvec<double, double, double>(M, p, M.cg_q64.as<double>());
            launch_dot<double, double>(c, ds, n3, p, M.cg_q64.as<double>(), scal + SC_PQ);
            launch_xr_update<double>(c, n3, x, r, p, M.cg_q64.as<double>(), scal, cur);
        }
        launch_dot<double, double>(c, ds, n3, r, r, scal + SC_RR);
        c.mark(PK_CG_ITER, true);
        GMGS_CUDA(cudaMemcpyAsync(M.scal_host + SC_RR, scal + SC_RR, sizeof(double), cudaMemcpyDeviceToHost,
                                  c.stream));
        GMGS_CUDA(cudaStreamSynchronize(c.stream));
        resnorm = std::sqrt(M.scal_host[SC_RR]) / normB;
        if (M.prm.verbose) std::printf(" It.: %4d Res.: %16.6e\n", its, resnorm);
        if (!std::isfinite(resnorm)) {
            status = GMGS_ERR_NONFINITE;
            break;
        }
        if (resnorm < M.prm.tol) {
            status = GMGS_OK;
            if (M.prm.verbose)
                std::printf("CG solver converged at iteration%5d to a solution with relative residual%16.6e\n", its,
                            resnorm);
            break;
        }
        if (hist) {
            const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            hist[3 * nhist + 0] = its;
            hist[3 * nhist + 1] = t;
            hist[3 * nhist + 2] = resnorm;
        }
        ++nhist;
    }
    if (status == GMGS_ERR_MAX_ITERATIONS && M.prm.verbose)
        std::printf("Exceed the maximum iterate numbers\n");
    if (iters_out) *iters_out = its;
    if (relres_out) *relres_out = resnorm;
    M.last_iters = its;
    M.last_relres = resnorm;
    return status;
}

}  // namespace gmgs
