// The C ABI of libgmgs (include/gmgs.h): argument validation, status codes,
// host <-> device copies and the call order of the reference's
// GetDeformation() / GetCartesianStress() (src/kernel/GetDeformation.m:1-22,
// src/kernel/GetCartesianStress.m:1-42).
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "setup.cuh"

struct gmgs_handle {
    gmgs::Model M;
    std::vector<int32_t> fixed_host;   // kept to re-apply after a density change
    std::vector<double> loads_host;
};

namespace {

thread_local std::string g_last_error;

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

template <class F>
int guarded(gmgs_handle* h, F&& f) {
    try {
        const int st = f();
#ifdef GMGS_CHECKED
        std::string m;
        if (gmgs::chk::report(m)) {
            g_last_error = m;
            if (h) h->M.err = m;
            return GMGS_ERR_CUDA;
        }
#endif
        return st;
    } catch (const gmgs::Error& e) {
        g_last_error = e.what();
#ifdef GMGS_CHECKED
        // an out-of-range access is the likelier cause of a failure in a checked build
        std::string m;
        if (gmgs::chk::report(m)) {
            g_last_error = m + " (the call then failed: " + e.what() + ")";
            if (h) h->M.err = g_last_error;
            return GMGS_ERR_CUDA;
        }
#endif
        if (h) h->M.err = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        if (h) h->M.err = g_last_error;
        return GMGS_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        if (h) h->M.err = e.what();
        return GMGS_ERR_CUDA;
    }
}

void fail(int status, const char* msg) { throw gmgs::Error(status, msg); }

// Host buffers of a call: a copy between the device and pageable host memory
// runs at link speed (about 190 GB/s on the Grace host) only when the pages
// are already mapped and the driver takes its direct path; a freshly
// allocated output is first faulted in page by page (20-30 GB/s on one core)
// and large pageable copies were seen to drop to 5-8 GB/s at times.  Large
// host ranges are therefore pinned for the duration of their copy
// (cudaHostRegister, about 2 ms per GB once the pages exist) and unpinned
// afterwards; a range that cannot be pinned (already pinned, or not
// registrable) is copied pageable as before.
constexpr size_t kPinMinBytes = 32u << 20;

class HostPin {
public:
    HostPin(const void* p, size_t bytes, bool read_only) {
        if (!p || bytes < kPinMinBytes) return;
        unsigned flags = cudaHostRegisterPortable | (read_only ? cudaHostRegisterReadOnly : 0u);
        if (cudaHostRegister(const_cast<void*>(p), bytes, flags) == cudaSuccess) p_ = const_cast<void*>(p);
        else cudaGetLastError();
    }
    HostPin(const HostPin&) = delete;
    HostPin& operator=(const HostPin&) = delete;
    ~HostPin() {
        if (p_ && cudaHostUnregister(p_) != cudaSuccess) cudaGetLastError();
    }

private:
    void* p_ = nullptr;
};

// An output buffer is faulted in (one byte written per page, from up to 8
// host threads) and then pinned while the GPU is still computing, so the
// device-to-host copy that follows finds every page mapped and locked.  Its
// contents are overwritten by the copy anyway.  join() before the copy; the
// destructor unpins, so the object must outlive the copy's synchronisation.
class HostPrefault {
public:
    HostPrefault(void* p, size_t bytes) {
        if (!p || bytes < kPinMinBytes) return;
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return; }
        manager_ = std::thread([this, p, bytes, dev]() {
            const long pg = sysconf(_SC_PAGESIZE);
            const size_t page = pg > 0 ? (size_t)pg : 4096;
            const unsigned hc = std::thread::hardware_concurrency();
            const size_t nt = std::min<size_t>(kMaxThreads, std::max<size_t>(1, hc / 2));
            char* base = static_cast<char*>(p);
            const size_t per = (bytes + nt - 1) / nt;
            std::vector<std::thread> touch;
            for (size_t t = 0; t < nt; ++t) {
                const size_t b = t * per, e = std::min(bytes, b + per);
                if (b >= e) break;
                touch.emplace_back([base, b, e, page]() {
                    volatile char* q = base;
                    for (size_t i = b; i < e; i += page) q[i] = 0;
                    q[e - 1] = 0;
                });
            }
            for (auto& t : touch) t.join();
            if (cudaSetDevice(dev) == cudaSuccess && cudaHostRegister(p, bytes, cudaHostRegisterPortable) == cudaSuccess)
                pinned_ = p;
            else
                cudaGetLastError();
        });
    }
    HostPrefault(const HostPrefault&) = delete;
    HostPrefault& operator=(const HostPrefault&) = delete;
    void join() {
        if (manager_.joinable()) manager_.join();
    }
    ~HostPrefault() {
        join();
        if (pinned_ && cudaHostUnregister(pinned_) != cudaSuccess) cudaGetLastError();
    }

private:
    static constexpr size_t kMaxThreads = 8;
    std::thread manager_;
    void* pinned_ = nullptr;
};

// the reference's level rule (DiscretizeDesignDomain.m:29-41); returns numLevels
int level_rule(int nely, int nelx, int nelz, const gmgs_params& p) {
    if (p.num_levels) {
        if (p.num_levels < 2) fail(GMGS_ERR_RESOLUTION, "There is no sufficient resolution to invoke GMGS!");
        return p.num_levels;
    }
    double num = (double)nelx * nely * nelz;
    if (num < (double)p.coarsest_resolution_control)
        fail(GMGS_ERR_RESOLUTION, "There is no Sufficient Resolution to Build Mesh Hierarchy!");
    int k = 0;
    while (num >= (double)p.coarsest_resolution_control) {
        ++k;
        const double f = std::ldexp(1.0, k);
        num = nelx / f * (nely / f) * (nelz / f);
        if (k > 20) break;
    }
    return k + 1;
}

void ensure_coarse(gmgs_handle* h) {
    gmgs::Model& M = h->M;
    if (!M.bc_set) fail(GMGS_ERR_STATE, "boundary conditions are not set");
    if (!M.coarse_ready) {
        const auto t0 = Clock::now();
        M.ctx.trace_point("bc: start");
        // the work buffers are set up while the coarsest blocks factor
        gmgs::build_coarse_bc(M, [&M]() { gmgs::alloc_work(M); });
        M.ctx.trace_point("bc: work buffers");
        M.coarse_ready = true;
        M.t_bc_ms = ms_since(t0);
    }
}

int64_t model_bytes(const gmgs::Model& M) {
    int64_t b = 0;
    for (const auto& lv : M.levels)
        for (const gmgs::DevBuf* d : {&lv.emask, &lv.nflag, &lv.etype, &lv.escale64, &lv.escale32, &lv.Ks64, &lv.Ks32,
                                      &lv.kslot, &lv.diag64, &lv.diag32, &lv.wdinv32, &lv.emask8, &lv.perel_nodes, &lv.node_slot, &lv.elem_slot,
                                      &lv.vr, &lv.vrp, &lv.vdx, &lv.vx, &lv.vy, &lv.tile_occ, &lv.tc_occ})
            b += (int64_t)d->bytes;
    for (const gmgs::DevBuf* d : {&M.ke0_dev, &M.rho, &M.F, &M.U, &M.free_idx, &M.cb.sinv, &M.cb.g, &M.cb.partial, &M.cb.ticket, &M.cvec_in, &M.cvec_out,
                                  &M.cg_x, &M.cg_r, &M.cg_p, &M.cg_dx, &M.cg_q64, &M.cg_y64, &M.cg_z64, &M.cg_q32,
                                  &M.cg_y32, &M.cg_z32, &M.cg_r32, &M.cg_r32b, &M.cg_pa, &M.cg_pb, &M.scal, &M.dot_partials, &M.dot_ticket, &M.tc_err})
        b += (int64_t)d->bytes;
    return b;
}

int solve_impl(gmgs_handle* h, double* U_host, double* U_dev, int32_t* iters, double* relres, double* hist) {
    gmgs::Model& M = h->M;
    ensure_coarse(h);
    gmgs::Level& l0 = M.levels[0];
    const size_t n3 = 3 * (size_t)l0.g.slots;
    if (M.U.bytes < n3 * sizeof(double)) M.U = gmgs::dalloc(n3 * sizeof(double));
    const auto t0 = Clock::now();
    HostPrefault pf(U_host, 3 * (size_t)l0.n_node * sizeof(double));
    M.ctx.trace_point("solve: start");
    const int st = gmgs::pcg_solve(M, M.F.as<double>(), M.U.as<double>(), iters, relres, hist);
    M.ctx.trace_point("solve: PCG (incl. work buffers)");
    if (st == GMGS_ERR_NONFINITE) fail(st, "CG residual is not finite (diverged)");
    M.solved = true;
    const int64_t nn = l0.n_node;
    if (U_host || U_dev) {
        gmgs::DevBuf tmp;
        double* dst = U_dev;
        if (!dst) {
            tmp = gmgs::dalloc(3 * nn * sizeof(double));
            dst = tmp.as<double>();
        }
        gmgs::launch_dense_to_compact<double>(M.ctx, nn, l0.g.slots, l0.node_slot.as<int32_t>(), M.U.as<double>(), dst);
        M.ctx.trace_point("solve: compaction");
        pf.join();
        M.ctx.trace_point("solve: host page prefault (join)");
        if (U_host)
            GMGS_CUDA(cudaMemcpyAsync(U_host, dst, 3 * nn * sizeof(double), cudaMemcpyDeviceToHost, M.ctx.stream));
        GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
        M.ctx.trace_point("solve: device-to-host copy");
    }
    M.t_solve_ms = ms_since(t0);
    if (st == GMGS_ERR_MAX_ITERATIONS) M.err = "Exceed the maximum iterate numbers";
    return st;
}

}  // namespace

namespace gmgs {
// error message for entry points that run without a handle
void set_thread_error(const std::string& msg) { g_last_error = msg; }

namespace chk {
const char* site_name(int site) {
    static const char* const names[SITE_COUNT] = {
        "none", "k_fine field staging", "k_fine node operands", "k_fine node flags", "k_fine element data",
        "k_fine element matrices", "k_fine shared ring", "k_fine outputs", "k_up32 fine operands",
        "k_up32 coarse values", "k_up32 output", "k_perel_vdown node list", "k_perel_vdown element data",
        "k_perel_vdown vectors", "k_perel_vdown element matrices", "k_perel_vdown output", "k_tc_vdown field staging",
        "k_tc_vdown element data", "k_tc_vdown node operands", "k_tc_vdown shared ring",
        "k_tc_vdown element-output buffer", "k_tc_vdown output", "k_matvec input gather", "k_matvec element data",
        "k_matvec output", "k_restrict", "k_prolong_post", "stress displacement gather", "stress outputs",
        "k_grad"};
    return site > 0 && site < SITE_COUNT ? names[site] : "unknown site";
}
#ifdef GMGS_CHECKED
static std::vector<Reader>& readers() {
    static std::vector<Reader> v;
    return v;
}
void add_reader(Reader r) { readers().push_back(r); }
bool report(std::string& msg) {
    cudaDeviceSynchronize();
    bool any = false;
    for (Reader r : readers()) {
        std::string m;
        if (r(m) && !any) {
            msg = m;
            any = true;
        }
    }
    return any;
}
#endif
}  // namespace chk
}  // namespace gmgs

extern "C" {

void gmgs_default_params(gmgs_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->tol = 1.0e-3;
    p->max_it = 20000;
    p->omega = 0.4;
    p->youngs_modulus = 1.0;
    p->poisson_ratio = 0.3;
    p->coarsest_resolution_control = 10000;
    p->num_levels = 0;
    p->precision = GMGS_FP64;
    p->verbose = 0;
}

const char* gmgs_status_string(int s) {
    switch (s) {
        case GMGS_OK: return "ok";
        case GMGS_ERR_INVALID_ARGUMENT: return "invalid argument";
        case GMGS_ERR_RESOLUTION: return "insufficient resolution for the multigrid hierarchy";
        case GMGS_ERR_NO_SOLID: return "no solid voxel";
        case GMGS_ERR_NO_LOADS: return "no loads";
        case GMGS_ERR_NO_FIXINGS: return "no constraints";
        case GMGS_ERR_NOT_SPD: return "coarsest-level matrix not positive definite";
        case GMGS_ERR_MAX_ITERATIONS: return "maximum number of iterations exceeded";
        case GMGS_ERR_NONFINITE: return "non-finite value";
        case GMGS_ERR_NO_SOLUTION: return "no deformation field available";
        case GMGS_ERR_CUDA: return "CUDA error";
        case GMGS_ERR_OUT_OF_MEMORY: return "out of device memory";
        case GMGS_ERR_STATE: return "call order";
        case GMGS_ERR_MESH: return "mesh not voxelisable";
        default: return "unknown status";
    }
}

const char* gmgs_last_error(const gmgs_handle* h) {
    if (h) return h->M.err.c_str();
    return g_last_error.c_str();
}

int gmgs_create(const int32_t* occ, int32_t ny, int32_t nx, int32_t nz, const double ele_size[3],
                const gmgs_params* params, gmgs_handle** out) {
    return guarded(nullptr, [&]() -> int {
        if (!out) fail(GMGS_ERR_INVALID_ARGUMENT, "out is NULL");
        *out = nullptr;
        if (!occ) fail(GMGS_ERR_INVALID_ARGUMENT, "occupancy is NULL");
        if (ny < 1 || nx < 1 || nz < 1) fail(GMGS_ERR_INVALID_ARGUMENT, "grid dimensions must be positive");
        gmgs_params p;
        if (params) p = *params; else gmgs_default_params(&p);
        if (!(p.tol > 0) || p.max_it < 0 || !(p.omega > 0) || !(p.youngs_modulus > 0) ||
            !(p.poisson_ratio > -1.0 && p.poisson_ratio < 0.5) || p.coarsest_resolution_control < 1 ||
            (p.precision != GMGS_FP64 && p.precision != GMGS_MIXED) || p.num_levels < 0)
            fail(GMGS_ERR_INVALID_ARGUMENT, "invalid solver parameters");
        double ele[3] = {1, 1, 1};
        if (ele_size)
            for (int i = 0; i < 3; ++i) {
                if (!(ele_size[i] > 0) || !std::isfinite(ele_size[i]))
                    fail(GMGS_ERR_INVALID_ARGUMENT, "element size must be positive");
                ele[i] = ele_size[i];
            }
        const int L = level_rule(ny, nx, nz, p);
        const int f = 1 << (L - 1);
        if (L > 16) fail(GMGS_ERR_RESOLUTION, "too many levels");
        const int64_t pny = ((int64_t)ny + f - 1) / f * f, pnx = ((int64_t)nx + f - 1) / f * f,
                      pnz = ((int64_t)nz + f - 1) / f * f;
        const int64_t slots = (pny + 17) * (pnx + 3) * (pnz + 3);
        if (slots > (int64_t)INT32_MAX) fail(GMGS_ERR_INVALID_ARGUMENT, "grid too large for 32-bit slot indices");

        const auto t0 = Clock::now();
        auto h = std::make_unique<gmgs_handle>();
        gmgs::Model& M = h->M;
        M.prm = p;
        M.nely = ny; M.nelx = nx; M.nelz = nz;
        M.ny = (int)pny; M.nx = (int)pnx; M.nz = (int)pnz;
        std::memcpy(M.ele, ele, sizeof(ele));
        M.num_levels = L;
        int dev = 0;
        GMGS_CUDA(cudaGetDevice(&dev));
        GMGS_CUDA(cudaDeviceGetAttribute(&M.ctx.num_sms, cudaDevAttrMultiProcessorCount, dev));
        GMGS_CUDA(cudaStreamCreateWithFlags(&M.ctx.stream, cudaStreamNonBlocking));
        M.own_stream = true;
        {
            const char* tr = std::getenv("GMGS_TRACE");
            M.ctx.trace = tr && tr[0] && tr[0] != '0';
        }
        M.ctx.trace_point("create: start");
        {
            gmgs::DevBuf occ_dev = gmgs::dalloc((size_t)ny * nx * nz * sizeof(int32_t));
            HostPin pin(occ, (size_t)ny * nx * nz * sizeof(int32_t), true);
            GMGS_CUDA(cudaMemcpyAsync(occ_dev.p, occ, (size_t)ny * nx * nz * sizeof(int32_t), cudaMemcpyHostToDevice,
                                      M.ctx.stream));
            GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
            M.ctx.trace_point("create: occupancy to device");
            gmgs::build_levels(M, occ_dev.as<int32_t>());
        }
        M.ctx.trace_point("create: occupancy buffer freed");
        gmgs::build_operators(M);
        M.ops_ready = true;
        M.t_create_ms = ms_since(t0);
        *out = h.release();
        return GMGS_OK;
    });
}

int gmgs_set_bc(gmgs_handle* h, const int32_t* fixed, int64_t nfixed, const double* loads, int64_t nload) {
    return guarded(h, [&]() -> int {
        if (!h) fail(GMGS_ERR_INVALID_ARGUMENT, "handle is NULL");
        if (nload <= 0 || !loads) fail(GMGS_ERR_NO_LOADS, "No Loads! Unable to Perform Static FEA!");
        if (nfixed <= 0 || !fixed) fail(GMGS_ERR_NO_FIXINGS, "No Constraints! Unable to Perform Static FEA!");
        h->M.ctx.trace_point("set_bc: start");
        gmgs::apply_bc(h->M, fixed, nfixed, loads, nload);
        h->M.ctx.trace_point("set_bc: fixed nodes + loads");
        h->fixed_host.assign(fixed, fixed + nfixed);
        h->loads_host.assign(loads, loads + 4 * nload);
        h->M.bc_set = true;
        // like the reference, a later call changes level 1 only: the coarse
        // fixed DOFs and the coarsest factorisation come from SetupSolver(),
        // which GetDeformation.m:12-16 runs once per hierarchy
        return GMGS_OK;
    });
}

int gmgs_set_density(gmgs_handle* h, const double* rho, double penal) {
    return guarded(h, [&]() -> int {
        if (!h || !rho) fail(GMGS_ERR_INVALID_ARGUMENT, "NULL argument");
        if (!std::isfinite(penal) || penal < 0) fail(GMGS_ERR_INVALID_ARGUMENT, "invalid penalty");
        gmgs::Model& M = h->M;
        const int64_t ne = M.levels[0].n_elem;
        for (int64_t i = 0; i < ne; ++i)
            if (!(rho[i] > 0) || !std::isfinite(rho[i])) fail(GMGS_ERR_INVALID_ARGUMENT, "density must be positive");
        gmgs::DevBuf d = gmgs::dalloc(ne * sizeof(double));
        {
            HostPin pin(rho, ne * sizeof(double), true);
            GMGS_CUDA(cudaMemcpyAsync(d.p, rho, ne * sizeof(double), cudaMemcpyHostToDevice, M.ctx.stream));
            GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
        }
        M.penal = penal;
        gmgs::set_density_dev(M, d.as<double>());
        M.coarse_ready = false;
        M.solved = false;
        if (M.bc_set)
            gmgs::apply_bc(M, h->fixed_host.data(), (int64_t)h->fixed_host.size(), h->loads_host.data(),
                           (int64_t)h->loads_host.size() / 4);
        return GMGS_OK;
    });
}

int gmgs_solve(gmgs_handle* h, double* U, int32_t* iters, double* relres, double* hist) {
    return guarded(h, [&]() -> int {
        if (!h) fail(GMGS_ERR_INVALID_ARGUMENT, "handle is NULL");
        return solve_impl(h, U, nullptr, iters, relres, hist);
    });
}

int gmgs_solve_dev(gmgs_handle* h, double* U_dev, int32_t* iters, double* relres, double* hist) {
    return guarded(h, [&]() -> int {
        if (!h) fail(GMGS_ERR_INVALID_ARGUMENT, "handle is NULL");
        return solve_impl(h, nullptr, U_dev, iters, relres, hist);
    });
}

static int stress_impl(gmgs_handle* h, double* nodal_host, float* vox_host, double* nodal_dev, float* vox_dev) {
    gmgs::Model& M = h->M;
    if (!M.solved) fail(GMGS_ERR_NO_SOLUTION, "No Deformation Field Available, compute the deformation first");
    const auto t0 = Clock::now();
    gmgs::Level& l0 = M.levels[0];
    gmgs::DevBuf tn, tv;
    double* nd = nodal_dev;
    float* vd = vox_dev;
    if (nodal_host && !nd) { tn = gmgs::dalloc(6 * l0.n_node * sizeof(double)); nd = tn.as<double>(); }
    if (vox_host && !vd) { tv = gmgs::dalloc(6 * l0.n_elem * sizeof(float)); vd = tv.as<float>(); }
    HostPrefault pfn(nodal_host, 6 * (size_t)l0.n_node * sizeof(double));
    HostPrefault pfv(vox_host, 6 * (size_t)l0.n_elem * sizeof(float));
    gmgs::stress_dev(M, M.U.as<double>(), nd, vd);
    pfn.join();
    pfv.join();
    if (nodal_host)
        GMGS_CUDA(cudaMemcpyAsync(nodal_host, nd, 6 * l0.n_node * sizeof(double), cudaMemcpyDeviceToHost, M.ctx.stream));
    if (vox_host)
        GMGS_CUDA(cudaMemcpyAsync(vox_host, vd, 6 * l0.n_elem * sizeof(float), cudaMemcpyDeviceToHost, M.ctx.stream));
    GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
    M.t_stress_ms = ms_since(t0);
    return GMGS_OK;
}

int gmgs_stress(gmgs_handle* h, double* nodal, float* per_voxel) {
    return guarded(h, [&]() -> int {
        if (!h || (!nodal && !per_voxel)) fail(GMGS_ERR_INVALID_ARGUMENT, "NULL argument");
        return stress_impl(h, nodal, per_voxel, nullptr, nullptr);
    });
}

int gmgs_stress_dev(gmgs_handle* h, double* nodal, float* per_voxel) {
    return guarded(h, [&]() -> int {
        if (!h || (!nodal && !per_voxel)) fail(GMGS_ERR_INVALID_ARGUMENT, "NULL argument");
        return stress_impl(h, nullptr, nullptr, nodal, per_voxel);
    });
}

static int grad_impl(gmgs_handle* h, const double* ell_host, const double* ell_dev, double* out_host, double* out_dev) {
    gmgs::Model& M = h->M;
    if (!M.has_density) fail(GMGS_ERR_STATE, "the gradient needs gmgs_set_density");
    if (!M.solved) fail(GMGS_ERR_NO_SOLUTION, "No Deformation Field Available, compute the deformation first");
    gmgs::Level& l0 = M.levels[0];
    const int64_t nn = l0.n_node, S = l0.g.slots;
    HostPrefault pf(out_host, (size_t)l0.n_elem * sizeof(double));
    gmgs::DevBuf lam;
    const double* L = M.U.as<double>();
    if (ell_host || ell_dev) {
        gmgs::DevBuf ec, ed = gmgs::dalloc(3 * S * sizeof(double));
        const double* src = ell_dev;
        if (ell_host) {
            ec = gmgs::dalloc(3 * nn * sizeof(double));
            HostPin pin(ell_host, 3 * nn * sizeof(double), true);
            GMGS_CUDA(cudaMemcpyAsync(ec.p, ell_host, 3 * nn * sizeof(double), cudaMemcpyHostToDevice, M.ctx.stream));
            GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
            src = ec.as<double>();
        }
        GMGS_CUDA(cudaMemsetAsync(ed.p, 0, 3 * S * sizeof(double), M.ctx.stream));
        gmgs::launch_compact_to_dense<double>(M.ctx, nn, S, l0.node_slot.as<int32_t>(), src, ed.as<double>());
        lam = gmgs::dalloc(3 * S * sizeof(double));
        // adjoint solve K lam = ell with the same PCG (self-adjoint system)
        const int st = gmgs::pcg_solve(M, ed.as<double>(), lam.as<double>(), nullptr, nullptr, nullptr);
        if (st == GMGS_ERR_NONFINITE) fail(st, "adjoint CG diverged");
        L = lam.as<double>();
    }
    gmgs::DevBuf to;
    double* od = out_dev;
    if (!od) { to = gmgs::dalloc(l0.n_elem * sizeof(double)); od = to.as<double>(); }
    gmgs::grad_dev(M, M.U.as<double>(), L, od);
    pf.join();
    if (out_host)
        GMGS_CUDA(cudaMemcpyAsync(out_host, od, l0.n_elem * sizeof(double), cudaMemcpyDeviceToHost, M.ctx.stream));
    GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
    return GMGS_OK;
}

int gmgs_grad(gmgs_handle* h, const double* ell, double* dJdrho) {
    return guarded(h, [&]() -> int {
        if (!h || !dJdrho) fail(GMGS_ERR_INVALID_ARGUMENT, "NULL argument");
        return grad_impl(h, ell, nullptr, dJdrho, nullptr);
    });
}

int gmgs_grad_dev(gmgs_handle* h, const double* ell, double* dJdrho) {
    return guarded(h, [&]() -> int {
        if (!h || !dJdrho) fail(GMGS_ERR_INVALID_ARGUMENT, "NULL argument");
        return grad_impl(h, nullptr, ell, nullptr, dJdrho);
    });
}

int gmgs_apply_operator(gmgs_handle* h, int32_t level, const double* x, double* y) {
    return guarded(h, [&]() -> int {
        if (!h || !x || !y) fail(GMGS_ERR_INVALID_ARGUMENT, "NULL argument");
        gmgs::Model& M = h->M;
        if (level < 1 || level > M.num_levels) fail(GMGS_ERR_INVALID_ARGUMENT, "level out of range");
        if (level == 2 && M.lean_level1)
            fail(GMGS_ERR_STATE, "level 2 keeps only FP32 element matrices on a mixed-precision handle with a density "
                                 "field; use an FP64 handle to apply it");
        ensure_coarse(h);
        gmgs::Level& lv = M.levels[level - 1];
        const int64_t nn = lv.n_node, S = lv.g.slots;
        gmgs::DevBuf xc = gmgs::dalloc(3 * nn * sizeof(double)), xd = gmgs::dalloc(3 * S * sizeof(double)),
                     yd = gmgs::dalloc(3 * S * sizeof(double));
        HostPin pin_in(x, 3 * nn * sizeof(double), true), pin_out(y, 3 * nn * sizeof(double), false);
        GMGS_CUDA(cudaMemcpyAsync(xc.p, x, 3 * nn * sizeof(double), cudaMemcpyHostToDevice, M.ctx.stream));
        GMGS_CUDA(cudaMemsetAsync(xd.p, 0, 3 * S * sizeof(double), M.ctx.stream));
        gmgs::launch_compact_to_dense<double>(M.ctx, nn, S, lv.node_slot.as<int32_t>(), xc.as<double>(), xd.as<double>());
        gmgs::apply_operator_dense(M, level - 1, xd.as<double>(), yd.as<double>());
        gmgs::launch_dense_to_compact<double>(M.ctx, nn, S, lv.node_slot.as<int32_t>(), yd.as<double>(), xc.as<double>());
        GMGS_CUDA(cudaMemcpyAsync(y, xc.p, 3 * nn * sizeof(double), cudaMemcpyDeviceToHost, M.ctx.stream));
        GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
        return GMGS_OK;
    });
}

int gmgs_apply_preconditioner(gmgs_handle* h, const double* r, double* z) {
    return guarded(h, [&]() -> int {
        if (!h || !r || !z) fail(GMGS_ERR_INVALID_ARGUMENT, "NULL argument");
        gmgs::Model& M = h->M;
        ensure_coarse(h);
        gmgs::Level& lv = M.levels[0];
        const int64_t nn = lv.n_node, S = lv.g.slots;
        gmgs::DevBuf xc = gmgs::dalloc(3 * nn * sizeof(double)), xd = gmgs::dalloc(3 * S * sizeof(double)),
                     yd = gmgs::dalloc(3 * S * sizeof(double));
        HostPin pin_in(r, 3 * nn * sizeof(double), true), pin_out(z, 3 * nn * sizeof(double), false);
        GMGS_CUDA(cudaMemcpyAsync(xc.p, r, 3 * nn * sizeof(double), cudaMemcpyHostToDevice, M.ctx.stream));
        GMGS_CUDA(cudaMemsetAsync(xd.p, 0, 3 * S * sizeof(double), M.ctx.stream));
        GMGS_CUDA(cudaMemsetAsync(yd.p, 0, 3 * S * sizeof(double), M.ctx.stream));
        gmgs::launch_compact_to_dense<double>(M.ctx, nn, S, lv.node_slot.as<int32_t>(), xc.as<double>(), xd.as<double>());
        gmgs::vcycle_apply_fp64(M, xd.as<double>(), yd.as<double>());
        gmgs::launch_dense_to_compact<double>(M.ctx, nn, S, lv.node_slot.as<int32_t>(), yd.as<double>(), xc.as<double>());
        GMGS_CUDA(cudaMemcpyAsync(z, xc.p, 3 * nn * sizeof(double), cudaMemcpyDeviceToHost, M.ctx.stream));
        GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
        return GMGS_OK;
    });
}

int gmgs_apply_operator_dev(gmgs_handle* h, int32_t level, const double* x, double* y) {
    return guarded(h, [&]() -> int {
        if (!h || !x || !y) fail(GMGS_ERR_INVALID_ARGUMENT, "NULL argument");
        gmgs::Model& M = h->M;
        if (level < 1 || level > M.num_levels) fail(GMGS_ERR_INVALID_ARGUMENT, "level out of range");
        if (level == 2 && M.lean_level1)
            fail(GMGS_ERR_STATE, "level 2 keeps only FP32 element matrices on a mixed-precision handle with a density "
                                 "field; use an FP64 handle to apply it");
        ensure_coarse(h);
        gmgs::Level& lv = M.levels[level - 1];
        const int64_t nn = lv.n_node, S = lv.g.slots;
        gmgs::DevBuf xd = gmgs::dalloc(3 * S * sizeof(double)), yd = gmgs::dalloc(3 * S * sizeof(double));
        GMGS_CUDA(cudaMemsetAsync(xd.p, 0, 3 * S * sizeof(double), M.ctx.stream));
        gmgs::launch_compact_to_dense<double>(M.ctx, nn, S, lv.node_slot.as<int32_t>(), x, xd.as<double>());
        gmgs::apply_operator_dense(M, level - 1, xd.as<double>(), yd.as<double>());
        gmgs::launch_dense_to_compact<double>(M.ctx, nn, S, lv.node_slot.as<int32_t>(), yd.as<double>(), y);
        GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
        return GMGS_OK;
    });
}

int gmgs_apply_preconditioner_dev(gmgs_handle* h, const double* r, double* z) {
    return guarded(h, [&]() -> int {
        if (!h || !r || !z) fail(GMGS_ERR_INVALID_ARGUMENT, "NULL argument");
        gmgs::Model& M = h->M;
        ensure_coarse(h);
        gmgs::Level& lv = M.levels[0];
        const int64_t nn = lv.n_node, S = lv.g.slots;
        gmgs::DevBuf xd = gmgs::dalloc(3 * S * sizeof(double)), yd = gmgs::dalloc(3 * S * sizeof(double));
        GMGS_CUDA(cudaMemsetAsync(xd.p, 0, 3 * S * sizeof(double), M.ctx.stream));
        GMGS_CUDA(cudaMemsetAsync(yd.p, 0, 3 * S * sizeof(double), M.ctx.stream));
        gmgs::launch_compact_to_dense<double>(M.ctx, nn, S, lv.node_slot.as<int32_t>(), r, xd.as<double>());
        gmgs::vcycle_apply_fp64(M, xd.as<double>(), yd.as<double>());
        gmgs::launch_dense_to_compact<double>(M.ctx, nn, S, lv.node_slot.as<int32_t>(), yd.as<double>(), z);
        GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
        return GMGS_OK;
    });
}

int gmgs_dot_dev(gmgs_handle* h, const double* x, const double* y, int64_t n, double* result) {
    return guarded(h, [&]() -> int {
        if (!h || !x || !y || !result || n < 0) fail(GMGS_ERR_INVALID_ARGUMENT, "invalid argument");
        gmgs::Model& M = h->M;
        if (!M.dot_partials.p) {
            M.dot_blocks = M.ctx.num_sms * 4;
            M.dot_partials = gmgs::dalloc(M.dot_blocks * sizeof(double));
            M.dot_ticket = gmgs::dalloc(sizeof(unsigned int));
            GMGS_CUDA(cudaMemsetAsync(M.dot_ticket.p, 0, sizeof(unsigned int), M.ctx.stream));
        }
        if (!M.scal.p) M.scal = gmgs::dalloc(8 * sizeof(double));
        const gmgs::DotScratch ds{M.dot_partials.as<double>(), M.dot_ticket.as<unsigned int>(), M.dot_blocks};
        double* out = M.scal.as<double>() + 7;
        gmgs::launch_dot<double, double>(M.ctx, ds, n, x, y, out);
        GMGS_CUDA(cudaMemcpyAsync(result, out, sizeof(double), cudaMemcpyDeviceToHost, M.ctx.stream));
        GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
        return GMGS_OK;
    });
}

int gmgs_num_levels(const gmgs_handle* h, int32_t* out) {
    if (!h || !out) return GMGS_ERR_INVALID_ARGUMENT;
    *out = h->M.num_levels;
    return GMGS_OK;
}

int gmgs_num_nodes(const gmgs_handle* h, int32_t level, int64_t* out) {
    if (!h || !out || level < 1 || level > h->M.num_levels) return GMGS_ERR_INVALID_ARGUMENT;
    *out = h->M.levels[level - 1].n_node;
    return GMGS_OK;
}

int gmgs_num_elements(const gmgs_handle* h, int32_t level, int64_t* out) {
    if (!h || !out || level < 1 || level > h->M.num_levels) return GMGS_ERR_INVALID_ARGUMENT;
    *out = h->M.levels[level - 1].n_elem;
    return GMGS_OK;
}

int gmgs_padded_dims(const gmgs_handle* h, int32_t dims[3]) {
    if (!h || !dims) return GMGS_ERR_INVALID_ARGUMENT;
    dims[0] = h->M.ny; dims[1] = h->M.nx; dims[2] = h->M.nz;
    return GMGS_OK;
}

int gmgs_set_stream(gmgs_handle* h, void* stream) {
    return guarded(h, [&]() -> int {
        if (!h) fail(GMGS_ERR_INVALID_ARGUMENT, "handle is NULL");
        gmgs::Model& M = h->M;
        GMGS_CUDA(cudaStreamSynchronize(M.ctx.stream));
        if (stream) {
            if (M.own_stream) GMGS_CUDA(cudaStreamDestroy(M.ctx.stream));
            M.ctx.stream = (cudaStream_t)stream;
            M.own_stream = false;
        } else if (!M.own_stream) {
            GMGS_CUDA(cudaStreamCreateWithFlags(&M.ctx.stream, cudaStreamNonBlocking));
            M.own_stream = true;
        }
        return GMGS_OK;
    });
}

int gmgs_set_tolerance(gmgs_handle* h, double tol, int32_t max_it) {
    if (!h || !(tol > 0) || max_it < 0) return GMGS_ERR_INVALID_ARGUMENT;
    h->M.prm.tol = tol;
    h->M.prm.max_it = max_it;
    return GMGS_OK;
}

int gmgs_device_bytes(const gmgs_handle* h, int64_t* out) {
    if (!h || !out) return GMGS_ERR_INVALID_ARGUMENT;
    *out = model_bytes(h->M);
    return GMGS_OK;
}

int gmgs_memory_stats(int64_t* current_bytes, int64_t* peak_bytes, int32_t reset_peak) {
    if (current_bytes) *current_bytes = gmgs::g_dev_bytes.load();
    if (peak_bytes) *peak_bytes = gmgs::g_dev_peak.load();
    if (reset_peak) gmgs::g_dev_peak.store(gmgs::g_dev_bytes.load());
    return GMGS_OK;
}

int gmgs_launch_count(const gmgs_handle* h, int64_t* out) {
    if (!h || !out) return GMGS_ERR_INVALID_ARGUMENT;
    *out = h->M.ctx.launches;
    return GMGS_OK;
}

int gmgs_phase_times(const gmgs_handle* h, double out[4]) {
    if (!h || !out) return GMGS_ERR_INVALID_ARGUMENT;
    out[0] = h->M.t_create_ms;
    out[1] = h->M.t_bc_ms;
    out[2] = h->M.t_solve_ms;
    out[3] = h->M.t_stress_ms;
    return GMGS_OK;
}

int gmgs_set_profiling(gmgs_handle* h, int32_t enable) {
    return guarded(h, [&]() -> int {
        if (!h) fail(GMGS_ERR_INVALID_ARGUMENT, "handle is NULL");
        gmgs::Ctx& c = h->M.ctx;
        GMGS_CUDA(cudaStreamSynchronize(c.stream));
        for (auto& s : c.prof_slot) { s.used = 0; s.bytes = 0; }
        c.prof = enable != 0;
        return GMGS_OK;
    });
}

int gmgs_kernel_time(gmgs_handle* h, int32_t kernel, int64_t* launches, double* total_ms, double* bytes) {
    return guarded(h, [&]() -> int {
        if (!h || kernel < 0 || kernel >= gmgs::PK_COUNT) fail(GMGS_ERR_INVALID_ARGUMENT, "bad kernel id");
        gmgs::Ctx& c = h->M.ctx;
        GMGS_CUDA(cudaStreamSynchronize(c.stream));
        const gmgs::ProfSlot& s = c.prof_slot[kernel];
        double tot = 0;
        for (int i = 0; i + 1 < s.used; i += 2) {
            float ms = 0;
            GMGS_CUDA(cudaEventElapsedTime(&ms, s.ev[i], s.ev[i + 1]));
            tot += ms;
        }
        if (launches) *launches = s.used / 2;
        if (total_ms) *total_ms = tot;
        if (bytes) *bytes = s.bytes;
        return GMGS_OK;
    });
}

void gmgs_destroy(gmgs_handle* h) {
    if (!h) return;
    gmgs::Model& M = h->M;
    if (M.ctx.stream) cudaStreamSynchronize(M.ctx.stream);
    gmgs::reset_graphs(M);
    M.levels.clear();
    for (auto& s : M.ctx.prof_slot)
        for (cudaEvent_t e : s.ev) cudaEventDestroy(e);
    if (M.scal_host) cudaFreeHost(M.scal_host);
    const bool own = M.own_stream;
    cudaStream_t s = M.ctx.stream;
    delete h;
    if (own && s) cudaStreamDestroy(s);
}

}  // extern "C"
