// Mesh voxelisation on the GPU: CreateVoxilizedModel(triFaceModelFile,
// finestResCtrl) of the reference (src/common/CreateVoxilizedModel.m:10-26).
//
// The reference sizes the grid from the mesh bounding box
// (src/common/AdaptData4Voxelize.m:5-18) and voxelises by ray parity with
// A. H. Aitkenhead's VOXELISE, vendored as src/common/Voxelize.m: rays along
// x, y and z through the voxel centres, a voxel is inside for one direction
// when it lies between the 2k-1-th and 2k-th distinct crossing of its ray,
// rays with an odd number of crossings take an 8-neighbour vote afterwards,
// and a voxel is solid when at least two directions agree.  The result is
// flipped along y (CreateVoxilizedModel.m:21).
//
// One thread per ray; each ray only tests the facets whose bounding box
// covers it (per-ray candidate lists built on the host).
// The decisions are exact comparisons of FP64 expressions, so this file is
// compiled without FMA contraction (device: -fmad=false, host:
// -ffp-contract=off) and evaluates every expression in the reference's
// order; the occupancy is then bit-identical to an FP64 evaluation of
// Voxelize.m.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "setup.cuh"

namespace gmgs {
void set_thread_error(const std::string& msg);   // api.cu

namespace {

constexpr int MAXC = 256;             // crossings kept per ray
constexpr int NF = 18;                // per-facet values (SoA planes)
enum { X1, X2, X3, Y1, Y2, Y3, Z1, Z2, Z3, Y1P, Y2P, Y3P, PA, PB, PC, PD, FMINX, FMAXX };
enum { VF_VERTEX = 1, VF_OVERFLOW = 2 };

double mround(double x) { return std::copysign(std::floor(std::fabs(x) + 0.5), x); }

// MATLAB's a:d:b (d > 0): first half a + k d, second half (a + n d) - (n - k) d
std::vector<double> colon(double a, double d, double b) {
    const double q = (b - a) / d;
    const double tol = 2.0 * std::numeric_limits<double>::epsilon() * std::max(std::fabs(a), std::fabs(b)) / d;
    const long n = (long)std::floor(q + tol);
    std::vector<double> v;
    if (n < 0) return v;
    v.resize(n + 1);
    const double c = a + (double)n * d;
    const long half = (n + 1) / 2;
    for (long k = 0; k <= n; ++k) v[k] = k < half ? a + (double)k * d : c - (double)(n - k) * d;
    return v;
}

int nearest(const std::vector<double>& g, double v) {
    double best = std::numeric_limits<double>::infinity();
    int idx = 0;
    for (size_t i = 0; i < g.size(); ++i) {
        const double d = std::fabs(g[i] - v);
        if (d < best) { best = d; idx = (int)i; }
    }
    return idx;
}

// per-facet edge predictions and plane coefficients (Voxelize.m:222-265)
__global__ void k_facet_prep(int64_t m, double* __restrict__ F) {
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < m; f += (int64_t)gridDim.x * blockDim.x) {
        const double x1 = F[X1 * m + f], x2 = F[X2 * m + f], x3 = F[X3 * m + f];
        const double y1 = F[Y1 * m + f], y2 = F[Y2 * m + f], y3 = F[Y3 * m + f];
        const double z1 = F[Z1 * m + f], z2 = F[Z2 * m + f], z3 = F[Z3 * m + f];
        F[Y1P * m + f] = y2 - ((y2 - y3) * (x2 - x1) / (x2 - x3));
        F[Y2P * m + f] = y3 - ((y3 - y1) * (x3 - x2) / (x3 - x1));
        F[Y3P * m + f] = y1 - ((y1 - y2) * (x1 - x3) / (x1 - x2));
        F[PA * m + f] = y1 * (z2 - z3) + y2 * (z3 - z1) + y3 * (z1 - z2);
        F[PB * m + f] = z1 * (x2 - x3) + z2 * (x3 - x1) + z3 * (x1 - x2);
        double pc = x1 * (y2 - y3) + x2 * (y3 - y1) + x3 * (y1 - y2);
        if (fabs(pc) < 1e-14) pc = 0.0;
        F[PC * m + f] = pc;
        F[PD * m + f] = -x1 * (y2 * z3 - y3 * z2) - x2 * (y3 * z1 - y1 * z3) - x3 * (y1 * z2 - y2 * z1);
        F[FMINX * m + f] = fmin(fmin(x1, x2), x3);
        F[FMAXX * m + f] = fmax(fmax(x1, x2), x3);
    }
}

struct RayArgs {
    const double* F;
    int64_t m;
    const double *gx, *gy, *gz;
    int nx, ny, nz;
    int ix0, ix1, iy0, iy1;               // ray window (inclusive)
    const int64_t* ray_ptr;               // candidate facets of window ray t: ray_fac[ray_ptr[t] .. ray_ptr[t+1])
    const int32_t* ray_fac;
    double zlo, zhi;                      // mesh z limits with the 1e-12 margin
    uint8_t* out;                         // [ix][iy][iz]
    uint8_t* odd;                         // [ix][iy]
    int* flags;
};

__device__ __forceinline__ double dmround(double x) { return copysign(floor(fabs(x) + 0.5), x); }

// one ray along z through (gx[ix], gy[iy]) (Voxelize.m:142-302)
__global__ void __launch_bounds__(128) k_rays(RayArgs a) {
    const int wx = a.ix1 - a.ix0 + 1, wy = a.iy1 - a.iy0 + 1;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)wx * wy) return;
    const int ix = a.ix0 + (int)(t % wx), iy = a.iy0 + (int)(t / wx);
    const double xv = a.gx[ix], yv = a.gy[iy];
    const double* F = a.F;
    const int64_t m = a.m;
    double zs[MAXC];
    int nzc = 0;
    for (int64_t k = a.ray_ptr[t]; k < a.ray_ptr[t + 1]; ++k) {
        const int f = a.ray_fac[k];
        if (!(F[FMINX * m + f] <= xv && F[FMAXX * m + f] >= xv)) continue;
        const double x1 = F[X1 * m + f], x2 = F[X2 * m + f], x3 = F[X3 * m + f];
        const double y1 = F[Y1 * m + f], y2 = F[Y2 * m + f], y3 = F[Y3 * m + f];
        if ((x1 == xv && y1 == yv) || (x2 == xv && y2 == yv) || (x3 == xv && y3 == yv)) {
            atomicOr(a.flags, VF_VERTEX);
            return;
        }
        const double yr1 = y2 - ((y2 - y3) * (x2 - xv) / (x2 - x3));
        const double p1 = F[Y1P * m + f];
        if (!((p1 > y1 && yr1 > yv) || (p1 < y1 && yr1 < yv))) continue;
        const double yr2 = y3 - ((y3 - y1) * (x3 - xv) / (x3 - x1));
        const double p2 = F[Y2P * m + f];
        if (!((p2 > y2 && yr2 > yv) || (p2 < y2 && yr2 < yv))) continue;
        const double yr3 = y1 - ((y1 - y2) * (x1 - xv) / (x1 - x2));
        const double p3 = F[Y3P * m + f];
        if (!((p3 > y3 && yr3 > yv) || (p3 < y3 && yr3 < yv))) continue;
        const double z = (-F[PD * m + f] - F[PA * m + f] * xv - F[PB * m + f] * yv) / F[PC * m + f];
        if (!(z >= a.zlo && z <= a.zhi)) continue;
        if (nzc == MAXC) {
            atomicOr(a.flags, VF_OVERFLOW);
            return;
        }
        zs[nzc++] = dmround(z * 1e12) / 1e12;
    }
    if (nzc == 0) return;
    for (int i = 1; i < nzc; ++i) {            // insertion sort, then drop repeats
        const double v = zs[i];
        int j = i - 1;
        while (j >= 0 && zs[j] > v) { zs[j + 1] = zs[j]; --j; }
        zs[j + 1] = v;
    }
    int nu = 1;
    for (int i = 1; i < nzc; ++i)
        if (zs[i] != zs[nu - 1]) zs[nu++] = zs[i];
    const int64_t col = ((int64_t)ix * a.ny + iy) * a.nz;
    if (nu & 1) {
        a.odd[(int64_t)ix * a.ny + iy] = 1;
        return;
    }
    for (int p = 0; p < nu; p += 2)
        for (int k = 0; k < a.nz; ++k)
            if (a.gz[k] > zs[p] && a.gz[k] < zs[p + 1]) a.out[col + k] = 1;
}

// rays with an odd number of crossings, in the order the reference records
// them (y outer, x inner): the voxel is inside when >= 4 of the 8
// neighbouring rays have it inside (Voxelize.m:306-330).  A correction reads
// and writes one z position only, so every z position is an independent
// sequence: one thread per z walks the ordered list.
__global__ void k_correct(uint8_t* out, const int32_t* __restrict__ odd_xy, int n_odd, int nx, int ny, int nz) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nz) return;
    for (int c = 0; c < n_odd; ++c) {
        const int ix = odd_xy[2 * c], iy = odd_xy[2 * c + 1];
        int s = 0;
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy) {
                if (!dx && !dy) continue;
                const int jx = ix + dx, jy = iy + dy;
                if (jx >= 0 && jx < nx && jy >= 0 && jy < ny) s += out[((int64_t)jx * ny + jy) * nz + k];
            }
        if (s >= 4) out[((int64_t)ix * ny + iy) * nz + k] = 1;
    }
}

// majority of the three directions, permuted to (y, x, z) and flipped in y
__global__ void k_vote(const uint8_t* __restrict__ vx, const uint8_t* __restrict__ vy, const uint8_t* __restrict__ vz,
                       int NX, int NY, int NZ, int32_t* __restrict__ occ) {
    const int64_t total = (int64_t)NX * NY * NZ;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int iyo = (int)(i % NY);
        const int64_t r = i / NY;
        const int ix = (int)(r % NX), iz = (int)(r / NX);
        const int iy = NY - 1 - iyo;
        const int v = vz[((int64_t)ix * NY + iy) * NZ + iz] +      // rays along z: [x][y][z]
                      vx[((int64_t)iy * NZ + iz) * NX + ix] +      // rays along x: [y][z][x]
                      vy[((int64_t)iz * NX + ix) * NY + iy];       // rays along y: [z][x][y]
        occ[i] = v >= 2 ? 1 : 0;
    }
}

// one direction: the mesh axes (u, v, w) with rays along w
void ray_direction(const std::vector<double>& mesh, int64_t m, int au, int av, int aw, const std::vector<double>& gu,
                   const std::vector<double>& gv, const std::vector<double>& gw, DevBuf& out, DevBuf& dflags,
                   cudaStream_t st) {
    const int nu = (int)gu.size(), nv = (int)gv.size(), nw = (int)gw.size();
    // facet planes in the ray frame: X = axis u, Y = axis v, Z = axis w
    std::vector<double> F((size_t)NF * m);
    double umin = INFINITY, umax = -INFINITY, vmin = INFINITY, vmax = -INFINITY, wmin = INFINITY, wmax = -INFINITY;
    std::vector<double> fvmin(m), fvmax(m);
    for (int64_t f = 0; f < m; ++f) {
        for (int k = 0; k < 3; ++k) {
            const double u = mesh[(f * 3 + au) * 3 + k], v = mesh[(f * 3 + av) * 3 + k], w = mesh[(f * 3 + aw) * 3 + k];
            F[(X1 + k) * m + f] = u;
            F[(Y1 + k) * m + f] = v;
            F[(Z1 + k) * m + f] = w;
            umin = std::min(umin, u); umax = std::max(umax, u);
            vmin = std::min(vmin, v); vmax = std::max(vmax, v);
            wmin = std::min(wmin, w); wmax = std::max(wmax, w);
        }
        fvmin[f] = std::min(std::min(F[Y1 * m + f], F[Y2 * m + f]), F[Y3 * m + f]);
        fvmax[f] = std::max(std::max(F[Y1 * m + f], F[Y2 * m + f]), F[Y3 * m + f]);
    }
    int ix0 = nearest(gu, umin), ix1 = nearest(gu, umax), iy0 = nearest(gv, vmin), iy1 = nearest(gv, vmax);
    if (ix0 > ix1) std::swap(ix0, ix1);
    if (iy0 > iy1) std::swap(iy0, iy1);
    // candidate facets per ray (Voxelize.m:144-150): min_v <= gv[iy] <= max_v and
    // min_u <= gu[ix] <= max_u, binned by each facet's bounding box
    const int wx = ix1 - ix0 + 1, rows = iy1 - iy0 + 1;
    const int64_t nrays = (int64_t)wx * rows;
    std::vector<int64_t> ptr(nrays + 1, 0);
    std::vector<int> blo(4 * m);
    for (int64_t f = 0; f < m; ++f) {
        const double fumin = std::min(std::min(F[X1 * m + f], F[X2 * m + f]), F[X3 * m + f]);
        const double fumax = std::max(std::max(F[X1 * m + f], F[X2 * m + f]), F[X3 * m + f]);
        int* b = &blo[4 * f];
        b[0] = (int)(std::lower_bound(gu.begin() + ix0, gu.begin() + ix1 + 1, fumin) - gu.begin());
        b[1] = (int)(std::upper_bound(gu.begin() + ix0, gu.begin() + ix1 + 1, fumax) - gu.begin()) - 1;
        b[2] = (int)(std::lower_bound(gv.begin() + iy0, gv.begin() + iy1 + 1, fvmin[f]) - gv.begin());
        b[3] = (int)(std::upper_bound(gv.begin() + iy0, gv.begin() + iy1 + 1, fvmax[f]) - gv.begin()) - 1;
        for (int iy = b[2]; iy <= b[3]; ++iy)
            for (int ix = b[0]; ix <= b[1]; ++ix) ++ptr[(int64_t)(iy - iy0) * wx + (ix - ix0) + 1];
    }
    for (int64_t r = 0; r < nrays; ++r) ptr[r + 1] += ptr[r];
    std::vector<int32_t> fac(std::max<int64_t>(1, ptr[nrays]));
    {
        std::vector<int64_t> pos(ptr.begin(), ptr.end() - 1);
        for (int64_t f = 0; f < m; ++f) {
            const int* b = &blo[4 * f];
            for (int iy = b[2]; iy <= b[3]; ++iy)
                for (int ix = b[0]; ix <= b[1]; ++ix) fac[pos[(int64_t)(iy - iy0) * wx + (ix - ix0)]++] = (int32_t)f;
        }
    }
    DevBuf dF = dalloc(F.size() * sizeof(double)), dgu = dalloc(nu * sizeof(double)), dgv = dalloc(nv * sizeof(double)),
           dgw = dalloc(nw * sizeof(double)), dptr = dalloc(ptr.size() * sizeof(int64_t)),
           dfac = dalloc(fac.size() * sizeof(int32_t)), dodd = dalloc((size_t)nu * nv);
    out = dalloc((size_t)nu * nv * nw);
    GMGS_CUDA(cudaMemcpyAsync(dF.p, F.data(), F.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    GMGS_CUDA(cudaMemcpyAsync(dgu.p, gu.data(), nu * sizeof(double), cudaMemcpyHostToDevice, st));
    GMGS_CUDA(cudaMemcpyAsync(dgv.p, gv.data(), nv * sizeof(double), cudaMemcpyHostToDevice, st));
    GMGS_CUDA(cudaMemcpyAsync(dgw.p, gw.data(), nw * sizeof(double), cudaMemcpyHostToDevice, st));
    GMGS_CUDA(cudaMemcpyAsync(dptr.p, ptr.data(), ptr.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    GMGS_CUDA(cudaMemcpyAsync(dfac.p, fac.data(), fac.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    GMGS_CUDA(cudaMemsetAsync(out.p, 0, (size_t)nu * nv * nw, st));
    GMGS_CUDA(cudaMemsetAsync(dodd.p, 0, (size_t)nu * nv, st));
    k_facet_prep<<<(unsigned)std::min<int64_t>((m + 255) / 256, 4096), 256, 0, st>>>(m, dF.as<double>());
    GMGS_CUDA(cudaGetLastError());
    RayArgs a{dF.as<double>(), m, dgu.as<double>(), dgv.as<double>(), dgw.as<double>(), nu, nv, nw, ix0, ix1, iy0, iy1,
              dptr.as<int64_t>(), dfac.as<int32_t>(), wmin - 1e-12, wmax + 1e-12, out.as<uint8_t>(),
              dodd.as<uint8_t>(), dflags.as<int>()};
    k_rays<<<(unsigned)((nrays + 127) / 128), 128, 0, st>>>(a);
    GMGS_CUDA(cudaGetLastError());
    // the odd rays in the reference's order (y outer, x inner)
    std::vector<uint8_t> odd((size_t)nu * nv);
    GMGS_CUDA(cudaMemcpyAsync(odd.data(), dodd.p, odd.size(), cudaMemcpyDeviceToHost, st));
    GMGS_CUDA(cudaStreamSynchronize(st));
    std::vector<int32_t> odd_xy;
    for (int iy = iy0; iy <= iy1; ++iy)
        for (int ix = ix0; ix <= ix1; ++ix)
            if (odd[(size_t)ix * nv + iy]) { odd_xy.push_back(ix); odd_xy.push_back(iy); }
    if (!odd_xy.empty()) {
        DevBuf dxy = dalloc(odd_xy.size() * sizeof(int32_t));
        GMGS_CUDA(cudaMemcpyAsync(dxy.p, odd_xy.data(), odd_xy.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
        k_correct<<<(nw + 127) / 128, 128, 0, st>>>(out.as<uint8_t>(), dxy.as<int32_t>(), (int)(odd_xy.size() / 2), nu,
                                                   nv, nw);
        GMGS_CUDA(cudaGetLastError());
        GMGS_CUDA(cudaStreamSynchronize(st));
    }
    GMGS_CUDA(cudaStreamSynchronize(st));   // host vectors and temporaries go out of scope
}

}  // namespace

// voxel counts from the bounding box of all vertices (AdaptData4Voxelize.m:7-11)
// and voxel centres from the extent of the facets (Voxelize.m:38-52)
static void grids(const double* vertices, int64_t nv, const std::vector<double>& mesh, int64_t m, int res,
                  int dims[3], std::vector<double> g[3]) {
    double vlo[3], vhi[3], lo[3], hi[3];
    for (int d = 0; d < 3; ++d) { vlo[d] = lo[d] = INFINITY; vhi[d] = hi[d] = -INFINITY; }
    for (int64_t v = 0; v < nv; ++v)
        for (int d = 0; d < 3; ++d) {
            vlo[d] = std::min(vlo[d], vertices[v * 3 + d]);
            vhi[d] = std::max(vhi[d], vertices[v * 3 + d]);
        }
    for (int64_t f = 0; f < m; ++f)
        for (int d = 0; d < 3; ++d)
            for (int k = 0; k < 3; ++k) {
                lo[d] = std::min(lo[d], mesh[(f * 3 + d) * 3 + k]);
                hi[d] = std::max(hi[d], mesh[(f * 3 + d) * 3 + k]);
            }
    double ext[3], emax = 0;
    for (int d = 0; d < 3; ++d) { ext[d] = vhi[d] - vlo[d]; emax = std::max(emax, ext[d]); }
    if (!(emax > 0)) throw Error(GMGS_ERR_INVALID_ARGUMENT, "degenerate mesh bounding box");
    for (int d = 0; d < 3; ++d) {
        dims[d] = (int)mround((double)res * (ext[d] / emax));
        if (dims[d] < 1) throw Error(GMGS_ERR_INVALID_ARGUMENT, "resolution too small for the mesh aspect ratio");
        if (!(hi[d] > lo[d])) throw Error(GMGS_ERR_MESH, "the facets span no volume");
        const double w = (hi[d] - lo[d]) / ((double)dims[d] + 0.5);
        g[d] = colon(lo[d] + w / 2, w, hi[d] - w / 2);
    }
}

}  // namespace gmgs

extern "C" int gmgs_voxelize_mesh(const double* vertices, int64_t nv, const int32_t* faces, int64_t nf,
                                  int32_t finest_resolution, int32_t dims[3], int32_t* occupancy) {
    using namespace gmgs;
    try {
        if (!vertices || !faces || !dims || nv < 3 || nf < 1 || finest_resolution < 1)
            throw Error(GMGS_ERR_INVALID_ARGUMENT, "gmgs_voxelize_mesh: bad arguments");
        if (nf > INT32_MAX) throw Error(GMGS_ERR_INVALID_ARGUMENT, "gmgs_voxelize_mesh: too many faces");
        // meshXYZ(f, axis, vertex) (AdaptData4Voxelize.m:15-18)
        std::vector<double> mesh((size_t)nf * 9);
        for (int64_t f = 0; f < nf; ++f)
            for (int k = 0; k < 3; ++k) {
                const int32_t v = faces[f * 3 + k];
                if (v < 0 || v >= nv) throw Error(GMGS_ERR_INVALID_ARGUMENT, "gmgs_voxelize_mesh: face vertex out of range");
                for (int d = 0; d < 3; ++d) {
                    const double c = vertices[v * 3 + d];
                    if (!std::isfinite(c)) throw Error(GMGS_ERR_NONFINITE, "gmgs_voxelize_mesh: non-finite vertex");
                    mesh[(f * 3 + d) * 3 + k] = c;
                }
            }
        int gdims[3];
        std::vector<double> g[3];
        grids(vertices, nv, mesh, nf, finest_resolution, gdims, g);
        const int NX = (int)g[0].size(), NY = (int)g[1].size(), NZ = (int)g[2].size();
        dims[0] = NY;
        dims[1] = NX;
        dims[2] = NZ;
        if (!occupancy) return GMGS_OK;
        if (NX < 1 || NY < 1 || NZ < 1) throw Error(GMGS_ERR_INVALID_ARGUMENT, "gmgs_voxelize_mesh: empty grid");
        cudaStream_t st;
        GMGS_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } guard{st};
        DevBuf flags = dalloc(sizeof(int)), vx, vy, vz;
        GMGS_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int), st));
        // Voxelize.m:62-80: rays along x in the (y, z) frame, along y in (z, x), along z in (x, y)
        ray_direction(mesh, nf, 1, 2, 0, g[1], g[2], g[0], vx, flags, st);
        ray_direction(mesh, nf, 2, 0, 1, g[2], g[0], g[1], vy, flags, st);
        ray_direction(mesh, nf, 0, 1, 2, g[0], g[1], g[2], vz, flags, st);
        int hflags = 0;
        GMGS_CUDA(cudaMemcpyAsync(&hflags, flags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        GMGS_CUDA(cudaStreamSynchronize(st));
        if (hflags & VF_VERTEX)
            throw Error(GMGS_ERR_MESH, "a ray crosses a mesh vertex exactly; the reference's voxeliser cannot "
                                       "handle this case (Voxelize.m:184 calls an undefined helper)");
        if (hflags & VF_OVERFLOW) throw Error(GMGS_ERR_MESH, "more than 256 mesh crossings on one ray");
        const int64_t total = (int64_t)NX * NY * NZ;
        DevBuf occ = dalloc(total * sizeof(int32_t));
        k_vote<<<(unsigned)std::min<int64_t>((total + 255) / 256, 65535), 256, 0, st>>>(
            vx.as<uint8_t>(), vy.as<uint8_t>(), vz.as<uint8_t>(), NX, NY, NZ, occ.as<int32_t>());
        GMGS_CUDA(cudaGetLastError());
        GMGS_CUDA(cudaMemcpyAsync(occupancy, occ.p, total * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        GMGS_CUDA(cudaStreamSynchronize(st));
        return GMGS_OK;
    } catch (const gmgs::Error& e) {
        set_thread_error(e.what());
        return e.status;
    } catch (const std::bad_alloc&) {
        set_thread_error("host allocation failed");
        return GMGS_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        set_thread_error(e.what());
        return GMGS_ERR_CUDA;
    }
}
