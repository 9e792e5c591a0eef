// Allocation-free inner product (gmgs_dot_dev_noalloc in include/gmgs.h).
//
// For callers that cannot allocate device memory: hosts whose device memory
// belongs to their own allocator (a MATLAB MEX shim working on gpuArray
// buffers, a framework whose caching allocator must see every allocation) and
// code paths that cannot afford the implicit device synchronisation of
// cudaMalloc / cudaFree.  The block partials and the arrival counter of the
// deterministic reduction live in a fixed static device array instead of
// per-handle scratch, so the call allocates nothing.
#include "gmgs_internal.cuh"

namespace gmgs {
void set_thread_error(const std::string& msg);   // api.cu
}

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 8192;                                   // elements reduced by one block
constexpr int kMaxPartials = 65536;                            // blocks per call
constexpr long long kMaxN = (long long)kChunk * kMaxPartials;  // 536,870,912 elements
static_assert(kMaxN == GMGS_DOT_NOALLOC_MAX_N, "limit must match the header");

// Block partials in [0, kMaxPartials), the arrival counter in the next slot.
// Every GPU that loads the library holds these 512 KiB until the process exits.
static __device__ __align__(256) double g_noalloc_scratch[kMaxPartials + 32];

__global__ void __launch_bounds__(kThreads) k_dot_noalloc(const double* __restrict__ x, const double* __restrict__ y,
                                                          long long n, double* __restrict__ scratch,
                                                          double* __restrict__ result) {
    __shared__ double sh[kThreads / 32];
    __shared__ bool last;
    const long long base = (long long)blockIdx.x * kChunk;
    double s = 0.0;
    for (int k = threadIdx.x; k < kChunk; k += kThreads) {
        const long long i = base + k;
        if (i < n) s += x[i] * y[i];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = s;
    __syncthreads();
    if (w == 0) {
        s = l < kThreads / 32 ? sh[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    }
    unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + kMaxPartials);
    if (threadIdx.x == 0) {
        scratch[blockIdx.x] = s;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // the last block to arrive sums the partials in block order: the result
    // does not depend on scheduling
    __threadfence();
    double t = 0.0;
    for (unsigned int i = threadIdx.x; i < gridDim.x; i += kThreads) t += ((volatile double*)scratch)[i];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    __syncthreads();
    if (l == 0) sh[w] = t;
    __syncthreads();
    if (w == 0) {
        t = l < kThreads / 32 ? sh[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (l == 0) {
            *result = t;
            *counter = 0u;
        }
    }
}

// Device address of the static scratch for the current device and context.
// A host-side reference to the array's name is not a device address, so the
// address is looked up on every call: after the module is loaded on a device
// (the first call there) the lookup is a cheap table query, and a pointer
// cached by device ordinal could outlive a cudaDeviceReset or a change of
// the current context.
int scratch_for_current_device(double** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        gmgs::set_thread_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return GMGS_ERR_CUDA;
    }
    *out = static_cast<double*>(p);
    return GMGS_OK;
}

}  // namespace

extern "C" int gmgs_dot_dev_noalloc(const double* x, const double* y, int64_t n, double* result, void* stream) {
    if (!x || !y || !result || n < 0) {
        gmgs::set_thread_error("gmgs_dot_dev_noalloc: NULL pointer or negative length");
        return GMGS_ERR_INVALID_ARGUMENT;
    }
    if (n > kMaxN) {
        gmgs::set_thread_error("gmgs_dot_dev_noalloc: n exceeds GMGS_DOT_NOALLOC_MAX_N (536,870,912); "
                               "use gmgs_dot_dev for longer vectors");
        return GMGS_ERR_INVALID_ARGUMENT;
    }
    double* scratch = nullptr;
    const int st = scratch_for_current_device(&scratch);
    if (st != GMGS_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (n == 0) {
        e = cudaMemsetAsync(result, 0, sizeof(double), s);
    } else {
        // the arrival counter must start at zero
        e = cudaMemsetAsync(scratch + kMaxPartials, 0, sizeof(unsigned int), s);
        if (e == cudaSuccess) {
            const unsigned int blocks = (unsigned int)((n + kChunk - 1) / kChunk);
            k_dot_noalloc<<<blocks, kThreads, 0, s>>>(x, y, (long long)n, scratch, result);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        gmgs::set_thread_error(std::string("gmgs_dot_dev_noalloc: ") + cudaGetErrorString(e));
        return GMGS_ERR_CUDA;
    }
    return GMGS_OK;
}
