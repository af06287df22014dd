// noalloc.cu -- the residual statistic sqrt(sum res^2)/nshg (the totres of
// phSolver/compressible/rstat.f:108, phgpu_stats.totres of phgpu_solmfg) for
// callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: a host solver that hands all device
// memory to its own pool or to another framework's allocator, a run that is
// not allowed to grow its device footprint after set-up, or a code path that
// must not synchronize the device the way cudaMalloc and cudaFree can.  Such
// a caller owns the input and the output and gives both to this entry point,
// which allocates nothing: its working storage (one partial sum per block and
// a completion counter) is the fixed array g_rstat_scratch below, which every
// GPU that loads the library holds until the process exits.
#include <mutex>

#include "phgpu_impl.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 8;
constexpr long long kTile = (long long)kThreads * kPerThread;  // elements per block
constexpr int kMaxBlocks = PHGPU_RSTAT_NOALLOC_MAX_N / (int)kTile;
static_assert((long long)kMaxBlocks * kTile == PHGPU_RSTAT_NOALLOC_MAX_N, "max size must be whole tiles");

// partial sums of the blocks, then one 64-bit completion counter
static __device__ __align__(256) double g_rstat_scratch[kMaxBlocks + 1];

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ double block_sum(double v) {
    __shared__ double sh[kThreads / 32];
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x < 32) {
        s = threadIdx.x < kThreads / 32 ? sh[threadIdx.x] : 0.0;
        s = warp_sum(s);
    }
    __syncthreads();
    return s;  // valid in thread 0
}

// each block sums the squares of one fixed tile; the last block to finish adds
// the partials in block order, so the result does not depend on scheduling
__global__ void __launch_bounds__(kThreads)
k_rstat_noalloc(const double* __restrict__ r, long long n, double nshg, double* __restrict__ out,
                double* __restrict__ scratch) {
    const long long base = (long long)blockIdx.x * kTile;
    double acc = 0.0;
#pragma unroll
    for (int i = 0; i < kPerThread; ++i) {
        const long long k = base + (long long)i * kThreads + threadIdx.x;
        if (k < n) {
            const double v = r[k];
            acc = fma(v, v, acc);
        }
    }
    const double bs = block_sum(acc);
    unsigned long long* counter = reinterpret_cast<unsigned long long*>(scratch + kMaxBlocks);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        scratch[blockIdx.x] = bs;
        __threadfence();
        last = atomicAdd(counter, 1ull) == (unsigned long long)(gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double v = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) v += ((volatile double*)scratch)[b];
    const double total = block_sum(v);
    if (threadIdx.x == 0) *out = sqrt(total) / nshg;
}

// device address of g_rstat_scratch, looked up once per device
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

}  // namespace

extern "C" int phgpu_rstat_noalloc(const double* res, int nshg, double* totres, void* stream) {
    if (!res || !totres || nshg <= 0) return PHGPU_ERR_INVALID;
    const long long n = 5ll * nshg;
    if (n > PHGPU_RSTAT_NOALLOC_MAX_N) return PHGPU_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PHGPU_ERR_CUDA;
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch_ptr[dev]) {
            // set-up on the first call on this device, with the device current: the
            // symbol is a host-side stand-in, the kernel needs its device address
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_rstat_scratch) != cudaSuccess) return PHGPU_ERR_CUDA;
            g_scratch_ptr[dev] = static_cast<double*>(p);
        }
        scratch = g_scratch_ptr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the scratch array looked up above belongs to the current device: a stream of another device
    // would run the kernel there on this device's address
    int sdev = dev;
    if (s && cudaStreamGetDevice(s, &sdev) == cudaSuccess && sdev != dev) return PHGPU_ERR_INVALID;
    // the completion counter must start at zero; the partials are all rewritten
    if (cudaMemsetAsync(scratch + kMaxBlocks, 0, sizeof(unsigned long long), s) != cudaSuccess)
        return PHGPU_ERR_CUDA;
    const int blocks = (int)((n + kTile - 1) / kTile);
    k_rstat_noalloc<<<blocks, kThreads, 0, s>>>(res, n, (double)nshg, totres, scratch);
    return cudaGetLastError() == cudaSuccess ? PHGPU_OK : PHGPU_ERR_CUDA;
}
