// bt_signal_noalloc: the signal functional S = sum_i w[i] Re(u[i]) of a state
// that already lives on the GPU, computed without allocating memory.
//
// Why it exists: some callers cannot allocate device memory at the moment they
// need a signal -- a host loop that runs inside CUDA stream capture (a
// cudaMalloc there invalidates the capture), a real-time acquisition or
// serving thread whose allocator is frozen after start-up, or code running
// under a memory pool that forbids growth.  The regular path (bt_solve, and the
// deterministic sums behind bt_solve's S0) allocates its block partials per
// call; this entry point keeps them in a file-scope device array instead.
//
// Scratch: kNoAllocMaxBlocks doubles (8 KB) in a static __device__ array.  Every
// GPU that loads the library holds it until the process exits.  Host code must
// not take the address of the array directly (the host-side symbol is only a
// stand-in): the first call on each device, with that device current, looks up
// its device address with cudaGetSymbolAddress and caches it.  That first call
// should therefore happen before any stream capture begins.  The cache is keyed
// by the device's current CUDA context as well (its unique id, read through the
// driver entry point cuCtxGetId): after cudaDeviceReset the module is loaded
// again, possibly at another address, and the next call looks the address up
// again -- so after a reset, too, make one call before capturing.
//
// Limits and sharing: n must be at most kNoAllocMaxBlocks * kNoAllocPerBlock
// elements (2,097,152 dofs); larger inputs are rejected.  Every call on a
// device shares the one scratch array and leaves its partials in it; each call
// overwrites exactly the partials it reads, so nothing needs clearing, but
// calls that overlap on the GPU (different streams, no ordering) race on the
// scratch and must be serialised by the caller.
#include "bt_common.cuh"

#include <mutex>

namespace bt {

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocItems = 8;  // elements per thread
constexpr int kNoAllocPerBlock = kNoAllocThreads * kNoAllocItems;
constexpr int kNoAllocMaxBlocks = 1024;
constexpr int kMaxDevices = 64;

// The scratch: block partial sums of the first pass.
static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxBlocks];

// pass 1: block b sums w[i] * u[2i] over its kNoAllocPerBlock elements
__global__ void __launch_bounds__(kNoAllocThreads)
k_signal_partials(const double* __restrict__ w, const double* __restrict__ u, int64_t n,
                  double* __restrict__ partials) {
    __shared__ double sm[32];
    double acc[1] = {0.0};
    const int64_t base = (int64_t)blockIdx.x * kNoAllocPerBlock;
#pragma unroll
    for (int k = 0; k < kNoAllocItems; ++k) {
        const int64_t i = base + (int64_t)k * kNoAllocThreads + threadIdx.x;
        if (i < n) acc[0] += w[i] * u[2 * i];
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}

// pass 2: one block adds the partials in block order
__global__ void __launch_bounds__(kNoAllocThreads)
k_signal_finish(const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
    __shared__ double sm[32];
    double acc[1] = {0.0};
    for (int b = threadIdx.x; b < nblocks; b += kNoAllocThreads) acc[0] += partials[b];
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) *out = acc[0];
}

std::mutex g_noalloc_mutex;
double* g_noalloc_addr[kMaxDevices] = {nullptr};
unsigned long long g_noalloc_ctx[kMaxDevices] = {0};

// Unique id of the calling thread's current CUDA context (0 when the driver
// does not provide it).  Context ids are never reused within a process, so a
// changed id means the cached symbol address may be stale.
unsigned long long current_context_id() {
    using GetCurrentFn = int (*)(void**);
    using GetIdFn = int (*)(void*, unsigned long long*);
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<GetCurrentFn>(f1);
            get_id = reinterpret_cast<GetIdFn>(f2);
        }
        looked_up = true;
    }
    if (!get_current || !get_id) return 0;
    void* c = nullptr;
    unsigned long long id = 0;
    if (get_current(&c) != 0 || !c || get_id(c, &id) != 0) return 0;
    return id;
}

}  // namespace

}  // namespace bt

extern "C" int bt_signal_noalloc(const double* d_weights, const double* d_u, int64_t n, double* d_signal,
                                 void* cuda_stream) {
    using namespace bt;
    if (!d_weights || !d_u || !d_signal || n < 1) return BT_ERR_INVALID;
    if (n > (int64_t)kNoAllocMaxBlocks * kNoAllocPerBlock) return BT_ERR_INVALID;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return BT_ERR_CUDA;
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        const unsigned long long cid = current_context_id();
        if (!g_noalloc_addr[dev] || g_noalloc_ctx[dev] != cid) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || !p) return BT_ERR_CUDA;
            g_noalloc_addr[dev] = static_cast<double*>(p);
            g_noalloc_ctx[dev] = current_context_id();   // the lookup may have created the context
        }
        scratch = g_noalloc_addr[dev];
    }
    const int nblocks = (int)((n + kNoAllocPerBlock - 1) / kNoAllocPerBlock);
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    k_signal_partials<<<nblocks, kNoAllocThreads, 0, s>>>(d_weights, d_u, n, scratch);
    k_signal_finish<<<1, kNoAllocThreads, 0, s>>>(scratch, nblocks, d_signal);
    return cudaGetLastError() == cudaSuccess ? BT_OK : BT_ERR_CUDA;
}
