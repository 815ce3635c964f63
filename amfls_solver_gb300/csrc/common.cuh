// Shared device/host helpers for the GB300 AMFLS library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

namespace amfls_gpu {

// Host-side CUDA error check that turns a failure into an exception; the
// C ABI layer converts it into an error code and a message.
struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
    }
}

#define AMFLS_CUDA(call) ::amfls_gpu::check_cuda((call), #call)

// Kernel launches made by this thread (reported per solve).  Launch sites
// use AMFLS_LAUNCHED() right after the <<<...>>> statement.
inline long long& launch_count() {
    static thread_local long long count = 0;
    return count;
}

#define AMFLS_LAUNCHED()                                             \
    do {                                                             \
        ::amfls_gpu::check_cuda(cudaGetLastError(), "kernel launch"); \
        ++::amfls_gpu::launch_count();                               \
    } while (0)

// Stream-ordered device allocation from the device's default memory pool.
// A solve allocates and frees its buffers on its own stream: unlike
// cudaFree, cudaFreeAsync does not synchronise the whole device, so solves
// running concurrently on different streams do not stall each other.
template <typename T>
inline void stream_alloc(T** p, size_t bytes, cudaStream_t s) {
    check_cuda(cudaMallocAsync(reinterpret_cast<void**>(p), bytes, s), "cudaMallocAsync");
}
inline void stream_free(const void* p, cudaStream_t s) {
    if (p) cudaFreeAsync(const_cast<void*>(p), s);
}

// Keeps freed blocks of the current device's default memory pool cached in
// the process (release threshold = unlimited) instead of returning them to
// the driver at every synchronisation, so consecutive solves reuse their
// buffers.  Called by each solve; takes effect once per device.
void keep_pool_memory();

// Waits until the work enqueued on `stream` so far has finished, blocking the
// calling thread on a blocking-sync event instead of spinning (concurrent
// solves on many host threads then leave the CPU cores to the threads that
// launch work).
void stream_wait(cudaStream_t stream);

// Streaming multiprocessors of the current device
// (cudaDevAttrMultiProcessorCount), queried once per device.
inline int sm_count() {
    static int cached[64] = {};
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    const int slot = dev >= 0 && dev < 64 ? dev : 0;
    int v = __atomic_load_n(&cached[slot], __ATOMIC_RELAXED);
    if (v == 0) {
        check_cuda(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev),
                   "cudaDeviceGetAttribute(MultiProcessorCount)");
        v = v > 0 ? v : 1;
        __atomic_store_n(&cached[slot], v, __ATOMIC_RELAXED);
    }
    return v;
}

// Grid cap of the grid-stride and reduction kernels: eight resident
// 256-thread blocks per SM.
inline int grid_cap() { return 8 * sm_count(); }

// Upper bound of grid_cap() (devices of up to 256 SMs), for sizing the
// per-block partial-sum scratch that is allocated once.
constexpr int kMaxGridCap = 8 * 256;

constexpr int kWarp = 32;
constexpr int kPanel = 32;  // columns per V panel (row-major n x 32 tiles)

__host__ __device__ inline long long ceil_div(long long a, long long b) {
    return (a + b - 1) / b;
}

#if defined(__CUDACC__)
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Sum over all threads of a block (blockDim.x multiple of 32, <= 1024).
// Fixed reduction tree, so the result is deterministic for a fixed launch.
__device__ inline double block_sum(double v, double* scratch32) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch32[warp] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    double r = 0.0;
    if (warp == 0) {
        r = lane < nw ? scratch32[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;  // valid in warp 0
}

__device__ inline double block_max(double v, double* scratch32) {
    v = warp_max(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch32[warp] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    double r = 0.0;
    if (warp == 0) {
        r = lane < nw ? scratch32[lane] : 0.0;
        r = warp_max(r);
    }
    return r;
}

// "Last block done" pattern: every block writes its partial, the block that
// arrives last (by an atomic ticket) sees all partials after a fence.
// Returns true in the last block; the counter is reset for the next launch.
__device__ inline bool arrive_last(unsigned int* counter, unsigned int nblocks) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int ticket = atomicAdd(counter, 1u);
        last = (ticket == nblocks - 1);
        if (last) *counter = 0u;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}
#endif

}  // namespace amfls_gpu
