// Allocation-free dense transpose product: x = A^T y for a row-major A.
//
// For callers that cannot call cudaMalloc: code running while a CUDA stream
// is being captured into a graph (allocation is not a capturable operation),
// real-time loops that must never synchronise the device (cudaMalloc and
// cudaFree may), and hosts whose memory manager owns every device byte and
// forbids a library from allocating behind its back.  The regular path
// (amfls_gpu_dense_operator_create + amfls_gpu_operator_apply_transpose)
// allocates its partial-sum scratch when the operator is created; this entry
// point takes the matrix directly and keeps those partial sums in one
// fixed-size array in device global memory that every GPU loading the
// library holds until the process exits.
//
// The product splits the rows of A into chunks; a first kernel writes one
// partial sum per (chunk, column) into the array, a second adds the chunks
// in a fixed order.  Every partial is written before it is read, so nothing
// has to start at zero, but calls share the array: two calls whose kernels
// overlap on the GPU (different streams, no ordering between them) race on
// it and return garbage.  Calls on one stream are ordered and safe.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../../include/amfls_gpu.h"
#include "common.cuh"

namespace amfls_gpu {
namespace {

// 1 Mi doubles (8 MiB): chunks * cols must fit.
constexpr long long kNoAllocScratchDoubles = 1LL << 20;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};
int g_sm_count[kMaxDevices] = {};

// Device address of the scratch array on the current device, and that
// device's SM count (for the launch sizes).  Looked up once per device (with
// that device current) and cached for the life of the process: the name of
// the array in host code is only a host-side stand-in, not a device address.
// The cached address belongs to the device's primary context; a
// cudaDeviceReset (or any other teardown of that context) invalidates it.
double* scratch_on_current_device(int* sm_count) {
    int dev = -1;
    AMFLS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_ptr[dev] == nullptr) {
        void* ptr = nullptr;
        AMFLS_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_partials));
        int sms = 0;
        AMFLS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        g_sm_count[dev] = std::max(1, sms);
        g_scratch_ptr[dev] = static_cast<double*>(ptr);
    }
    *sm_count = g_sm_count[dev];
    return g_scratch_ptr[dev];
}

__global__ void noalloc_chunk_sums(const double* __restrict__ a, int rows, int cols, int chunk,
                                   const double* __restrict__ y, double* partial) {
    const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (col >= cols) return;
    const int r0 = c * chunk, r1 = min(rows, r0 + chunk);
    double acc = 0.0;
    for (int r = r0; r < r1; ++r) acc = fma(a[(long long)r * cols + col], __ldg(y + r), acc);
    partial[(long long)c * cols + col] = acc;
}

__global__ void noalloc_add_chunks(const double* partial, int chunks, int cols, double* x) {
    for (long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x; col < cols;
         col += (long long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < chunks; ++c) s += partial[(long long)c * cols + col];
        x[col] = s;
    }
}

}  // namespace

// defined in capi.cu: the thread's message for amfls_gpu_last_error()
void set_last_error(const std::string& message);

}  // namespace amfls_gpu

extern "C" int amfls_gpu_dense_apply_transpose_noalloc(int rows, int cols, const double* d_values,
                                                       const double* d_y, double* d_x,
                                                       void* stream) {
    using namespace amfls_gpu;
    try {
        if (rows <= 0 || cols <= 0 || d_values == nullptr || d_y == nullptr || d_x == nullptr)
            throw std::invalid_argument("dense no-alloc transpose product: invalid arguments");
        if (cols > kNoAllocScratchDoubles)
            throw std::length_error(
                "dense no-alloc transpose product: cols = " + std::to_string(cols) +
                " exceeds the fixed scratch of " + std::to_string(kNoAllocScratchDoubles) +
                " doubles; use amfls_gpu_operator_apply_transpose instead");
        int sms = 1;
        double* scratch = scratch_on_current_device(&sms);
        // as many row chunks as fill the GPU (8 blocks per SM), bounded by the
        // scratch capacity
        const int col_blocks = (cols + 255) / 256;
        const int target_blocks = 8 * sms;
        long long chunks = std::max(1, std::min((target_blocks + col_blocks - 1) / col_blocks,
                                                (rows + 63) / 64));
        chunks = std::min<long long>(chunks, kNoAllocScratchDoubles / cols);
        const int chunk = static_cast<int>((rows + chunks - 1) / chunks);
        chunks = (rows + chunk - 1) / chunk;
        const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        noalloc_chunk_sums<<<dim3(col_blocks, static_cast<unsigned>(chunks)), 256, 0, s>>>(
            d_values, rows, cols, chunk, d_y, scratch);
        AMFLS_LAUNCHED();
        noalloc_add_chunks<<<std::max(1, std::min(col_blocks, target_blocks)), 256, 0, s>>>(
            scratch, static_cast<int>(chunks), cols, d_x);
        AMFLS_LAUNCHED();
        set_last_error("");
        return AMFLS_GPU_OK;
    } catch (const std::invalid_argument& e) {
        set_last_error(e.what());
        return AMFLS_GPU_INVALID_ARGUMENT;
    } catch (const std::length_error& e) {
        set_last_error(e.what());
        return AMFLS_GPU_LENGTH_ERROR;
    } catch (const CudaError& e) {
        set_last_error(e.what());
        return AMFLS_GPU_CUDA_ERROR;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return AMFLS_GPU_RUNTIME_ERROR;
    }
}
