// Counter-addressed standard normals on the device.
//
// Same stream as the reference's gaussian_matrix
// (src/algorithms/mathematics/random/gaussian.cpp:13-55): entry (row, col) of
// a block whose first global column is `first` uses index
// (first + col) * rows + row, key = mix(seed) ^ mix(stream + 0xd2b74407b1ce6e93),
// two open-interval uniforms from mix(key ^ 2i) and mix(key ^ (2i+1)) (the
// splitmix64 finaliser, 53-bit mantissa, +1 so zero never occurs) and the
// Box-Muller cosine branch.  The device's log and cos are within a few ulp of
// the host libm's, so entries match the reference to ~1e-15 relative.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "gaussian.hpp"

namespace amfls_gpu {
namespace {

__device__ __forceinline__ std::uint64_t mix64(std::uint64_t v) {
    v += 0x9e3779b97f4a7c15ULL;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31);
}

__device__ __forceinline__ double unit_open(std::uint64_t bits) {
    return static_cast<double>((bits >> 11) + 1ULL) * (1.0 / 9007199254740992.0);
}

__global__ void gaussian_kernel(int rows, int cols, std::uint64_t key, std::uint64_t first,
                                double* out, long long ld) {
    const long long total = (long long)rows * cols;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t / rows);
        const int r = (int)(t % rows);
        const std::uint64_t idx = (first + (std::uint64_t)c) * (std::uint64_t)rows + (std::uint64_t)r;
        const double u1 = unit_open(mix64(key ^ (2ULL * idx)));
        const double u2 = unit_open(mix64(key ^ (2ULL * idx + 1ULL)));
        out[(long long)c * ld + r] =
            sqrt(-2.0 * log(u1)) * cos(6.283185307179586476925286766559 * u2);
    }
}

}  // namespace

std::uint64_t gaussian_key(std::uint64_t seed, std::uint64_t stream) {
    auto mix = [](std::uint64_t v) {
        v += 0x9e3779b97f4a7c15ULL;
        v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
        v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
        return v ^ (v >> 31);
    };
    return mix(seed) ^ mix(stream + 0xd2b74407b1ce6e93ULL);
}

void gaussian_block(int rows, int cols, std::uint64_t seed, std::uint64_t stream,
                    std::uint64_t first_column, double* d_out, long long ld, cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return;
    const long long total = (long long)rows * cols;
    const int grid = (int)std::min<long long>(2432, (total + 255) / 256);
    gaussian_kernel<<<grid, 256, 0, s>>>(rows, cols, gaussian_key(seed, stream), first_column,
                                         d_out, ld);
    AMFLS_LAUNCHED();
}

}  // namespace amfls_gpu

namespace amfls_gpu {
namespace {

// dots[c] = sum_i (b_i / ||b||) R[i, c]   (one block per column chunk)
__global__ void direction_dots_kernel(const double* R, int rows, int cols, const double* b,
                                      double bnorm, double* dots) {
    __shared__ double scratch[32];
    for (int c = blockIdx.x; c < cols; c += gridDim.x) {
        double s = 0.0;
        for (int i = threadIdx.x; i < rows; i += blockDim.x)
            s = fma(b[i] / bnorm, R[(long long)c * rows + i], s);
        s = block_sum(s, scratch);
        if (threadIdx.x == 0) dots[c] = s;
        __syncthreads();
    }
}

__global__ void direction_update_kernel(double* R, int rows, int cols, const double* b,
                                        double bnorm, const double* dots) {
    const long long total = (long long)rows * cols;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t / rows);
        const int i = (int)(t % rows);
        R[t] -= dots[c] * (b[i] / bnorm);
    }
}

}  // namespace

// Project b/||b|| out of every column (amfls.cpp:205-229).
void project_out_direction(double* R, int rows, int cols, const double* b, double bnorm,
                           cudaStream_t s) {
    if (!(bnorm != 0.0) || cols <= 0) return;
    double* dots = nullptr;
    AMFLS_CUDA(cudaMallocAsync(&dots, sizeof(double) * cols, s));
    direction_dots_kernel<<<std::min(cols, grid_cap()), 256, 0, s>>>(R, rows, cols, b, bnorm, dots);
    AMFLS_LAUNCHED();
    const long long total = (long long)rows * cols;
    direction_update_kernel<<<(int)std::min<long long>(2432, (total + 255) / 256), 256, 0, s>>>(
        R, rows, cols, b, bnorm, dots);
    AMFLS_LAUNCHED();
    AMFLS_CUDA(cudaFreeAsync(dots, s));
}

}  // namespace amfls_gpu
