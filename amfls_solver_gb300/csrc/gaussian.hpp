#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace amfls_gpu {

std::uint64_t gaussian_key(std::uint64_t seed, std::uint64_t stream);

// rows x cols standard normals (column-major, leading dimension ld) for global
// columns first_column, first_column+1, ...
void gaussian_block(int rows, int cols, std::uint64_t seed, std::uint64_t stream,
                    std::uint64_t first_column, double* d_out, long long ld, cudaStream_t s);

}  // namespace amfls_gpu

namespace amfls_gpu {
// Remove the component along b/||b|| from each column of R (rows x cols).
void project_out_direction(double* R, int rows, int cols, const double* b, double bnorm,
                           cudaStream_t s);
}  // namespace amfls_gpu
