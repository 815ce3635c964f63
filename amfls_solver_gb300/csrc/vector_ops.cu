#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "vector_ops.hpp"

namespace amfls_gpu {
namespace {

constexpr int kThreads = 256;

__global__ void max_pass_kernel(VectorSet set, NormResult* out, double* partials,
                                unsigned* counter) {
    __shared__ double scratch[32];
    for (int v = 0; v < set.count; ++v) {
        double mx = 0.0, bad = 0.0;
        const double* x = set.v[v];
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < set.n[v];
             i += (long long)gridDim.x * blockDim.x) {
            const double a = x[i];
            if (!isfinite(a)) bad += 1.0;
            else mx = fmax(mx, fabs(a));
        }
        const double bm = block_max(mx, scratch);
        const double bb = block_sum(bad, scratch);
        if (threadIdx.x == 0) {
            partials[(2 * v) * gridDim.x + blockIdx.x] = bm;
            partials[(2 * v + 1) * gridDim.x + blockIdx.x] = bb;
        }
    }
    if (arrive_last(counter, gridDim.x)) {
        for (int v = 0; v < set.count; ++v) {
            double mx = 0.0, bad = 0.0;
            for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
                mx = fmax(mx, partials[(2 * v) * gridDim.x + b]);
                bad += partials[(2 * v + 1) * gridDim.x + b];
            }
            mx = block_max(mx, scratch);
            bad = block_sum(bad, scratch);
            if (threadIdx.x == 0) {
                out->max_abs[v] = mx;
                out->nonfinite[v] = bad > 0.0 ? 1 : 0;
                int e = 0;
                if (mx > 0.0) (void)frexp(mx, &e);
                out->exponent[v] = e;
                out->count[v] = set.n[v];
            }
        }
    }
}

__global__ void sum_pass_kernel(VectorSet set, NormResult* out, double* partials,
                                unsigned* counter) {
    __shared__ double scratch[32];
    for (int v = 0; v < set.count; ++v) {
        const int e = out->exponent[v];
        const bool skip = out->nonfinite[v] != 0 || out->max_abs[v] == 0.0;
        double acc = 0.0;
        const double* x = set.v[v];
        if (!skip) {
            for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < set.n[v];
                 i += (long long)gridDim.x * blockDim.x) {
                const double s = scalbn(fabs(x[i]), -e);
                acc = fma(s, s, acc);
            }
        }
        const double bs = block_sum(acc, scratch);
        if (threadIdx.x == 0) partials[v * gridDim.x + blockIdx.x] = bs;
    }
    if (arrive_last(counter, gridDim.x)) {
        for (int v = 0; v < set.count; ++v) {
            double acc = 0.0;
            for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
                acc += partials[v * gridDim.x + b];
            acc = block_sum(acc, scratch);
            if (threadIdx.x == 0) out->scaled_sumsq[v] = acc;
        }
    }
}

}  // namespace

void norm_passes(const VectorSet& set, NormResult* out, double* partials, unsigned* counter,
                 cudaStream_t stream) {
    long long longest = 1;
    for (int i = 0; i < set.count; ++i) longest = std::max(longest, set.n[i]);
    const int grid = (int)std::max<long long>(1, std::min<long long>(grid_cap(), (longest + 1023) / 1024));
    max_pass_kernel<<<grid, kThreads, 0, stream>>>(set, out, partials, counter);
    AMFLS_LAUNCHED();
    sum_pass_kernel<<<grid, kThreads, 0, stream>>>(set, out, partials, counter);
    AMFLS_LAUNCHED();
}

double euclid_from(const NormResult& r, int i) {
    if (r.nonfinite[i]) return NAN;
    if (r.max_abs[i] == 0.0) return 0.0;
    return std::ldexp(std::sqrt(r.scaled_sumsq[i]), r.exponent[i]);
}

}  // namespace amfls_gpu
