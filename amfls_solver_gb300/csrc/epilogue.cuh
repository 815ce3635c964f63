// Fused epilogue of single-column products (see device_operator.hpp).
#pragma once

#include "common.cuh"
#include "device_operator.hpp"

namespace amfls_gpu {

__device__ __forceinline__ void epilogue_row(const Epilogue& ep, int row, double t, double& sq_t,
                                             double& sq_out, double& dot, double& mx_t,
                                             double& mx_out, int& nonfin) {
    double out = t;
    if (ep.sub_table) {
        const int c = *ep.sub_col;
        out = t - (*ep.coef) * ep.sub_table[c >> 5][(long long)row * 32 + (c & 31)];
    } else if (ep.sub) out = t - (*ep.coef) * ep.sub[(long long)row * ep.sub_stride];
    else if (ep.fma_vec) out = fma(ep.lambda, ep.fma_vec[row], t);
    else if (ep.minus_vec) out = t - ep.minus_vec[row];
    if (ep.t_out) ep.t_out[row] = t;
    if (ep.out) ep.out[row] = out;
    if (ep.red) {
        sq_t = fma(t, t, sq_t);
        sq_out = fma(out, out, sq_out);
        if (ep.dot_vec) dot = fma(out, ep.dot_vec[row], dot);
        // fmax(mx, |v|) (NaN ignored) and the finiteness test on the bit
        // patterns, off the FP64 pipe: magnitudes of non-NaN doubles order
        // like their bits, and mx starts at +0 so it is never NaN
        constexpr unsigned long long kInf = 0x7ff0000000000000ull;
        const unsigned long long at = __double_as_longlong(t) & 0x7fffffffffffffffull;
        const unsigned long long ao = __double_as_longlong(out) & 0x7fffffffffffffffull;
        const unsigned long long mt = __double_as_longlong(mx_t), mo = __double_as_longlong(mx_out);
        if (at <= kInf && at > mt) mx_t = __longlong_as_double(at);
        if (ao <= kInf && ao > mo) mx_out = __longlong_as_double(ao);
        if (at >= kInf || ao >= kInf) ++nonfin;
    }
}

// Maximum / sum over a block of 64-bit integers (warp shuffles, then warp 0),
// valid in warp 0.  Integer pipes: the FP64 pipe of this GPU is scarce.
__device__ inline unsigned long long block_umax(unsigned long long v, unsigned long long* sc) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sc[warp] = v;
    __syncthreads();
    unsigned long long r = 0;
    if (warp == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sc[lane] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w = __shfl_xor_sync(0xffffffffu, r, o);
            r = w > r ? w : r;
        }
    }
    return r;
}

__device__ inline unsigned long long block_usum(unsigned long long v, unsigned long long* sc) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sc[warp] = v;
    __syncthreads();
    unsigned long long r = 0;
    if (warp == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sc[lane] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;
}

// Cross-block reduction of the epilogue terms into *ep.red.  The sums run on
// the FP64 pipe in a fixed tree; the maxima (non-negative magnitudes, so
// their bit patterns order like their values) and the non-finite count run
// on the integer pipes, with the results fmax / a count would give.  Per
// block: 6 slots of `partials` (maxima and count stored as bit patterns).
__device__ inline void finish_reduction(const Epilogue& ep, double sq_t, double sq_out, double dot,
                                 double mx_t, double mx_out, int nonfin, double* partials,
                                 unsigned* counter) {
    __shared__ double scratch[32];
    __shared__ unsigned long long uscratch[32];
    if (!ep.red) return;
    const double s0 = block_sum(sq_t, scratch);
    const double s1 = block_sum(sq_out, scratch);
    const double s2 = block_sum(dot, scratch);
    const unsigned long long m3 = block_umax(__double_as_longlong(mx_t), uscratch);
    const unsigned long long m4 = block_umax(__double_as_longlong(mx_out), uscratch);
    const unsigned long long c5 = block_usum((unsigned long long)nonfin, uscratch);
    if (threadIdx.x == 0) {
        double* p = partials + blockIdx.x * 6;
        p[0] = s0;
        p[1] = s1;
        p[2] = s2;
        p[3] = __longlong_as_double(m3);
        p[4] = __longlong_as_double(m4);
        p[5] = __longlong_as_double(c5);
    }
    if (arrive_last(counter, gridDim.x)) {
        double a[3] = {0.0, 0.0, 0.0};
        unsigned long long mx[2] = {0ull, 0ull}, cnt = 0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
            const double* p = partials + b * 6;
            a[0] += p[0];
            a[1] += p[1];
            a[2] += p[2];
            const unsigned long long x3 = __double_as_longlong(p[3]);
            const unsigned long long x4 = __double_as_longlong(p[4]);
            mx[0] = x3 > mx[0] ? x3 : mx[0];
            mx[1] = x4 > mx[1] ? x4 : mx[1];
            cnt += __double_as_longlong(p[5]);
        }
        const double r0 = block_sum(a[0], scratch);
        const double r1 = block_sum(a[1], scratch);
        const double r2 = block_sum(a[2], scratch);
        const unsigned long long r3 = block_umax(mx[0], uscratch);
        const unsigned long long r4 = block_umax(mx[1], uscratch);
        const unsigned long long r5 = block_usum(cnt, uscratch);
        if (threadIdx.x == 0) {
            ep.red->sq_t = r0;
            ep.red->sq_out = r1;
            ep.red->dot = r2;
            ep.red->max_t = __longlong_as_double(r3);
            ep.red->max_out = __longlong_as_double(r4);
            ep.red->nonfinite = (int)r5;
        }
    }
}


}  // namespace amfls_gpu
