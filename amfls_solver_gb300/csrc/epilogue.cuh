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

__device__ inline void finish_reduction(const Epilogue& ep, double sq_t, double sq_out, double dot,
                                 double mx_t, double mx_out, int nonfin, double* partials,
                                 unsigned* counter) {
    __shared__ double scratch[32];
    if (!ep.red) return;
    double v[6] = {sq_t, sq_out, dot, mx_t, mx_out, (double)nonfin};
    double r[6];
    for (int i = 0; i < 6; ++i)
        r[i] = (i == 3 || i == 4) ? block_max(v[i], scratch) : block_sum(v[i], scratch);
    if (threadIdx.x == 0)
        for (int i = 0; i < 6; ++i) partials[blockIdx.x * 6 + i] = r[i];
    if (arrive_last(counter, gridDim.x)) {
        for (int i = 0; i < 6; ++i) {
            double a = (i == 3 || i == 4) ? 0.0 : 0.0;
            for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
                const double p = partials[b * 6 + i];
                a = (i == 3 || i == 4) ? fmax(a, p) : a + p;
            }
            r[i] = (i == 3 || i == 4) ? block_max(a, scratch) : block_sum(a, scratch);
        }
        if (threadIdx.x == 0) {
            ep.red->sq_t = r[0];
            ep.red->sq_out = r[1];
            ep.red->dot = r[2];
            ep.red->max_t = r[3];
            ep.red->max_out = r[4];
            ep.red->nonfinite = (int)r[5];
        }
    }
}


}  // namespace amfls_gpu
