// Row-vector CSR products: one column, fused epilogue, rows grouped by
// length.
//
// The rows of a side are binned by length into six bins of g = 32, 16, 8, 4,
// 2, 1 lanes per row (g = the largest power of two <= length / 16, at most
// 32), and within a bin ordered longest first (a stable order, fixed when the
// operator is built).  A warp task is 32 / g rows of one bin; the warps of a
// resident grid take tasks round robin, heaviest bins first.  In a task each
// group of g lanes sums one row: lane l of the group takes elements
// l, l + g, l + 2g, ... as a sequential FMA chain (four elements' indices,
// values and x gathers in flight before their FMAs), then the group adds its
// lanes with a fixed butterfly.  Rows of fewer than 32 nonzeros (g = 1) are
// therefore one lane's sequential chain in storage order, the reference's
// order (sparse_csr_operator.cpp:203-235), and come out bit for bit equal to
// it; longer rows are summed in a different, fixed order.
//
// Why this shape on this GPU: its FP64 pipe retires two lanes' FMAs per SM
// clock and charges a warp instruction in full however few lanes are active,
// so every FMA instruction should carry 32 useful lanes.  Length-sorted bins
// keep the lanes of a warp on rows of nearly the same length (a g = 1 warp of
// 32 one-nonzero rows is one FMA instruction with 32 useful lanes), and about
// 16 elements per lane keep the butterfly (log2 g adds per lane) small.  No
// shared memory and a small register footprint give the high occupancy that
// hides the two dependent memory rounds (index, then gather) of each step.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"
#include "csr_tiles.cuh"
#include "epilogue.cuh"

namespace amfls_gpu {
namespace csr_vector {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kBins = 6;            // bin b: g = 32 >> b lanes per row, 1 << b rows per warp
constexpr int kElemsPerLane = 16;   // row length / lanes targeted by the binning
constexpr int kUnroll = 4;          // elements per lane in flight

struct Table {
    const int* rows = nullptr;        // rows by bin, longest first within a bin
    long long warp_start[kBins + 1];  // warp tasks of bins 0 .. b-1
    int row_start[kBins + 1];         // rows of bin b: rows[row_start[b] .. row_start[b+1])
};

// Bin of a row of `len` nonzeros.
__host__ __device__ inline int bin_of(long long len) {
    int g = 32, b = 0;
    while (g > 1 && len < (long long)g * kElemsPerLane) {
        g >>= 1;
        ++b;
    }
    return b;
}

template <typename V>
__global__ void __launch_bounds__(kThreads)
vector_product_kernel(const int* __restrict__ off, const int* __restrict__ idx,
                      const V* __restrict__ val, Table t, const double* __restrict__ x,
                      Epilogue ep, double* partials, unsigned* counter) {
    using A = csr_tiles::acc_t<V>;
    if (ep.guard && *ep.guard == 0) return;
    const int lane = threadIdx.x & 31;
    double sq_t = 0.0, sq_out = 0.0, dot = 0.0, mx_t = 0.0, mx_out = 0.0;
    int nonfin = 0;
    const long long total = t.warp_start[kBins];
    const long long stride = (long long)gridDim.x * kWarps;
    for (long long wt = (long long)blockIdx.x * kWarps + (threadIdx.x >> 5); wt < total;
         wt += stride) {
        int b = 0;
#pragma unroll
        for (int i = 1; i < kBins; ++i) b += wt >= t.warp_start[i] ? 1 : 0;
        const int shift = 5 - b;  // log2 of the lanes per row
        const int g = 1 << shift;
        const int sub = lane & (g - 1);
        const long long local = (wt - t.warp_start[b]) * (32 >> shift) + (lane >> shift);
        const bool active = local < (long long)(t.row_start[b + 1] - t.row_start[b]);
        const int row = active ? t.rows[t.row_start[b] + local] : 0;
        A acc = A(0);
        if (active) {
            int e = off[row] + sub;
            const int end = off[row + 1];
            for (; e + (kUnroll - 1) * g < end; e += kUnroll * g) {
                int j[kUnroll];
                A v[kUnroll], xv[kUnroll];
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) j[u] = __ldcs(idx + e + u * g);
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) v[u] = csr_tiles::load_value(val + e + u * g);
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) xv[u] = csr_tiles::to_acc<A>(__ldg(x + j[u]));
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) acc = fma(v[u], xv[u], acc);
            }
            for (; e < end; e += g)
                acc = fma((A)csr_tiles::load_value(val + e), csr_tiles::to_acc<A>(__ldg(x + __ldcs(idx + e))),
                          acc);
        }
        for (int o = g >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (active && sub == 0)
            epilogue_row(ep, row, (double)acc, sq_t, sq_out, dot, mx_t, mx_out, nonfin);
    }
    finish_reduction(ep, sq_t, sq_out, dot, mx_t, mx_out, nonfin, partials, counter);
}

}  // namespace csr_vector
}  // namespace amfls_gpu
