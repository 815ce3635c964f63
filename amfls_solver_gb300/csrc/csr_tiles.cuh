// Tiled CSR products: nnz-balanced row blocks, one warp per tile.
//
// A side of the operator (A or its stored transpose) is cut once, on the
// host, into tiles: a tile is either a run of consecutive rows whose
// nonzeros total at most E (and at most E rows), or, for a row longer than
// E, one E-element slice of that row.  Every warp of the grid walks its own
// tiles (warp w takes tiles w, w + W, ... with W warps in the grid) and no
// warp waits on another, so the only synchronisation is __syncwarp and an
// SM keeps many independent tiles in flight.  Work on a tile:
//   1. coalesced loads of the tile's values and column indices (E / 32 of
//      each per lane, all issued before any is used), then the gathers
//      x[j_e], again all in flight together; values and gathered x go to the
//      warp's shared-memory buffers, and so do the tile's row offsets;
//   2. row sums: for one column lane i takes rows i, i + 32, ..., for C > 1
//      columns a group of C lanes takes a row (lane c, column c); a row of at
//      most kSeqMax nonzeros is summed as a sequential FMA chain in storage
//      order (per column) -- the
//      order of the reference's SparseCsrOperator::apply
//      (src/algorithms/mathematics/operators/sparse_csr_operator.cpp:203-235),
//      so those rows come out bit for bit equal to it; a longer row in the
//      tile is summed by the whole warp (strided lanes, fixed butterfly);
//   3. results: each row's sum goes out through the fused epilogue (one
//      column) or into the column-major output block.
// A slice of a long row is summed by the warp; the slices' partial sums go
// to global memory and the slice that arrives last (atomic ticket) adds them
// in slice order.  Every sum is taken in an order fixed by the matrix, so
// results are deterministic.  For C > 1 columns x is staged row-major
// beforehand so that one gather reads C contiguous doubles.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"
#include "epilogue.cuh"

namespace amfls_gpu {
namespace csr_tiles {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kE1 = 256;     // elements per tile, single-column products
constexpr int kEC = 64;      // elements per tile, 2..8 columns
constexpr int kSeqMax = 64;  // longest row summed by a single lane
static_assert(kEC <= kSeqMax, "multi-column tiles sum every row sequentially");

struct Table {
    const int4* tiles = nullptr;      // {first row, end row, first element, end element}
    const int* split = nullptr;       // long-row id of a slice tile, -1 for a row block
    const int2* long_rows = nullptr;  // {first slice tile, slice count}
    unsigned* long_count = nullptr;   // arrival tickets, zero between launches
    double* long_part = nullptr;      // C partial sums per tile
    int ntiles = 0;
};

// Shared memory of one warp: values and gathered x (E x C), row offsets.
template <int C, int E>
constexpr int warp_smem_bytes() {
    return E * 8 + E * C * 8 + (E + 8) * 4;
}

template <int C, int E>
constexpr int smem_bytes() {
    return kWarps * warp_smem_bytes<C, E>();
}

template <int C, int E, bool kFused>
__global__ void __launch_bounds__(kThreads)
tile_product_kernel(const int* __restrict__ off, const int* __restrict__ idx,
                    const double* __restrict__ val, Table tb, const double* __restrict__ x,
                    double* __restrict__ y, long long ldy, int ncols, Epilogue ep,
                    double* partials, unsigned* counter) {
    if (kFused && ep.guard && *ep.guard == 0) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char* wbase = smem + warp * warp_smem_bytes<C, E>();
    double* vs = reinterpret_cast<double*>(wbase);  // E values
    double* xs = vs + E;                            // E x C gathered x
    int* ro = reinterpret_cast<int*>(xs + E * C);   // E + 1 row offsets
    constexpr int kPer = E / 32;

    double sq_t = 0.0, sq_out = 0.0, dot = 0.0, mx_t = 0.0, mx_out = 0.0;
    int nonfin = 0;
    const int total_warps = gridDim.x * kWarps;
    for (int t = blockIdx.x * kWarps + warp; t < tb.ntiles; t += total_warps) {
        const int4 d = tb.tiles[t];
        const int R = d.y - d.x, n = d.w - d.z;
        const int q = tb.split[t];

        // 1. loads and gathers
        double a[kPer];
        int j[kPer];
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            const int i = lane + 32 * u;
            j[u] = i < n ? __ldcs(idx + d.z + i) : -1;
            a[u] = i < n ? __ldcs(val + d.z + i) : 0.0;
        }
        if (q < 0)
            for (int i = lane; i <= R; i += 32) ro[i] = __ldcs(off + d.x + i) - d.z;
        if constexpr (C == 1) {
            double xv[kPer];
#pragma unroll
            for (int u = 0; u < kPer; ++u) xv[u] = j[u] >= 0 ? __ldg(x + j[u]) : 0.0;
#pragma unroll
            for (int u = 0; u < kPer; ++u) {
                vs[lane + 32 * u] = a[u];
                xs[lane + 32 * u] = xv[u];
            }
        } else {
            static_assert(C % 2 == 0, "multi-column tiles gather pairs of doubles");
#pragma unroll
            for (int u = 0; u < kPer; ++u) {
                vs[lane + 32 * u] = a[u];
                if (j[u] >= 0) {
                    const double2* src =
                        reinterpret_cast<const double2*>(x + (long long)j[u] * C);
                    double2* dst = reinterpret_cast<double2*>(xs + (lane + 32 * u) * C);
#pragma unroll
                    for (int h = 0; h < C / 2; ++h) dst[h] = __ldg(src + h);
                }
            }
        }
        __syncwarp();

        // 2./3. row sums and results
        if (q < 0 && C > 1) {
            // C lanes per row (lane c of the group takes column c), 32 / C rows
            // at a time; rows of these tiles have at most kEC <= kSeqMax nonzeros
            constexpr int kGroups = 32 / C;
            const int g = lane / C, c = lane % C;
            for (int i = g; i < R; i += kGroups) {
                const int b0 = ro[i], b1 = ro[i + 1];
                double acc = 0.0;
                for (int e = b0; e < b1; ++e) acc = fma(vs[e], xs[e * C + c], acc);
                if (c < ncols) y[d.x + i + c * ldy] = acc;
            }
        } else if (q < 0) {
            unsigned wide = 0;  // bit k: row lane + 32 k is left to the whole warp
            for (int k = 0, i = lane; i < R; ++k, i += 32) {
                const int b0 = ro[i], b1 = ro[i + 1];
                if (b1 - b0 > kSeqMax) {
                    wide |= 1u << k;
                    continue;
                }
                double acc[C];
#pragma unroll
                for (int c = 0; c < C; ++c) acc[c] = 0.0;
                int e = b0;
                for (; e + 4 <= b1; e += 4) {
                    double av[4], xv[4][C];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        av[u] = vs[e + u];
#pragma unroll
                        for (int c = 0; c < C; ++c) xv[u][c] = xs[(e + u) * C + c];
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int c = 0; c < C; ++c) acc[c] = fma(av[u], xv[u][c], acc[c]);
                }
                for (; e < b1; ++e) {
                    const double av = vs[e];
#pragma unroll
                    for (int c = 0; c < C; ++c) acc[c] = fma(av, xs[e * C + c], acc[c]);
                }
                const int r = d.x + i;
                if constexpr (kFused) {
                    epilogue_row(ep, r, acc[0], sq_t, sq_out, dot, mx_t, mx_out, nonfin);
                } else {
#pragma unroll
                    for (int c = 0; c < C; ++c)
                        if (c < ncols) y[r + c * ldy] = acc[c];
                }
            }
            // rows longer than kSeqMax: the whole warp, one row at a time
            for (int k = 0; k * 32 < R; ++k) {
                unsigned pending = __ballot_sync(0xffffffffu, (wide >> k) & 1u);
                while (pending) {
                    const int src = __ffs(pending) - 1;
                    pending &= pending - 1;
                    const int i = src + 32 * k;
                    const int b0 = ro[i], b1 = ro[i + 1];
                    double acc[C];
#pragma unroll
                    for (int c = 0; c < C; ++c) acc[c] = 0.0;
                    for (int e = b0 + lane; e < b1; e += 32) {
                        const double av = vs[e];
#pragma unroll
                        for (int c = 0; c < C; ++c) acc[c] = fma(av, xs[e * C + c], acc[c]);
                    }
#pragma unroll
                    for (int c = 0; c < C; ++c)
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1)
                            acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
                    if (lane == 0) {
                        const int r = d.x + i;
                        if constexpr (kFused) {
                            epilogue_row(ep, r, acc[0], sq_t, sq_out, dot, mx_t, mx_out, nonfin);
                        } else {
#pragma unroll
                            for (int c = 0; c < C; ++c)
                                if (c < ncols) y[r + c * ldy] = acc[c];
                        }
                    }
                }
            }
        } else {
            // a slice of one long row: lane groups of C (lane c, column c)
            // stride over the elements, then a fixed butterfly over the groups
            double acc[C];
#pragma unroll
            for (int c = 0; c < C; ++c) acc[c] = 0.0;
            if constexpr (C == 1) {
                for (int e = lane; e < n; e += 32) acc[0] = fma(vs[e], xs[e], acc[0]);
                for (int o = 16; o > 0; o >>= 1)
                    acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], o);
            } else {
                const int g = lane / C, cl = lane % C;
                double part = 0.0;
                for (int e = g; e < n; e += 32 / C) part = fma(vs[e], xs[e * C + cl], part);
                for (int o = 16; o >= C; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
                // lane c (group 0) now holds column c; hand every column to lane 0
#pragma unroll
                for (int c = 0; c < C; ++c) acc[c] = __shfl_sync(0xffffffffu, part, c);
            }
            if (lane == 0) {
                const int2 lr = tb.long_rows[q];
#pragma unroll
                for (int c = 0; c < C; ++c) tb.long_part[(long long)t * C + c] = acc[c];
                __threadfence();
                const unsigned ticket = atomicAdd(&tb.long_count[q], 1u);
                if (ticket == static_cast<unsigned>(lr.y - 1)) {
                    tb.long_count[q] = 0u;
                    __threadfence();
                    double sum[C];
#pragma unroll
                    for (int c = 0; c < C; ++c) sum[c] = 0.0;
                    for (int u = 0; u < lr.y; ++u)
#pragma unroll
                        for (int c = 0; c < C; ++c)
                            sum[c] += __ldcg(&tb.long_part[(long long)(lr.x + u) * C + c]);
                    if constexpr (kFused) {
                        epilogue_row(ep, d.x, sum[0], sq_t, sq_out, dot, mx_t, mx_out, nonfin);
                    } else {
#pragma unroll
                        for (int c = 0; c < C; ++c)
                            if (c < ncols) y[d.x + c * ldy] = sum[c];
                    }
                }
            }
        }
        __syncwarp();  // the buffers are reused by the warp's next tile
    }
    if constexpr (kFused)
        finish_reduction(ep, sq_t, sq_out, dot, mx_t, mx_out, nonfin, partials, counter);
}

}  // namespace csr_tiles
}  // namespace amfls_gpu
