// Tiled CSR products: nnz-balanced row blocks, one warp per tile.
//
// A side of the operator (A or its stored transpose) is cut once, on the
// host, into tiles: a tile is either a run of consecutive rows whose
// nonzeros total at most E (and at most E rows), a single row of up to
// kRowTaskTiles E nonzeros, or a kRowTaskTiles E-element slice of a longer
// row.  Every warp of the grid walks its own
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
//      tile is summed by 8 lanes (strided, fixed butterfly), four at a time;
//   3. results: each row's sum goes out through the fused epilogue (one
//      column) or into the column-major output block.
// A long row (or slice) is streamed through registers by the warp -- E / 32
// values, indices and gathers per lane in flight per step, lanes strided by
// element, then a fixed butterfly -- without shared memory.  Slices' partial
// sums go to global memory and the slice that arrives last (atomic ticket)
// adds them in slice order.  Every sum is taken in an order fixed by the matrix, so
// results are deterministic.  For C > 1 columns x is staged row-major
// beforehand so that one gather reads C contiguous doubles.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "common.cuh"
#include "epilogue.cuh"

namespace amfls_gpu {
namespace csr_tiles {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kE1 = 256;     // elements per tile, single-column products
constexpr int kEC = 64;      // elements per tile, 2..8 columns
constexpr int kSeqMax = 64;  // longest row summed by a single lane
constexpr int kRowTaskTiles = 16;  // a row of up to 16 E nonzeros is one warp task
static_assert(kEC <= kSeqMax, "multi-column tiles sum every row sequentially");

struct Table {
    const int4* tiles = nullptr;      // {first row, end row, first element, end element}
    // -1: a row block; -2: one whole row of more than E nonzeros; q >= 0: a
    // slice of long row q (rows longer than kRowTaskTiles E)
    const int* split = nullptr;
    const int2* long_rows = nullptr;  // {first slice tile, slice count}
    unsigned* long_count = nullptr;   // arrival tickets, zero between launches
    double* long_part = nullptr;      // C partial sums per tile
    int ntiles = 0;
};

// Values stored as V; FP64 values accumulate in FP64 (the exact path), FP32
// and BF16 values accumulate in FP32 with x rounded to FP32 on load.
template <typename V>
using acc_t = std::conditional_t<std::is_same_v<V, double>, double, float>;

template <typename A>
__device__ __forceinline__ A to_acc(double v) {
    return static_cast<A>(v);
}
__device__ __forceinline__ float load_value(const float* p) { return __ldcs(p); }
__device__ __forceinline__ double load_value(const double* p) { return __ldcs(p); }
__device__ __forceinline__ float load_value(const __nv_bfloat16* p) {
    return __bfloat162float(*p);
}

// Shared memory of one warp: values and gathered x (E x C), row offsets
// (E + 1) and the list of rows longer than kSeqMax (fewer than E / kSeqMax).
// Rounded up to 16 bytes so that every warp's buffers stay aligned for the
// 16-byte accesses to x.
template <int C, int E>
constexpr int warp_smem_bytes() {
    return (E * 8 + E * C * 8 + (E + 8 + E / kSeqMax) * 4 + 15) / 16 * 16;
}
static_assert(warp_smem_bytes<8, kEC>() % 16 == 0 && warp_smem_bytes<1, kE1>() % 16 == 0,
              "per-warp buffers must keep 16-byte alignment");

template <int C, int E>
constexpr int smem_bytes() {
    return kWarps * warp_smem_bytes<C, E>();
}

template <typename V, int C, int E, bool kFused>
__global__ void __launch_bounds__(kThreads)
tile_product_kernel(const int* __restrict__ off, const int* __restrict__ idx,
                    const V* __restrict__ val, Table tb, const double* __restrict__ x,
                    double* __restrict__ y, long long ldy, int ncols, Epilogue ep,
                    double* partials, unsigned* counter) {
    if (kFused && ep.guard && *ep.guard == 0) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char* wbase = smem + warp * warp_smem_bytes<C, E>();
    using A = acc_t<V>;
    A* vs = reinterpret_cast<A*>(wbase);           // E values (C > 1)
    A* xs = reinterpret_cast<A*>(wbase + E * 8);   // E x C gathered x (C > 1)
    // one column: (value, x) pairs, one 16-byte (8-byte for FP32) word each,
    // so the row sums read both with one shared-memory access
    using Pair = std::conditional_t<std::is_same_v<A, double>, double2, float2>;
    Pair* vx = reinterpret_cast<Pair*>(wbase);
    int* ro = reinterpret_cast<int*>(wbase + E * 8 + E * C * 8);  // E + 1 row offsets
    constexpr int kPer = E / 32;

    double sq_t = 0.0, sq_out = 0.0, dot = 0.0, mx_t = 0.0, mx_out = 0.0;
    int nonfin = 0;
    const int total_warps = gridDim.x * kWarps;
    for (int t = blockIdx.x * kWarps + warp; t < tb.ntiles; t += total_warps) {
        const int4 d = tb.tiles[t];
        const int R = d.y - d.x, n = d.w - d.z;
        const int q = tb.split[t];

        if (q != -1) {
            // a whole long row (q == -2) or a slice of one (q >= 0), through
            // registers: group g = lane / C takes elements g, g + 32 / C, ...,
            // lane c of the group column c
            constexpr int kG = 32 / C;
            const int g = lane / C, cl = lane % C;
            A part = 0;
            for (int base = d.z; base < d.w; base += E) {
                constexpr int kStep = E / kG;
                A av[kStep], xv[kStep];
                int jv[kStep];
#pragma unroll
                for (int u = 0; u < kStep; ++u) {
                    const int e = base + g + kG * u;
                    jv[u] = e < d.w ? __ldcs(idx + e) : -1;
                    av[u] = e < d.w ? load_value(val + e) : A(0);
                }
#pragma unroll
                for (int u = 0; u < kStep; ++u)
                    xv[u] = jv[u] >= 0 ? to_acc<A>(__ldg(x + (long long)jv[u] * C + cl)) : A(0);
#pragma unroll
                for (int u = 0; u < kStep; ++u) part = fma(av[u], xv[u], part);
            }
            for (int o = 16; o >= C; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
            double acc[C];
#pragma unroll
            for (int c = 0; c < C; ++c) acc[c] = __shfl_sync(0xffffffffu, part, c);
            if (lane == 0) {
                if (q == -2) {
                    if constexpr (kFused) {
                        epilogue_row(ep, d.x, acc[0], sq_t, sq_out, dot, mx_t, mx_out, nonfin);
                    } else {
#pragma unroll
                        for (int c = 0; c < C; ++c)
                            if (c < ncols) y[d.x + c * ldy] = acc[c];
                    }
                } else {
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
                            epilogue_row(ep, d.x, sum[0], sq_t, sq_out, dot, mx_t, mx_out,
                                         nonfin);
                        } else {
#pragma unroll
                            for (int c = 0; c < C; ++c)
                                if (c < ncols) y[d.x + c * ldy] = sum[c];
                        }
                    }
                }
            }
            continue;
        }

        // 1. loads and gathers
        A a[kPer];
        int j[kPer];
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            const int i = lane + 32 * u;
            j[u] = i < n ? __ldcs(idx + d.z + i) : -1;
            a[u] = i < n ? load_value(val + d.z + i) : A(0);
        }
        for (int i = lane; i <= R; i += 32) ro[i] = __ldcs(off + d.x + i) - d.z;
        if constexpr (C == 1) {
            A xv[kPer];
#pragma unroll
            for (int u = 0; u < kPer; ++u) xv[u] = j[u] >= 0 ? to_acc<A>(__ldg(x + j[u])) : A(0);
#pragma unroll
            for (int u = 0; u < kPer; ++u) {
                Pair p;
                p.x = a[u];
                p.y = xv[u];
                vx[lane + 32 * u] = p;
            }
        } else {
            static_assert(C % 2 == 0, "multi-column tiles gather pairs of doubles");
#pragma unroll
            for (int u = 0; u < kPer; ++u) {
                vs[lane + 32 * u] = a[u];
                if (j[u] >= 0) {
                    const double2* src =
                        reinterpret_cast<const double2*>(x + (long long)j[u] * C);
                    A* dst = xs + (lane + 32 * u) * C;
#pragma unroll
                    for (int h = 0; h < C / 2; ++h) {
                        const double2 p = __ldg(src + h);
                        dst[2 * h] = to_acc<A>(p.x);
                        dst[2 * h + 1] = to_acc<A>(p.y);
                    }
                }
            }
        }
        __syncwarp();

        // 2./3. row sums and results
        if constexpr (C > 1) {
            // C lanes per row (lane c of the group takes column c), 32 / C rows
            // at a time; rows of these tiles have at most kEC <= kSeqMax nonzeros
            constexpr int kGroups = 32 / C;
            const int g = lane / C, c = lane % C;
            for (int i = g; i < R; i += kGroups) {
                const int b0 = ro[i], b1 = ro[i + 1];
                A acc = 0;
                for (int e = b0; e < b1; ++e) acc = fma(vs[e], xs[e * C + c], acc);
                if (c < ncols) y[d.x + i + c * ldy] = static_cast<double>(acc);
            }
        } else {
            unsigned wide = 0;  // bit k: row lane + 32 k is left to the whole warp
            for (int k = 0, i = lane; i < R; ++k, i += 32) {
                const int b0 = ro[i], b1 = ro[i + 1];
                if (b1 - b0 > kSeqMax) {
                    wide |= 1u << k;
                    continue;
                }
                A acc[C];  // C == 1 on this path
                acc[0] = 0;
                int e = b0;
                for (; e + 4 <= b1; e += 4) {
                    Pair p[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) p[u] = vx[e + u];
#pragma unroll
                    for (int u = 0; u < 4; ++u) acc[0] = fma(p[u].x, p[u].y, acc[0]);
                }
                for (; e < b1; ++e) {
                    const Pair p = vx[e];
                    acc[0] = fma(p.x, p.y, acc[0]);
                }
                const int r = d.x + i;
                if constexpr (kFused) {
                    epilogue_row(ep, r, static_cast<double>(acc[0]), sq_t, sq_out, dot, mx_t,
                                 mx_out, nonfin);
                } else {
#pragma unroll
                    for (int c = 0; c < C; ++c)
                        if (c < ncols) y[r + c * ldy] = static_cast<double>(acc[c]);
                }
            }
            // rows longer than kSeqMax (fewer than E / kSeqMax of them): listed
            // after the row offsets, then summed four at a time by 8-lane
            // groups (strided lanes, fixed butterfly within the group)
            int* wl = ro + E + 1;
            int nw = 0;
            for (int k = 0; k * 32 < R; ++k) {
                const unsigned bits = __ballot_sync(0xffffffffu, (wide >> k) & 1u);
                if ((wide >> k) & 1u) wl[nw + __popc(bits & ((1u << lane) - 1u))] = lane + 32 * k;
                nw += __popc(bits);
            }
            __syncwarp();
            const int g = lane >> 3, gl = lane & 7;
            for (int w0 = 0; w0 < nw; w0 += 4) {
                const bool mine = w0 + g < nw;
                const int i = mine ? wl[w0 + g] : 0;
                const int b0 = mine ? ro[i] : 0, b1 = mine ? ro[i + 1] : 0;
                A acc = 0;
                for (int e = b0 + gl; e < b1; e += 8) {
                    const Pair p = vx[e];
                    acc = fma(p.x, p.y, acc);
                }
#pragma unroll
                for (int o = 4; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (mine && gl == 0) {
                    const int r = d.x + i;
                    if constexpr (kFused) {
                        epilogue_row(ep, r, static_cast<double>(acc), sq_t, sq_out, dot, mx_t,
                                     mx_out, nonfin);
                    } else {
                        y[r] = static_cast<double>(acc);
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
