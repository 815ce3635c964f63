// Tiled CSR products: nnz-balanced warp tasks, one warp per task.
//
// A side of the operator (A or its stored transpose) is cut once, on the
// host, into warp tasks listed longest first.  The warps of the grid take
// them round by round in snake order (round k of W = grid warps: warp w
// takes task k W + w when k is even, k W + W - 1 - w when k is odd); no warp
// waits on another, so the only synchronisation is __syncwarp and an SM
// keeps many independent tasks in flight.  The assignment is static so that
// each thread adds its rows' epilogue terms in an order fixed by the table.
//
// Single-column products (C == 1).  The FP64 pipe of this GPU retires two
// lanes' FMAs per SM clock and a warp instruction costs the same with one
// lane active as with 32, so on sides whose median row has at most
// kChainShort nonzeros the row sums are laid out to keep every lane of
// every FMA busy (chain tables, kChains):
//   * a chain group is up to 32 rows of (nearly) the same length, at most
//     kChainMax nonzeros each; lane l sums row l of the group as a
//     sequential FMA chain from 0 in storage order -- the order of the
//     reference's SparseCsrOperator::apply
//     (src/algorithms/mathematics/operators/sparse_csr_operator.cpp:203-235),
//     so these rows come out bit for bit equal to it.  The group's elements
//     are staged kChainStep per row at a time: coalesced loads of values and
//     indices (consecutive lanes take consecutive elements of one row), the
//     gathers x[j], then a transposed store to shared memory from which
//     each lane reads its own row's next elements without bank conflicts.
//     A group whose rows hold at most one nonzero takes kFlatRows rows, 8
//     per lane, straight from registers.  Rows of up to kChainShort
//     nonzeros are grouped within windows of consecutive rows (so that
//     neighbouring rows share sectors in time), longer chain rows by length
//     over the whole side;
//   * a row longer than kChainMax is one warp task (up to kRowTaskTiles E
//     nonzeros) or cut into kRowTaskTiles E-element slices.
// On sides of longer rows a chain group would need many dependent staging
// passes, and row blocks are used instead: runs of consecutive rows whose
// nonzeros total at most E (and at most E rows), with rows longer than E as
// whole-row tasks or slices:
//   1. coalesced loads of the tile's values and column indices (E / 32 of
//      each per lane, all issued before any is used), then the gathers
//      x[j_e], again all in flight together; values and gathered x go to the
//      warp's shared-memory buffers, and so do the tile's row offsets;
//   2. row sums: one column -- lane i takes rows i, i + 32, ... of at most
//      kSeqMax nonzeros as sequential chains in storage order (bit for bit
//      the reference's), longer rows of the tile go to 8-lane groups
//      (strided, fixed butterfly), four rows at a time; C = 2..8 columns (X
//      staged row-major so that one gather reads C contiguous doubles) -- a
//      group of C lanes takes a row (lane c, column c), each a sequential
//      chain (rows of these tiles have at most E = kEC <= kSeqMax nonzeros);
//   3. results go through the fused epilogue (one column) or into the
//      column-major output block.
// A long row (or slice) is streamed through registers by the warp -- E / 32
// values, indices and gathers per lane in flight per step, lanes strided by
// element, then a fixed butterfly -- without shared memory.  Slices' partial
// sums go to global memory and the slice that arrives last (atomic ticket)
// adds them in slice order.  Every sum is taken in an order fixed by the
// matrix, so results are deterministic.
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
constexpr int kSeqMax = 64;  // longest row of a multi-column row block
constexpr int kRowTaskTiles = 16;  // a row of up to 16 E nonzeros is one warp task
static_assert(kEC <= kSeqMax, "multi-column tiles sum every row sequentially");
constexpr int kChainMax = 64;     // longest row summed as a per-lane chain (C == 1)
constexpr int kChainShort = 16;   // chain rows up to this length are grouped in windows
constexpr int kChainWindow = 1024;  // short chain rows per window
constexpr int kChainStep = 8;     // elements per row staged at a time
constexpr int kFlatRows = 256;    // rows of a group whose rows hold at most one nonzero
// task kinds (Table::split): row block, whole long row, chain group; q >= 0
// is a slice of long row q
constexpr int kRowBlock = -1, kWholeRow = -2, kChainGroup = -3;

struct Table {
    // row block, whole row or slice: {first row, end row, first element, end
    // element}; chain group: {first position in chain, rows, longest row, 0}
    const int4* tiles = nullptr;
    // kRowBlock, kWholeRow, kChainGroup, or q >= 0: a slice of long row q
    // (rows longer than kRowTaskTiles E)
    const int* split = nullptr;
    // the rows of the chain groups, group by group: {row, first element}, the
    // first element -1 for an empty row
    const int2* chain = nullptr;
    const int2* long_rows = nullptr;  // {first slice tile, slice count}
    unsigned* long_count = nullptr;   // arrival tickets, zero between launches
    double* long_part = nullptr;      // C partial sums per tile
    int ntiles = 0;
    int nnz = 0;
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

// Row stride (in (value, x) pairs) of the transposed chain staging for K
// elements per row: 32 rows plus padding that makes the stores of a
// quarter-warp (8 lanes: 8 / K rows x K elements) hit distinct 16-byte bank
// groups when K is a power of two.
__host__ __device__ constexpr int chain_stride(int k) { return 32 + kChainStep / k; }

// Pairs of the largest staging, max over K of K x chain_stride(K).
constexpr int chain_pairs() {
    int m = 0;
    for (int k = 1; k <= kChainStep; ++k) m = m > k * chain_stride(k) ? m : k * chain_stride(k);
    return m;
}

// s / k for 0 <= s < 256 and 1 <= k <= 8 as (s * magic) >> 11 with magic =
// ceil(2048 / k): the excess s (magic - 2048 / k) / 2048 stays below 1 / k,
// so the quotient is exact.
__host__ __device__ constexpr int chain_magic(int k) { return (2048 + k - 1) / k; }
static_assert(kChainStep * 32 <= 256, "chain_magic covers slots below 256");

// Shared memory of one warp.  A row block: values and gathered x (E x C;
// one column as (value, x) pairs), row offsets (E + 1) and, for one column,
// the list of rows longer than kSeqMax (fewer than E / kSeqMax).  One
// column also stages chain groups there (chain_pairs() pairs of up to 16
// bytes).  Rounded up to 16 bytes so that every warp's buffers stay
// aligned for 16-byte accesses.
template <int C, int E>
constexpr int warp_smem_bytes() {
    constexpr int block = (E * 8 + E * C * 8 + (E + 8 + E / kSeqMax) * 4 + 15) / 16 * 16;
    constexpr int chains = (chain_pairs() * 16 + 15) / 16 * 16;
    return C == 1 && chains > block ? chains : block;
}

static_assert(warp_smem_bytes<8, kEC>() % 16 == 0 && warp_smem_bytes<1, kE1>() % 16 == 0,
              "per-warp buffers must keep 16-byte alignment");

template <int C, int E>
constexpr int smem_bytes() {
    return kWarps * warp_smem_bytes<C, E>();
}

// Resident CTAs per SM each instantiation is compiled for (its register
// budget): the chain paths keep 8 loads, gathers and the pass state per lane
// in flight (80 registers), row blocks of one column fit 64, and FP64 row
// blocks of C > 1 columns 40 (C = 2), 48 (C = 4) and 80 (C = 8).
constexpr int min_blocks(int c, bool chains) {
    return c == 1 ? (chains ? 3 : 4) : c == 2 ? 6 : c == 4 ? 5 : 3;
}

// kChains: the table of a single-column side holds chain groups (and long
// rows) rather than row blocks; each instantiation carries only its paths.
template <typename V, int C, int E, bool kFused, bool kChains>
__global__ void __launch_bounds__(kThreads, min_blocks(C, kChains))
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
    int* ro = reinterpret_cast<int*>(wbase + E * 8 + E * C * 8);  // E + 1 row offsets
    // one column: (value, x) pairs, one 16-byte (8-byte for FP32) word each,
    // so that a chain step or a row sum reads both with one shared-memory
    // access
    using Pair = std::conditional_t<std::is_same_v<A, double>, double2, float2>;
    Pair* vx = reinterpret_cast<Pair*>(wbase);
    A* vx1 = reinterpret_cast<A*>(wbase);  // pair p: vx1[2 p] value, vx1[2 p + 1] x
    constexpr int kPer = E / 32;

    double sq_t = 0.0, sq_out = 0.0, dot = 0.0, mx_t = 0.0, mx_out = 0.0;
    int nonfin = 0;
    // static assignment, so that every thread sums its rows' epilogue terms
    // in an order fixed by the table and the grid: the table lists the
    // longest tasks first and round k of W = gridDim.x kWarps tasks goes to
    // the warps in snake order (warp w takes task k W + w in even rounds,
    // k W + W - 1 - w in odd ones); chain tasks are short, so the next
    // one's descriptor is fetched while the current one runs
    const int nwarps = gridDim.x * kWarps, w = blockIdx.x * kWarps + warp;
    auto task_of = [&](int k) { return k * nwarps + ((k & 1) ? nwarps - 1 - w : w); };
    int t = task_of(0);
    int4 dn = make_int4(0, 0, 0, 0);
    int qn = 0;
    if (kChains && t < tb.ntiles) {
        dn = tb.tiles[t];
        qn = tb.split[t];
    }
    for (int k = 0; t < tb.ntiles; t = task_of(++k)) {
        int4 d;
        int q;
        if constexpr (kChains) {
            d = dn;
            q = qn;
            const int tn = task_of(k + 1);
            if (tn < tb.ntiles) {
                dn = tb.tiles[tn];
                qn = tb.split[tn];
            }
        } else {
            d = tb.tiles[t];
            q = tb.split[t];
        }

        if (kChains && C == 1 && q == kChainGroup && d.z <= 1) {
            // up to kFlatRows rows of at most one nonzero: lane l takes
            // group rows l + 32 u, each y = fma(a, x, 0)
            constexpr int kU = kFlatRows / 32;
            int rows[kU], jv[kU];
            A av[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                int2 ce = make_int2(-1, -1);
                if (lane + 32 * u < d.y) ce = __ldg(tb.chain + d.x + lane + 32 * u);
                rows[u] = ce.x;
                jv[u] = ce.y >= 0 ? __ldcs(idx + ce.y) : -1;
                av[u] = ce.y >= 0 ? load_value(val + ce.y) : A(0);
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const A xv = jv[u] >= 0 ? to_acc<A>(__ldg(x + jv[u])) : A(0);
                const A acc = jv[u] >= 0 ? fma(av[u], xv, A(0)) : A(0);
                if (rows[u] >= 0) {
                    if constexpr (kFused) {
                        epilogue_row(ep, rows[u], static_cast<double>(acc), sq_t, sq_out, dot,
                                     mx_t, mx_out, nonfin);
                    } else {
                        if (ncols > 0) y[rows[u]] = static_cast<double>(acc);
                    }
                }
            }
        } else if (kChains && C == 1 && q == kChainGroup) {
            // lane l sums row l of the group (d.y <= 32 rows, the longest
            // d.z nonzeros), kChainStep elements per row per pass.  Element
            // loads need only the row's first element: slots past the end
            // of a row read the following elements (within the matrix) and
            // the chain skips them, so the row length can arrive with them
            const int2 ce = lane < d.y ? __ldg(tb.chain + d.x + lane) : make_int2(-1, -1);
            const int b = ce.y;
            const int len = b >= 0 ? __ldg(off + ce.x + 1) - b : 0;
            A acc = 0;
            for (int k0 = 0; k0 < d.z; k0 += kChainStep) {
                const int K = min(kChainStep, d.z - k0);
                const int stride = chain_stride(K), magic = chain_magic(K);
                const int nslots = d.y * K;
                // slot s = 32 u + lane of the K x 32 staging holds element
                // k0 + s % K of group row s / K: consecutive lanes read
                // consecutive elements of a row
                int jv[kChainStep];
#pragma unroll
                for (int u = 0; u < kChainStep; ++u) {
                    jv[u] = -1;
                    if (32 * u < nslots) {
                        const int sl = 32 * u + lane;
                        const int row = (sl * magic) >> 11;  // sl / K
                        const int e = sl - row * K;
                        const int rb = __shfl_sync(0xffffffffu, b, row & 31);
                        const int el = rb + k0 + e;
                        const bool ok = sl < nslots && rb >= 0 && el < tb.nnz;
                        jv[u] = ok ? __ldcs(idx + el) : -1;
                        const A a = ok ? load_value(val + el) : A(0);
                        if (sl < nslots) vx1[2 * (e * stride + row)] = a;
                    }
                }
#pragma unroll
                for (int u = 0; u < kChainStep; ++u) {
                    const int sl = 32 * u + lane;
                    if (32 * u < nslots && sl < nslots) {
                        const int row = (sl * magic) >> 11;
                        vx1[2 * ((sl - row * K) * stride + row) + 1] =
                            jv[u] >= 0 ? to_acc<A>(__ldg(x + jv[u])) : A(0);
                    }
                }
                __syncwarp();
                for (int e = 0; e < K; ++e) {
                    const Pair p = vx[e * stride + lane];
                    if (k0 + e < len) acc = fma(p.x, p.y, acc);
                }
                __syncwarp();  // the staging is rewritten by the next pass
            }
            if (ce.x >= 0) {
                if constexpr (kFused) {
                    epilogue_row(ep, ce.x, static_cast<double>(acc), sq_t, sq_out, dot, mx_t,
                                 mx_out, nonfin);
                } else {
                    if (ncols > 0) y[ce.x] = static_cast<double>(acc);
                }
            }
        } else if (q != kRowBlock) {
            // a whole long row (kWholeRow) or a slice of one (q >= 0), through
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
                if (q == kWholeRow) {
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
        } else if constexpr (!kChains) {
            // a row block: 1. loads and gathers
            const int R = d.y - d.x, n = d.w - d.z;
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
                for (int u = 0; u < kPer; ++u)
                    xv[u] = j[u] >= 0 ? to_acc<A>(__ldg(x + j[u])) : A(0);
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
                // C lanes per row (lane c of the group takes column c), 32 / C
                // rows at a time; rows of these tiles have at most kEC <=
                // kSeqMax nonzeros
                constexpr int kGroups = 32 / C;
                const int g = lane / C, c = lane % C;
                for (int i = g; i < R; i += kGroups) {
                    const int b0 = ro[i], b1 = ro[i + 1];
                    A acc = 0;
                    for (int e = b0; e < b1; ++e) acc = fma(vs[e], xs[e * C + c], acc);
                    if (c < ncols) y[d.x + i + c * ldy] = static_cast<double>(acc);
                }
            } else {
                // lane i takes rows i, i + 32, ... of at most kSeqMax nonzeros
                // (sequential chains in storage order)
                unsigned wide = 0;  // bit k: row lane + 32 k is left to 8-lane groups
                for (int k = 0, i = lane; i < R; ++k, i += 32) {
                    const int b0 = ro[i], b1 = ro[i + 1];
                    if (b1 - b0 > kSeqMax) {
                        wide |= 1u << k;
                        continue;
                    }
                    A acc = 0;
                    int e = b0;
                    for (; e + 4 <= b1; e += 4) {
                        Pair p[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) p[u] = vx[e + u];
#pragma unroll
                        for (int u = 0; u < 4; ++u) acc = fma(p[u].x, p[u].y, acc);
                    }
                    for (; e < b1; ++e) {
                        const Pair p = vx[e];
                        acc = fma(p.x, p.y, acc);
                    }
                    const int r = d.x + i;
                    if constexpr (kFused) {
                        epilogue_row(ep, r, static_cast<double>(acc), sq_t, sq_out, dot, mx_t,
                                     mx_out, nonfin);
                    } else {
                        if (ncols > 0) y[r] = static_cast<double>(acc);
                    }
                }
                // rows longer than kSeqMax (fewer than E / kSeqMax of them):
                // listed after the row offsets, then summed four at a time by
                // 8-lane groups (strided lanes, fixed butterfly within the group)
                int* wl = ro + E + 1;
                int nw = 0;
                for (int k = 0; k * 32 < R; ++k) {
                    const unsigned bits = __ballot_sync(0xffffffffu, (wide >> k) & 1u);
                    if ((wide >> k) & 1u)
                        wl[nw + __popc(bits & ((1u << lane) - 1u))] = lane + 32 * k;
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
                            epilogue_row(ep, r, static_cast<double>(acc), sq_t, sq_out, dot,
                                         mx_t, mx_out, nonfin);
                        } else {
                            y[r] = static_cast<double>(acc);
                        }
                    }
                }
            }
            __syncwarp();  // the buffers are reused by the warp's next tile
        }
    }
    if constexpr (kFused)
        finish_reduction(ep, sq_t, sq_out, dot, mx_t, mx_out, nonfin, partials, counter);
}

}  // namespace csr_tiles
}  // namespace amfls_gpu
