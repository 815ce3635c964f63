// CSR device operator: Y = A X and X = A^T Y in FP64 on sm_103a.
//
// Replaces the reference's SparseCsrOperator
// (src/algorithms/mathematics/operators/sparse_csr_operator.cpp:14-269):
//   * the constructor's one-pass validation and certified norm model
//     (offsets span the values, columns in range, no duplicate column in a
//     row, finite values; ||A|| <= min(sqrt(||A||_1 ||A||_inf), ||A||_F),
//     ||A|| >= max(max|a_ij|, max row/column 2-norm); rounding steps
//     2*max_row_nnz+2 and 2*max_col_nnz+2) runs as device kernels;
//   * apply streams nnz-balanced tiles of rows through shared memory with
//     bulk copies and sums each row by a merge-path segmented reduction
//     (csr_tiles.cuh); sums are taken in an order fixed by the tiling, so
//     results are deterministic for a given matrix;
//   * apply_transpose does NOT scatter: it runs the same gather kernel on a
//     transpose (CSR of A^T) built once on the device with a stable sort, so
//     each column sums its entries in row order like the reference's scatter;
//   * the double-double validation products use a row-length-binned
//     sub-warp kernel (rows grouped by length, G in {1,..,32} lanes a row).
// Row and column sums of |a_ij| for the norm model are accumulated
// sequentially in the reference's order (rows in CSR order, columns in row
// order), so those stored sums match the reference bit for bit.
#include <cub/cub.cuh>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "common.cuh"
#include "csr_operator.hpp"
#include "csr_tiles.cuh"
#include "csr_vector.cuh"
#include "dd.cuh"
#include "epilogue.cuh"
#include "fp_bounds.cuh"

namespace amfls_gpu {

namespace {

constexpr int kThreads = 256;
constexpr int kWarpsPerBlock = kThreads / 32;
// most CTAs a product launches (eight per SM)
inline int max_blocks() { return grid_cap(); }

// ------------------------------------------------------------- setup ----

__global__ void check_offsets_kernel(const long long* off, int rows, long long nnz,
                                     int* err, unsigned long long* max_len, int* lens,
                                     int elems_per_lane, int* bins) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows;
         r += (long long)gridDim.x * blockDim.x) {
        const long long a = off[r], b = off[r + 1];
        if (b < a) atomicOr(err, 1);
        if (r == 0 && a != 0) atomicOr(err, 2);
        if (r == rows - 1 && b != nnz) atomicOr(err, 2);
        const long long len = b > a ? b - a : 0;
        atomicMax(max_len, (unsigned long long)len);
        lens[r] = (int)(len > 0x7fffffffLL ? 0x7fffffffLL : len);
        long long want = (len + elems_per_lane - 1) / elems_per_lane;
        int g = 1, bin = 0;
        while (g < want && g < 32) {
            g <<= 1;
            ++bin;
        }
        bins[r] = bin;
    }
}

__global__ void expand_rows_kernel(const long long* off, const long long* idx64,
                                   const double* val, int rows, int cols, int* idx32,
                                   int* row_of, int* err) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows;
         r += (long long)gridDim.x * blockDim.x) {
        for (long long e = off[r]; e < off[r + 1]; ++e) {
            const long long c = idx64[e];
            if (c < 0 || c >= cols) {
                atomicOr(err, 4);
                idx32[e] = 0;
            } else {
                idx32[e] = (int)c;
            }
            if (!isfinite(val[e])) atomicOr(err, 8);
            row_of[e] = (int)r;
        }
    }
}

__global__ void gather_transpose_kernel(const int* perm, const int* row_of, const double* val,
                                        long long nnz, int* rows_t, double* vals_t) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nnz;
         p += (long long)gridDim.x * blockDim.x) {
        const int e = perm[p];
        rows_t[p] = row_of[e];
        vals_t[p] = val[e];
    }
}

__global__ void count_columns_kernel(const int* idx32, long long nnz, int* counts) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nnz;
         e += (long long)gridDim.x * blockDim.x)
        atomicAdd(&counts[idx32[e]], 1);
}

__global__ void duplicate_kernel(const long long* off_t, const int* rows_t, int cols, int* err) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < cols;
         c += (long long)gridDim.x * blockDim.x)
        for (long long p = off_t[c] + 1; p < off_t[c + 1]; ++p)
            if (rows_t[p] == rows_t[p - 1]) atomicOr(err, 16);
}

__device__ __forceinline__ void atomic_max_pos(double* addr, double v) {
    // nonnegative doubles order like their bit patterns
    atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

// Per row (mode 0) or per column of the transpose (mode 1): sequential sums
// in storage order, then the outward bounds of the norm model.
__global__ void norm_model_kernel(const long long* off, const double* val, int count,
                                  int is_column, double* acc /*[4]: max_sum, max_two_lower,
                                  max_entry, frob_partial_unused*/,
                                  double* frob_partials, unsigned* counter, double* frob_out) {
    __shared__ double scratch[32];
    double frob = 0.0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < count;
         r += (long long)gridDim.x * blockDim.x) {
        double s = 0.0, q = 0.0, mx = 0.0;
        const long long a = off[r], b = off[r + 1];
        for (long long e = a; e < b; ++e) {
            const double m = fabs(val[e]);
            mx = fmax(mx, m);
            s += m;
            q = fma(m, m, q);
        }
        const long long len = b - a;
        atomic_max_pos(&acc[0], fpb::sum_upper(s, len, true));
        atomic_max_pos(&acc[1], fpb::down_sqrt(fpb::sum_lower(q, len)));
        atomic_max_pos(&acc[2], mx);
        if (is_column) frob = __dadd_ru(frob, fpb::sum_upper(q, len, false));
    }
    if (!is_column) return;
    // upward-rounded block sum of the Frobenius terms
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) frob = __dadd_ru(frob, __shfl_xor_sync(0xffffffffu, frob, o));
    if (lane == 0) scratch[warp] = frob;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = __dadd_ru(t, scratch[w]);
        frob_partials[blockIdx.x] = t;
    }
    if (arrive_last(counter, gridDim.x) && threadIdx.x == 0) {
        double t = 0.0;
        for (unsigned i = 0; i < gridDim.x; ++i) t = __dadd_ru(t, frob_partials[i]);
        *frob_out = fpb::widen_up(t);
    }
}

__global__ void finish_model_kernel(const double* row_acc, const double* col_acc,
                                    const double* frob2, double* model) {
    // row_acc[0] = max row |.|-sum upper (=> ||A||_inf), col_acc[0] => ||A||_1
    const double one_inf = fpb::up_mul(fpb::up_sqrt(col_acc[0]), fpb::up_sqrt(row_acc[0]));
    const double frob = fpb::up_sqrt(*frob2);
    double upper = fmin(one_inf, frob);
    double lower = fmax(fmax(row_acc[2], col_acc[2]), fmax(row_acc[1], col_acc[1]));
    if (!isfinite(upper) || lower > upper) {
        upper = fpb::kInf;
        lower = 0.0;
    }
    model[0] = upper;
    model[1] = lower;
}

// -------------------------------------------------------------- SpMV ----

struct BinTable {
    long long warp_start[7];  // cumulative warps per bin (bin b: [ws[b], ws[b+1]))
    int row_start[7];         // rows of bin b in perm: [rs[b], rs[b+1])
};

__global__ void narrow_offsets_kernel(const long long* off, int count, int* off32) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r <= count;
         r += (long long)gridDim.x * blockDim.x)
        off32[r] = (int)off[r];
}

// Double-double product for the validation refinement.
__global__ void __launch_bounds__(kThreads)
spmv_dd_kernel(const long long* __restrict__ off, const int* __restrict__ idx,
               const double* __restrict__ val, const int* __restrict__ perm, BinTable bt,
               const double* __restrict__ x_hi, const double* __restrict__ x_lo, double* y_hi,
               double* y_lo, int* finite) {
    const int lane = threadIdx.x & 31;
    const long long total = bt.warp_start[6];
    for (long long wt = (long long)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); wt < total;
         wt += (long long)gridDim.x * kWarpsPerBlock) {
        int b = 0;
#pragma unroll
        for (int i = 1; i < 6; ++i) b += wt >= bt.warp_start[i] ? 1 : 0;
        const int g = 1 << b;
        const long long local = (wt - bt.warp_start[b]) * (32 >> b) + (lane >> b);
        const bool active = local < (long long)(bt.row_start[b + 1] - bt.row_start[b]);
        const int row = active ? perm[bt.row_start[b] + local] : 0;
        dd acc{0.0, 0.0};
        if (active) {
            const long long end = off[row + 1];
            for (long long e = off[row] + (lane & (g - 1)); e < end; e += g) {
                const int j = idx[e];
                acc = dd_add(acc, dd_mul_d(dd{x_hi[j], x_lo ? x_lo[j] : 0.0}, val[e]));
            }
        }
        for (int o = g >> 1; o > 0; o >>= 1) acc = dd_add(acc, dd_shfl_xor(acc, o));
        if (active && (lane & (g - 1)) == 0) {
            y_hi[row] = acc.hi;
            y_lo[row] = acc.lo;
            if (!isfinite(acc.hi) || !isfinite(acc.lo)) atomicAnd(finite, 0);
        }
    }
}

int grid_for(long long warps) {
    long long blocks = (warps + kWarpsPerBlock - 1) / kWarpsPerBlock;
    return (int)std::max<long long>(1, std::min<long long>(blocks, max_blocks()));
}

int setup_grid(long long items) {
    return (int)std::max<long long>(1, std::min<long long>((items + 255) / 256, 2 * grid_cap()));
}

}  // namespace

namespace {

// Elements of the value / index / offset copies: n rounded up to a multiple
// of 4 plus 4 (16-byte aligned ends; the tails are zero).
long long padded(long long n) { return ((n + 3) & ~3LL) + 4; }

// One tiling of one side (see csr_tiles.cuh), owned by the operator.
struct TileStore {
    int4* tiles = nullptr;
    int* split = nullptr;
    int2* chain = nullptr;
    int2* long_rows = nullptr;
    unsigned* long_count = nullptr;
    double* long_part = nullptr;
    int ntiles = 0;
    int nnz = 0;
    bool chains = false;  // chain groups rather than row blocks
    int grid = 1;

    csr_tiles::Table view() const {
        csr_tiles::Table t;
        t.tiles = tiles;
        t.split = split;
        t.chain = chain;
        t.long_rows = long_rows;
        t.long_count = long_count;
        t.long_part = long_part;
        t.ntiles = ntiles;
        t.nnz = nnz;
        return t;
    }
    void release() {
        cudaFree(tiles);
        cudaFree(split);
        cudaFree(chain);
        cudaFree(long_rows);
        cudaFree(long_count);
        cudaFree(long_part);
        *this = TileStore{};
    }
};

// Sides with fewer nonzeros use row blocks even when their rows are short:
// their tables hold about one task per resident warp, so a product takes
// as long as its slowest task, and a chain group (several dependent staging
// passes) is slower than a row block (one load round, one gather round).
constexpr long long kChainMinNonzeros = 1LL << 21;

// Warp tasks of one side: rows longer than `longer_than` as whole-row
// tasks (up to kRowTaskTiles E nonzeros) or kRowTaskTiles E-element slices;
// the other rows either as chain groups or as greedy row blocks of at most
// E nonzeros and E rows (see csr_tiles.cuh).  Chain groups are used for
// single-column tables (chains == true) of sides with at least
// kChainMinNonzeros nonzeros whose median row has at most kChainShort:
// there row blocks leave most lanes of every FMA idle behind the block's
// longest row, while on sides of longer rows a chain group needs many
// dependent staging passes and row blocks (a few rows of 8-lane sums)
// finish sooner.  AMFLS_GB300_CSR_CHAINS=0 in the environment turns chain
// groups off, =1 drops the size condition (for tests on small matrices).
// The table lists tasks by estimated latency, longest first (stable, so
// that the groups of a window stay together), for the kernel's snake-order
// assignment of tasks to warps.
void make_tiles(const std::vector<long long>& off, int count, int E, int C, bool chains,
                TileStore& ts, cudaStream_t stream, int force = -1) {
    using namespace csr_tiles;
    std::vector<int4> tiles;
    std::vector<int> split;
    std::vector<int2> chain, long_rows;
    std::vector<int> cost;  // dependent memory round trips of the task
    auto length = [&](int r) { return off[r + 1] - off[r]; };
    if (force >= 0) {  // the autotuner's candidates
        chains = force == 1 && count > 0;
    } else {
        if (chains) {
            const char* mode = std::getenv("AMFLS_GB300_CSR_CHAINS");
            const bool off_mode = mode && std::string(mode) == "0";
            const bool any_size = mode && std::string(mode) == "1";
            chains = !off_mode && count > 0 && (any_size || off[count] >= kChainMinNonzeros);
        }
        if (chains) {
            std::vector<long long> lens(count);
            for (int r = 0; r < count; ++r) lens[r] = length(r);
            std::nth_element(lens.begin(), lens.begin() + count / 2, lens.end());
            chains = lens[count / 2] <= kChainShort;
        }
    }
    const long long longer_than = chains ? kChainMax : E;
    const long long task = (long long)kRowTaskTiles * E;
    for (int r = 0; r < count; ++r) {
        const long long len = length(r);
        if (len <= longer_than) continue;
        if (len > task) {  // slices of one warp task each
            const int first = (int)tiles.size();
            for (long long e = off[r]; e < off[r + 1]; e += task) {
                tiles.push_back(make_int4(r, r + 1, (int)e, (int)std::min(e + task, off[r + 1])));
                split.push_back((int)long_rows.size());
                cost.push_back(2 * kRowTaskTiles + 2);
            }
            long_rows.push_back(make_int2(first, (int)tiles.size() - first));
        } else {  // one warp task for the whole row
            tiles.push_back(make_int4(r, r + 1, (int)off[r], (int)off[r + 1]));
            split.push_back(kWholeRow);
            cost.push_back(2 * (int)((len + E - 1) / E) + 1);
        }
    }
    // groups of consecutive entries of `rows` (sorted by length): up to
    // kFlatRows rows while none is longer than one, else up to 32
    auto add_groups = [&](const std::vector<int>& rows) {
        size_t g = 0;
        while (g < rows.size()) {
            long long longest = 0;
            size_t end = g;
            while (end < rows.size()) {
                const long long l = std::max(longest, length(rows[end]));
                if (end - g + 1 > (l <= 1 ? (size_t)kFlatRows : (size_t)32)) break;
                longest = l;
                ++end;
            }
            tiles.push_back(make_int4((int)chain.size(), (int)(end - g), (int)longest, 0));
            split.push_back(kChainGroup);
            cost.push_back(2 * (int)((longest + kChainStep - 1) / kChainStep) + 2);
            for (size_t i = g; i < end; ++i)
                chain.push_back(make_int2(rows[i], length(rows[i]) > 0 ? (int)off[rows[i]] : -1));
            g = end;
        }
    };
    if (chains) {
        // chain rows longer than kChainShort: by length (longest first) over
        // the whole side, stable in row order
        std::vector<int> rows;
        for (int r = 0; r < count; ++r)
            if (length(r) > kChainShort && length(r) <= kChainMax) rows.push_back(r);
        std::stable_sort(rows.begin(), rows.end(),
                         [&](int a, int b) { return length(a) > length(b); });
        add_groups(rows);
        // short rows: windows of kChainWindow consecutive ones, sorted by
        // length within the window (a counting sort, stable in row order)
        std::vector<int> window, sorted;
        auto flush = [&] {
            std::vector<int> start(kChainShort + 2, 0);
            for (int r : window) ++start[length(r) + 1];
            for (int l = 0; l <= kChainShort; ++l) start[l + 1] += start[l];
            sorted.assign(window.size(), 0);
            for (int r : window) sorted[start[length(r)]++] = r;
            add_groups(sorted);
            window.clear();
        };
        for (int r = 0; r < count; ++r) {
            if (length(r) > kChainShort) continue;
            window.push_back(r);
            if ((int)window.size() == kChainWindow) flush();
        }
        if (!window.empty()) flush();
    } else {
        int r = 0;
        while (r < count) {
            if (length(r) > longer_than) {
                ++r;
                continue;
            }
            const int r0 = r;
            const long long e0 = off[r];
            while (r < count && length(r) <= longer_than && off[r + 1] - e0 <= E && r - r0 < E)
                ++r;
            tiles.push_back(make_int4(r0, r, (int)e0, (int)off[r]));
            split.push_back(kRowBlock);
            cost.push_back(3);
        }
    }
    // longest first; slices of one row stay adjacent (equal cost, inserted
    // together), and each long row's first slice index follows the move
    std::vector<int> order(tiles.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<int4> tiles_sorted(tiles.size());
    std::vector<int> split_sorted(tiles.size());
    std::vector<char> seen(long_rows.size(), 0);
    for (size_t i = 0; i < order.size(); ++i) {
        tiles_sorted[i] = tiles[order[i]];
        split_sorted[i] = split[order[i]];
        const int q = split_sorted[i];
        if (q >= 0 && !seen[q]) {
            seen[q] = 1;
            long_rows[q].x = (int)i;
        }
    }
    tiles.swap(tiles_sorted);
    split.swap(split_sorted);

    ts.ntiles = (int)tiles.size();
    ts.nnz = (int)off[count];
    ts.chains = chains;
    const size_t nt = std::max<size_t>(1, tiles.size()), nl = std::max<size_t>(1, long_rows.size());
    const size_t nc = std::max<size_t>(1, chain.size());
    AMFLS_CUDA(cudaMalloc(&ts.tiles, sizeof(int4) * nt));
    AMFLS_CUDA(cudaMalloc(&ts.split, sizeof(int) * nt));
    AMFLS_CUDA(cudaMalloc(&ts.chain, sizeof(int2) * nc));
    AMFLS_CUDA(cudaMalloc(&ts.long_rows, sizeof(int2) * nl));
    AMFLS_CUDA(cudaMalloc(&ts.long_count, sizeof(unsigned) * nl));
    AMFLS_CUDA(cudaMalloc(&ts.long_part, sizeof(double) * C * nt));
    AMFLS_CUDA(cudaMemsetAsync(ts.long_count, 0, sizeof(unsigned) * nl, stream));
    if (!tiles.empty()) {
        AMFLS_CUDA(cudaMemcpyAsync(ts.tiles, tiles.data(), sizeof(int4) * tiles.size(),
                                   cudaMemcpyHostToDevice, stream));
        AMFLS_CUDA(cudaMemcpyAsync(ts.split, split.data(), sizeof(int) * split.size(),
                                   cudaMemcpyHostToDevice, stream));
    }
    if (!chain.empty())
        AMFLS_CUDA(cudaMemcpyAsync(ts.chain, chain.data(), sizeof(int2) * chain.size(),
                                   cudaMemcpyHostToDevice, stream));
    if (!long_rows.empty())
        AMFLS_CUDA(cudaMemcpyAsync(ts.long_rows, long_rows.data(),
                                   sizeof(int2) * long_rows.size(), cudaMemcpyHostToDevice,
                                   stream));
    AMFLS_CUDA(cudaStreamSynchronize(stream));  // host vectors go out of scope
}

// Column-major block (rows x ncols, leading dimension ld) -> row-major
// rows x C, zero-padded beyond ncols.
template <int C>
__global__ void rows_major_kernel(const double* __restrict__ x, long long ld, int rows, int ncols,
                                  double* __restrict__ xr) {
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < rows;
         j += (long long)gridDim.x * blockDim.x) {
        double v[C];
#pragma unroll
        for (int c = 0; c < C; ++c) v[c] = c < ncols ? x[j + c * ld] : 0.0;
        double2* dst = reinterpret_cast<double2*>(xr + j * C);
#pragma unroll
        for (int h = 0; h < C / 2; ++h) dst[h] = make_double2(v[2 * h], v[2 * h + 1]);
    }
}

// Resident CTAs for a tile kernel (every warp of the grid walks its own
// tiles), at most one warp per tile and at most max_blocks() CTAs.
template <typename V, int C, int E, bool kFused, bool kChains>
int tile_grid(int ntiles) {
    // resident CTAs per SM and SM count, set up once per instantiation (a
    // function-local static is initialised once even with concurrent callers)
    static const std::pair<int, int> occ = [] {
        constexpr int bytes = csr_tiles::smem_bytes<C, E>();
        auto kernel = csr_tiles::tile_product_kernel<V, C, E, kFused, kChains>;
        AMFLS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        int dev = 0, nb = 0, sms = 0;
        AMFLS_CUDA(cudaGetDevice(&dev));
        AMFLS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        AMFLS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, csr_tiles::kThreads,
                                                                 bytes));
        return std::make_pair(std::max(1, nb), sms);
    }();
    const int need = (ntiles + csr_tiles::kWarps - 1) / csr_tiles::kWarps;
    return std::max(1, std::min({need, occ.first * occ.second, max_blocks()}));
}

template <int C, bool kFused, bool kChains, typename V>
void launch_tiles_as(const int* off, const int* idx, const V* val, const TileStore& ts,
                     const double* x, double* y, long long ldy, int ncols, const Epilogue& ep,
                     double* partials, unsigned* counter, cudaStream_t stream) {
    constexpr int E = C == 1 ? csr_tiles::kE1 : csr_tiles::kEC;
    const int grid = tile_grid<V, C, E, kFused, kChains>(ts.ntiles);
    csr_tiles::tile_product_kernel<V, C, E, kFused, kChains>
        <<<grid, csr_tiles::kThreads, csr_tiles::smem_bytes<C, E>(), stream>>>(
            off, idx, val, ts.view(), x, y, ldy, ncols, ep, partials, counter);
    AMFLS_LAUNCHED();
}

template <int C, bool kFused, typename V>
void launch_tiles(const int* off, const int* idx, const V* val, const TileStore& ts,
                  const double* x, double* y, long long ldy, int ncols, const Epilogue& ep,
                  double* partials, unsigned* counter, cudaStream_t stream) {
    if constexpr (C == 1) {
        if (ts.chains) {
            launch_tiles_as<C, kFused, true>(off, idx, val, ts, x, y, ldy, ncols, ep, partials,
                                             counter, stream);
            return;
        }
    }
    launch_tiles_as<C, kFused, false>(off, idx, val, ts, x, y, ldy, ncols, ep, partials, counter,
                                      stream);
}

// Resident grid of the row-vector kernel, at most the blocks its warp tasks
// need and max_blocks().
template <typename V>
int vector_grid(long long warp_tasks) {
    static const int resident = [] {
        int dev = 0, nb = 0, sms = 0;
        AMFLS_CUDA(cudaGetDevice(&dev));
        AMFLS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        AMFLS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &nb, csr_vector::vector_product_kernel<V>, csr_vector::kThreads, 0));
        return std::max(1, nb) * sms;
    }();
    const long long need = (warp_tasks + csr_vector::kWarps - 1) / csr_vector::kWarps;
    return (int)std::max<long long>(1, std::min<long long>({need, (long long)resident,
                                                            (long long)max_blocks()}));
}

template <typename V>
void launch_vector(const int* off, const int* idx, const V* val, const csr_vector::Table& vt,
                   const double* x, const Epilogue& ep, double* partials, unsigned* counter,
                   cudaStream_t stream) {
    const int grid = vector_grid<V>(vt.warp_start[csr_vector::kBins]);
    csr_vector::vector_product_kernel<V><<<grid, csr_vector::kThreads, 0, stream>>>(
        off, idx, val, vt, x, ep, partials, counter);
    AMFLS_LAUNCHED();
}

}  // namespace

// Autotuning of the single-column tiling: sides with at least this many
// nonzeros time both tilings (row blocks, chain groups) at construction and
// keep the faster when it beats the size / row-length rule's choice by at
// least kTuneMargin; closer calls keep the rule's (deterministic) choice.
constexpr long long kTuneMinNonzeros = 1LL << 18;
constexpr double kTuneMargin = 0.10;
// The row-vector kernel replaces the kept tiling when it is at least this
// much faster (its 200 us against 222 us for chain groups on the A side of
// the 2M x 500k power-law matrix sat on the 10% line and flipped between
// runs).
constexpr double kVectorMargin = 0.05;

struct CsrOperator::Side {
    long long* off = nullptr;  // count+1
    int* off32 = nullptr;      // count+1, padded (bulk-copy source)
    int* idx = nullptr;        // nnz, padded
    double* val = nullptr;     // nnz, padded
    int* perm = nullptr;       // count (rows sorted by bin, double-double products)
    BinTable bins{};
    int count = 0;
    TileStore one;             // single-column products: chain groups or row blocks, long rows
    TileStore many;            // row blocks of kEC elements: 2..8 columns
    double tuned_us[2] = {0.0, 0.0};  // measured product time: row blocks, chain groups
    // row-vector single-column products (csr_vector.cuh): rows by bin and
    // length, used instead of `one` when `vector` is set
    int* vrows = nullptr;
    csr_vector::Table vtab{};
    bool vector = false;
    double vector_us = 0.0;
};

namespace {

// Mean device time of `reps` single-column products of one side over the
// table `ts` (after two untimed ones), CUDA events on `stream`.
double time_tiles(const int* off32, const int* idx, const double* val, const TileStore& ts,
                  const double* x, double* y, double* scratch, unsigned* counter,
                  cudaStream_t stream) {
    Epilogue ep;
    ep.out = y;
    cudaEvent_t e0, e1;
    AMFLS_CUDA(cudaEventCreate(&e0));
    AMFLS_CUDA(cudaEventCreate(&e1));
    constexpr int reps = 5;
    for (int i = 0; i < 2; ++i)
        launch_tiles<1, true>(off32, idx, val, ts, x, nullptr, 0, 1, ep, scratch, counter, stream);
    AMFLS_CUDA(cudaEventRecord(e0, stream));
    for (int i = 0; i < reps; ++i)
        launch_tiles<1, true>(off32, idx, val, ts, x, nullptr, 0, 1, ep, scratch, counter, stream);
    AMFLS_CUDA(cudaEventRecord(e1, stream));
    AMFLS_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    AMFLS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 1e3 * ms / reps;
}

// The same for the row-vector kernel.
double time_vector(const int* off32, const int* idx, const double* val,
                   const csr_vector::Table& vt, const double* x, double* y, double* scratch,
                   unsigned* counter, cudaStream_t stream) {
    Epilogue ep;
    ep.out = y;
    cudaEvent_t e0, e1;
    AMFLS_CUDA(cudaEventCreate(&e0));
    AMFLS_CUDA(cudaEventCreate(&e1));
    constexpr int reps = 5;
    for (int i = 0; i < 2; ++i) launch_vector(off32, idx, val, vt, x, ep, scratch, counter, stream);
    AMFLS_CUDA(cudaEventRecord(e0, stream));
    for (int i = 0; i < reps; ++i) launch_vector(off32, idx, val, vt, x, ep, scratch, counter, stream);
    AMFLS_CUDA(cudaEventRecord(e1, stream));
    AMFLS_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    AMFLS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 1e3 * ms / reps;
}

// Row order and bin boundaries of the row-vector kernel: rows by bin
// (descending lanes per row), longest first within a bin, ties in row order.
void make_vector_table(const std::vector<long long>& host_off, int count, int** d_rows,
                       csr_vector::Table& vt, cudaStream_t stream) {
    std::vector<int> order(std::max(1, count));
    std::vector<int> bin(count);
    int counts[csr_vector::kBins] = {};
    for (int r = 0; r < count; ++r) {
        bin[r] = csr_vector::bin_of(host_off[r + 1] - host_off[r]);
        ++counts[bin[r]];
    }
    std::iota(order.begin(), order.begin() + count, 0);
    std::stable_sort(order.begin(), order.begin() + count, [&](int a, int b) {
        if (bin[a] != bin[b]) return bin[a] < bin[b];
        return host_off[a + 1] - host_off[a] > host_off[b + 1] - host_off[b];
    });
    vt.row_start[0] = 0;
    vt.warp_start[0] = 0;
    for (int b = 0; b < csr_vector::kBins; ++b) {
        vt.row_start[b + 1] = vt.row_start[b] + counts[b];
        const long long per_warp = 1LL << b;
        vt.warp_start[b + 1] = vt.warp_start[b] + (counts[b] + per_warp - 1) / per_warp;
    }
    AMFLS_CUDA(cudaMalloc(d_rows, sizeof(int) * std::max(1, count)));
    AMFLS_CUDA(cudaMemcpyAsync(*d_rows, order.data(), sizeof(int) * std::max(1, count),
                               cudaMemcpyHostToDevice, stream));
    AMFLS_CUDA(cudaStreamSynchronize(stream));  // `order` goes out of scope
    vt.rows = *d_rows;
}

}  // namespace

CsrOperator::CsrOperator(int rows, int cols, const long long* d_offsets,
                         const long long* d_indices, const double* d_values, long long nnz,
                         cudaStream_t stream, int elems_per_lane)
    : rows_(rows), cols_(cols), nnz_(nnz), elems_per_lane_(elems_per_lane) {
    if (rows <= 0 || cols <= 0 || nnz < 0 || d_offsets == nullptr)
        throw std::invalid_argument("CSR operator dimensions are invalid");
    if (nnz > 0 && (d_indices == nullptr || d_values == nullptr))
        throw std::invalid_argument("CSR operator arrays are missing");
    if (nnz >= (1LL << 31))
        throw std::invalid_argument("CSR operator supports at most 2^31-1 nonzeros");
    a_ = std::make_unique<Side>();
    t_ = std::make_unique<Side>();
    try {
        build(d_offsets, d_indices, d_values, stream);
    } catch (...) {
        release();
        throw;
    }
}

CsrOperator::~CsrOperator() { release(); }

void CsrOperator::release() {
    for (Side* s : {a_.get(), t_.get()}) {
        if (!s) continue;
        cudaFree(s->off);
        cudaFree(s->idx);
        cudaFree(s->val);
        cudaFree(s->perm);
        cudaFree(s->off32);
        s->off = nullptr;
        s->idx = nullptr;
        s->val = nullptr;
        s->perm = nullptr;
        s->off32 = nullptr;
        s->one.release();
        s->many.release();
        cudaFree(s->vrows);
        s->vrows = nullptr;
    }
    cudaFree(scratch_);
    scratch_ = nullptr;
    cudaFree(xrows_);
    xrows_ = nullptr;
}

void CsrOperator::build_bins(Side& s, const int* d_bins, cudaStream_t stream) {
    // stable sort rows by bin -> perm; bin boundaries from a histogram
    const int n = s.count;
    int *keys_in = nullptr, *keys_out = nullptr, *vals_in = nullptr;
    AMFLS_CUDA(cudaMallocAsync(&keys_out, sizeof(int) * std::max(1, n), stream));
    AMFLS_CUDA(cudaMallocAsync(&vals_in, sizeof(int) * std::max(1, n), stream));
    AMFLS_CUDA(cudaMalloc(&s.perm, sizeof(int) * std::max(1, n)));
    keys_in = const_cast<int*>(d_bins);
    {
        std::vector<int> seq(n);
        for (int i = 0; i < n; ++i) seq[i] = i;
        AMFLS_CUDA(cudaMemcpyAsync(vals_in, seq.data(), sizeof(int) * n, cudaMemcpyHostToDevice,
                                   stream));
        size_t tmp_bytes = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys_in, keys_out, vals_in, s.perm, n,
                                        0, 3, stream);
        void* tmp = nullptr;
        AMFLS_CUDA(cudaMallocAsync(&tmp, std::max<size_t>(tmp_bytes, 1), stream));
        AMFLS_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys_in, keys_out, vals_in,
                                                   s.perm, n, 0, 3, stream));
        std::vector<int> sorted(n);
        AMFLS_CUDA(cudaMemcpyAsync(sorted.data(), keys_out, sizeof(int) * n,
                                   cudaMemcpyDeviceToHost, stream));
        AMFLS_CUDA(cudaStreamSynchronize(stream));
        AMFLS_CUDA(cudaFreeAsync(tmp, stream));
        long long counts[6] = {0, 0, 0, 0, 0, 0};
        for (int v : sorted) counts[v]++;
        s.bins.warp_start[0] = 0;
        s.bins.row_start[0] = 0;
        for (int b = 0; b < 6; ++b) {
            const long long rows_per_warp = 32 >> b;
            s.bins.warp_start[b + 1] =
                s.bins.warp_start[b] + (counts[b] + rows_per_warp - 1) / rows_per_warp;
            s.bins.row_start[b + 1] = s.bins.row_start[b] + (int)counts[b];
        }
    }
    AMFLS_CUDA(cudaFreeAsync(keys_out, stream));
    AMFLS_CUDA(cudaFreeAsync(vals_in, stream));
}

void CsrOperator::build(const long long* d_off, const long long* d_idx, const double* d_val,
                        cudaStream_t stream) {
    const long long nnz = nnz_;
    Side& A = *a_;
    Side& T = *t_;
    A.count = rows_;
    T.count = cols_;
    AMFLS_CUDA(cudaMalloc(&scratch_, sizeof(double) * (6 * kMaxGridCap + 64) + 64));
    counter_ = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(scratch_) +
                                           sizeof(double) * (6 * kMaxGridCap + 64));
    AMFLS_CUDA(cudaMemsetAsync(counter_, 0, 64, stream));
    AMFLS_CUDA(cudaMalloc(&A.off, sizeof(long long) * (rows_ + 1)));
    AMFLS_CUDA(cudaMalloc(&xrows_, sizeof(double) * 8 * (size_t)std::max(rows_, cols_)));
    const long long np = padded(nnz);
    AMFLS_CUDA(cudaMalloc(&A.idx, sizeof(int) * np));
    AMFLS_CUDA(cudaMalloc(&A.val, sizeof(double) * np));
    AMFLS_CUDA(cudaMalloc(&T.off, sizeof(long long) * (cols_ + 1)));
    AMFLS_CUDA(cudaMalloc(&T.idx, sizeof(int) * np));
    AMFLS_CUDA(cudaMalloc(&T.val, sizeof(double) * np));
    for (Side* sd : {&A, &T}) {
        AMFLS_CUDA(cudaMemsetAsync(sd->idx + nnz, 0, sizeof(int) * (np - nnz), stream));
        AMFLS_CUDA(cudaMemsetAsync(sd->val + nnz, 0, sizeof(double) * (np - nnz), stream));
        AMFLS_CUDA(cudaMalloc(&sd->off32, sizeof(int) * padded(sd->count + 1)));
        AMFLS_CUDA(cudaMemsetAsync(sd->off32, 0, sizeof(int) * padded(sd->count + 1), stream));
    }
    AMFLS_CUDA(cudaMemcpyAsync(A.off, d_off, sizeof(long long) * (rows_ + 1),
                               cudaMemcpyDeviceToDevice, stream));
    if (nnz > 0)
        AMFLS_CUDA(cudaMemcpyAsync(A.val, d_val, sizeof(double) * nnz, cudaMemcpyDeviceToDevice,
                                   stream));

    // work arrays: [err, pad][max_row_len][max_col_len] + row lens/bins + row_of + perm
    struct Work {
        int err;
        int pad;
        unsigned long long max_len_r;
        unsigned long long max_len_c;
        double row_acc[4];
        double col_acc[4];
        double frob2;
        double model[2];
    };
    Work* w = nullptr;
    AMFLS_CUDA(cudaMallocAsync(&w, sizeof(Work), stream));
    AMFLS_CUDA(cudaMemsetAsync(w, 0, sizeof(Work), stream));
    int *lens = nullptr, *bins = nullptr, *row_of = nullptr, *perm = nullptr, *counts = nullptr;
    const long long big = std::max<long long>(1, std::max<long long>(rows_, cols_));
    AMFLS_CUDA(cudaMallocAsync(&lens, sizeof(int) * big, stream));
    AMFLS_CUDA(cudaMallocAsync(&bins, sizeof(int) * big, stream));
    AMFLS_CUDA(cudaMallocAsync(&row_of, sizeof(int) * std::max<long long>(1, nnz), stream));
    AMFLS_CUDA(cudaMallocAsync(&perm, sizeof(int) * std::max<long long>(1, nnz), stream));
    AMFLS_CUDA(cudaMallocAsync(&counts, sizeof(int) * (cols_ + 1), stream));

    check_offsets_kernel<<<setup_grid(rows_), 256, 0, stream>>>(
        A.off, rows_, nnz, &w->err, &w->max_len_r, lens, elems_per_lane_, bins);
    AMFLS_LAUNCHED();
    int err = 0;
    AMFLS_CUDA(cudaMemcpyAsync(&err, &w->err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    AMFLS_CUDA(cudaStreamSynchronize(stream));
    auto fail = [&](const char* msg) {
        cudaFreeAsync(w, stream);
        cudaFreeAsync(lens, stream);
        cudaFreeAsync(bins, stream);
        cudaFreeAsync(row_of, stream);
        cudaFreeAsync(perm, stream);
        cudaFreeAsync(counts, stream);
        cudaStreamSynchronize(stream);
        throw std::invalid_argument(msg);
    };
    if (err & 2) fail("CSR row offsets do not span the values");
    if (err & 1) fail("CSR row offsets must be nondecreasing");
    build_bins(A, bins, stream);

    expand_rows_kernel<<<setup_grid(rows_), 256, 0, stream>>>(A.off, d_idx, d_val, rows_, cols_,
                                                              A.idx, row_of, &w->err);
    AMFLS_LAUNCHED();
    AMFLS_CUDA(cudaMemcpyAsync(&err, &w->err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    AMFLS_CUDA(cudaStreamSynchronize(stream));
    if (err & 4) fail("CSR column index is out of range");
    if (err & 8) fail("CSR values must be finite");

    // transpose: stable sort of entry ids by column
    AMFLS_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * (cols_ + 1), stream));
    if (nnz > 0) {
        count_columns_kernel<<<setup_grid(nnz), 256, 0, stream>>>(A.idx, nnz, counts);
        AMFLS_LAUNCHED();
        int* keys_sorted = nullptr;
        AMFLS_CUDA(cudaMallocAsync(&keys_sorted, sizeof(int) * nnz, stream));
        int* ids = perm;  // entry ids 0..nnz-1, the sort's payload
        fill_ids(ids, nnz, stream);
        int bits = 1;
        while ((1LL << bits) < cols_) ++bits;
        size_t tmp_bytes = 0;
        int* perm_out = nullptr;
        AMFLS_CUDA(cudaMallocAsync(&perm_out, sizeof(int) * nnz, stream));
        cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, A.idx, keys_sorted, ids, perm_out,
                                        (int)nnz, 0, bits, stream);
        void* tmp = nullptr;
        AMFLS_CUDA(cudaMallocAsync(&tmp, std::max<size_t>(1, tmp_bytes), stream));
        AMFLS_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, A.idx, keys_sorted, ids,
                                                   perm_out, (int)nnz, 0, bits, stream));
        gather_transpose_kernel<<<setup_grid(nnz), 256, 0, stream>>>(perm_out, row_of, A.val, nnz,
                                                                     T.idx, T.val);
        AMFLS_LAUNCHED();
        AMFLS_CUDA(cudaFreeAsync(tmp, stream));
        AMFLS_CUDA(cudaFreeAsync(perm_out, stream));
        AMFLS_CUDA(cudaFreeAsync(keys_sorted, stream));
    }
    // column offsets = exclusive scan of counts (counts[cols] = 0 gives the total)
    {
        size_t tb = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tb, counts, T.off, cols_ + 1, stream);
        void* tmp = nullptr;
        AMFLS_CUDA(cudaMallocAsync(&tmp, std::max<size_t>(1, tb), stream));
        // int counts -> long long offsets
        AMFLS_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, counts, T.off, cols_ + 1, stream));
        AMFLS_CUDA(cudaFreeAsync(tmp, stream));
    }
    duplicate_kernel<<<setup_grid(cols_), 256, 0, stream>>>(T.off, T.idx, cols_, &w->err);
    AMFLS_LAUNCHED();
    AMFLS_CUDA(cudaMemcpyAsync(&err, &w->err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    AMFLS_CUDA(cudaStreamSynchronize(stream));
    if (err & 16) fail("CSR rows must not contain duplicate columns");

    // transpose bins
    check_offsets_kernel<<<setup_grid(cols_), 256, 0, stream>>>(
        T.off, cols_, nnz, &w->err, &w->max_len_c, lens, elems_per_lane_, bins);
    AMFLS_LAUNCHED();
    build_bins(T, bins, stream);

    // int32 offsets and tilings of both sides for the streamed products
    for (Side* sd : {&A, &T}) {
        narrow_offsets_kernel<<<setup_grid(sd->count + 1), 256, 0, stream>>>(sd->off, sd->count,
                                                                             sd->off32);
        AMFLS_LAUNCHED();
        std::vector<long long> host_off(sd->count + 1);
        AMFLS_CUDA(cudaMemcpyAsync(host_off.data(), sd->off, sizeof(long long) * (sd->count + 1),
                                   cudaMemcpyDeviceToHost, stream));
        AMFLS_CUDA(cudaStreamSynchronize(stream));
        make_tiles(host_off, sd->count, csr_tiles::kE1, 1, true, sd->one, stream);
        make_tiles(host_off, sd->count, csr_tiles::kEC, 8, false, sd->many, stream);
        tune_single_column(*sd, host_off, stream);
    }

    // certified norm model
    norm_model_kernel<<<setup_grid(rows_), 256, 0, stream>>>(A.off, A.val, rows_, 0, w->row_acc,
                                                            nullptr, nullptr, nullptr);
    AMFLS_LAUNCHED();
    const int cgrid = setup_grid(cols_);
    double* frob_partials = nullptr;
    AMFLS_CUDA(cudaMallocAsync(&frob_partials, sizeof(double) * cgrid, stream));
    norm_model_kernel<<<cgrid, 256, 0, stream>>>(T.off, T.val, cols_, 1, w->col_acc,
                                                 frob_partials, counter_, &w->frob2);
    AMFLS_LAUNCHED();
    finish_model_kernel<<<1, 1, 0, stream>>>(w->row_acc, w->col_acc, &w->frob2, w->model);
    AMFLS_LAUNCHED();
    Work host{};
    AMFLS_CUDA(cudaMemcpyAsync(&host, w, sizeof(Work), cudaMemcpyDeviceToHost, stream));
    AMFLS_CUDA(cudaStreamSynchronize(stream));
    model_.norm_upper = host.model[0];
    model_.norm_lower = host.model[1];
    model_.apply_steps = 2LL * (long long)host.max_len_r + 2LL;
    model_.transpose_steps = 2LL * (long long)host.max_len_c + 2LL;
    max_row_nnz_ = (long long)host.max_len_r;
    max_col_nnz_ = (long long)host.max_len_c;

    AMFLS_CUDA(cudaFreeAsync(frob_partials, stream));
    AMFLS_CUDA(cudaFreeAsync(w, stream));
    AMFLS_CUDA(cudaFreeAsync(lens, stream));
    AMFLS_CUDA(cudaFreeAsync(bins, stream));
    AMFLS_CUDA(cudaFreeAsync(row_of, stream));
    AMFLS_CUDA(cudaFreeAsync(perm, stream));
    AMFLS_CUDA(cudaFreeAsync(counts, stream));
    AMFLS_CUDA(cudaStreamSynchronize(stream));
}

namespace {
__global__ void fill_ids_kernel(int* ids, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        ids[i] = (int)i;
}
}  // namespace

void CsrOperator::fill_ids(int* ids, long long n, cudaStream_t stream) {
    fill_ids_kernel<<<setup_grid(n), 256, 0, stream>>>(ids, n);
    AMFLS_LAUNCHED();
}

namespace {

// Single-column product of one side with a fused epilogue: the row-vector
// kernel when the side's autotuner chose it (vt non-null), else the tiles.
template <typename V>
void side_product1(const int* off32, const int* idx, const V* vals, const TileStore& one,
                   const double* x, const Epilogue& ep, double* partials, unsigned* counter,
                   cudaStream_t stream, const csr_vector::Table* vt = nullptr) {
    if (vt) {
        launch_vector(off32, idx, vals, *vt, x, ep, partials, counter, stream);
        return;
    }
    launch_tiles<1, true>(off32, idx, vals, one, x, nullptr, 0, 1, ep, partials, counter, stream);
}

// Block product of one side: eight columns per pass, each pass staging its
// columns row-major in `xrows` (ldx x 8).
template <typename V>
void side_block(const int* off32, const int* idx, const V* vals, const TileStore& one,
                const TileStore& many, const double* x, long long ldx, int block_cols,
                double* y, long long ldy, double* xrows, double* partials, unsigned* counter,
                cudaStream_t stream, const csr_vector::Table* vt = nullptr) {
    const Epilogue none;
    const int tgrid = setup_grid(ldx);
    for (int c0 = 0; c0 < block_cols; c0 += 8) {
        const int nc = std::min(8, block_cols - c0);
        const double* xc = x + c0 * ldx;
        double* yc = y + c0 * ldy;
        if (nc > 4) {
            rows_major_kernel<8><<<tgrid, 256, 0, stream>>>(xc, ldx, (int)ldx, nc, xrows);
            AMFLS_LAUNCHED();
            launch_tiles<8, false>(off32, idx, vals, many, xrows, yc, ldy, nc, none, nullptr,
                                   nullptr, stream);
        } else if (nc > 2) {
            rows_major_kernel<4><<<tgrid, 256, 0, stream>>>(xc, ldx, (int)ldx, nc, xrows);
            AMFLS_LAUNCHED();
            launch_tiles<4, false>(off32, idx, vals, many, xrows, yc, ldy, nc, none, nullptr,
                                   nullptr, stream);
        } else if (nc == 2) {
            rows_major_kernel<2><<<tgrid, 256, 0, stream>>>(xc, ldx, (int)ldx, nc, xrows);
            AMFLS_LAUNCHED();
            launch_tiles<2, false>(off32, idx, vals, many, xrows, yc, ldy, nc, none, nullptr,
                                   nullptr, stream);
        } else {
            Epilogue ep;
            ep.out = yc;
            side_product1(off32, idx, vals, one, xc, ep, partials, counter, stream, vt);
        }
    }
}

template <typename V>
__global__ void narrow_values_kernel(const double* in, long long n, V* out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        if constexpr (std::is_same_v<V, float>)
            out[i] = __double2float_rn(in[i]);
        else
            out[i] = __double2bfloat16(in[i]);
    }
}

}  // namespace

// The autotuner: time the rule's table and the other tiling on this side
// (products of a zero vector: the memory traffic and the instruction stream
// do not depend on the values) and keep the faster one when it wins by at
// least kTuneMargin.  AMFLS_GB300_CSR_CHAINS (either value) turns it off.
void CsrOperator::tune_single_column(Side& sd, const std::vector<long long>& host_off,
                                     cudaStream_t stream) {
    const char* force_vector = std::getenv("AMFLS_GB300_CSR_VECTOR");
    if (force_vector && force_vector[0] == '1' && sd.count > 0) {
        make_vector_table(host_off, sd.count, &sd.vrows, sd.vtab, stream);
        sd.vector = true;
        return;
    }
    if (std::getenv("AMFLS_GB300_CSR_CHAINS") || sd.count <= 0 ||
        host_off[sd.count] < kTuneMinNonzeros)
        return;
    const long long in = &sd == a_.get() ? cols_ : rows_;
    TileStore alt;
    make_tiles(host_off, sd.count, csr_tiles::kE1, 1, true, alt, stream, sd.one.chains ? 0 : 1);
    double *x = nullptr, *y = nullptr;
    AMFLS_CUDA(cudaMallocAsync(&x, sizeof(double) * in, stream));
    AMFLS_CUDA(cudaMallocAsync(&y, sizeof(double) * sd.count, stream));
    AMFLS_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * in, stream));
    const double t_rule = time_tiles(sd.off32, sd.idx, sd.val, sd.one, x, y, scratch_, counter_,
                                     stream);
    const double t_alt = time_tiles(sd.off32, sd.idx, sd.val, alt, x, y, scratch_, counter_,
                                    stream);
    // the row-vector kernel is the third candidate (AMFLS_GB300_CSR_VECTOR=0
    // leaves it out)
    double t_vec = 0.0;
    if (!(force_vector && force_vector[0] == '0')) {
        make_vector_table(host_off, sd.count, &sd.vrows, sd.vtab, stream);
        t_vec = time_vector(sd.off32, sd.idx, sd.val, sd.vtab, x, y, scratch_, counter_, stream);
    }
    AMFLS_CUDA(cudaFreeAsync(x, stream));
    AMFLS_CUDA(cudaFreeAsync(y, stream));
    AMFLS_CUDA(cudaStreamSynchronize(stream));
    sd.tuned_us[sd.one.chains ? 1 : 0] = t_rule;
    sd.tuned_us[alt.chains ? 1 : 0] = t_alt;
    sd.vector_us = t_vec;
    double best = t_rule;
    if (t_alt < (1.0 - kTuneMargin) * t_rule) {
        std::swap(sd.one, alt);
        best = t_alt;
    }
    alt.release();
    if (sd.vrows && t_vec < (1.0 - kVectorMargin) * best) {
        sd.vector = true;
    } else if (sd.vrows) {
        cudaFree(sd.vrows);
        sd.vrows = nullptr;
        sd.vtab = csr_vector::Table{};
    }
}

void CsrOperator::single_column_schedule(int chains[2], double microseconds[4]) const {
    const Side* sides[2] = {a_.get(), t_.get()};
    for (int i = 0; i < 2; ++i) {
        chains[i] = sides[i]->vector ? 2 : (sides[i]->one.chains ? 1 : 0);
        microseconds[2 * i] = sides[i]->tuned_us[0];
        microseconds[2 * i + 1] = sides[i]->tuned_us[1];
    }
}

bool CsrOperator::product1(bool transpose, const double* x, const Epilogue& ep,
                           cudaStream_t stream) const {
    const Side& s = transpose ? *t_ : *a_;
    side_product1(s.off32, s.idx, s.val, s.one, x, ep, ep.partials ? ep.partials : scratch_,
                  ep.counter ? ep.counter : counter_, stream, s.vector ? &s.vtab : nullptr);
    return true;
}

void CsrOperator::product(bool transpose, const double* x, int block_cols, double* y,
                          cudaStream_t stream) const {
    if (x == nullptr || y == nullptr || block_cols <= 0)
        throw std::invalid_argument("CSR product block is invalid");
    const Side& s = transpose ? *t_ : *a_;
    side_block(s.off32, s.idx, s.val, s.one, s.many, x, transpose ? rows_ : cols_, block_cols, y,
               transpose ? cols_ : rows_, xrows_, scratch_, counter_, stream,
               s.vector ? &s.vtab : nullptr);
}

// ------------------------------------------------- reduced precision ----

ReducedCsrOperator::ReducedCsrOperator(const CsrOperator& src, ValueType type,
                                       cudaStream_t stream)
    : src_(src), type_(type) {
    if (type != ValueType::fp32 && type != ValueType::bf16)
        throw std::invalid_argument("reduced CSR values must be FP32 or BF16");
    const long long np = padded(src.nnz_);
    const size_t vb = type == ValueType::fp32 ? 4 : 2;
    try {
        for (int side = 0; side < 2; ++side) {
            const double* in = side ? src.t_->val : src.a_->val;
            AMFLS_CUDA(cudaMalloc(&vals_[side], vb * np));
            AMFLS_CUDA(cudaMemsetAsync(vals_[side], 0, vb * np, stream));
            if (src.nnz_ > 0) {
                if (type == ValueType::fp32)
                    narrow_values_kernel<float><<<setup_grid(src.nnz_), 256, 0, stream>>>(
                        in, src.nnz_, static_cast<float*>(vals_[side]));
                else
                    narrow_values_kernel<__nv_bfloat16><<<setup_grid(src.nnz_), 256, 0, stream>>>(
                        in, src.nnz_, static_cast<__nv_bfloat16*>(vals_[side]));
                AMFLS_LAUNCHED();
            }
        }
        AMFLS_CUDA(cudaMalloc(&xrows_, sizeof(double) * 8 * (size_t)std::max(src.rows_, src.cols_)));
        AMFLS_CUDA(cudaMalloc(&scratch_, sizeof(double) * 6 * kMaxGridCap + 64));
        counter_ = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(scratch_) +
                                               sizeof(double) * 6 * kMaxGridCap);
        AMFLS_CUDA(cudaMemsetAsync(counter_, 0, 64, stream));
        AMFLS_CUDA(cudaStreamSynchronize(stream));
    } catch (...) {
        release();
        throw;
    }
    model_ = reduced_model(src.validation_error_model(), type);
}

ReducedCsrOperator::~ReducedCsrOperator() { release(); }

void ReducedCsrOperator::release() {
    for (void*& v : vals_) {
        cudaFree(v);
        v = nullptr;
    }
    cudaFree(xrows_);
    cudaFree(scratch_);
    xrows_ = nullptr;
    scratch_ = nullptr;
}

bool ReducedCsrOperator::product1(bool transpose, const double* x, const Epilogue& ep,
                                  cudaStream_t stream) const {
    const CsrOperator::Side& s = transpose ? *src_.t_ : *src_.a_;
    double* partials = ep.partials ? ep.partials : scratch_;
    unsigned* counter = ep.counter ? ep.counter : counter_;
    const void* v = vals_[transpose ? 1 : 0];
    const csr_vector::Table* vt = s.vector ? &s.vtab : nullptr;
    if (type_ == ValueType::fp32)
        side_product1(s.off32, s.idx, static_cast<const float*>(v), s.one, x, ep, partials,
                      counter, stream, vt);
    else
        side_product1(s.off32, s.idx, static_cast<const __nv_bfloat16*>(v), s.one, x, ep,
                      partials, counter, stream, vt);
    return true;
}

void ReducedCsrOperator::product(bool transpose, const double* x, int block_cols, double* y,
                                 cudaStream_t stream) const {
    if (x == nullptr || y == nullptr || block_cols <= 0)
        throw std::invalid_argument("CSR product block is invalid");
    const CsrOperator::Side& s = transpose ? *src_.t_ : *src_.a_;
    const long long ldx = transpose ? src_.rows_ : src_.cols_;
    const long long ldy = transpose ? src_.cols_ : src_.rows_;
    const void* v = vals_[transpose ? 1 : 0];
    const csr_vector::Table* vt = s.vector ? &s.vtab : nullptr;
    if (type_ == ValueType::fp32)
        side_block(s.off32, s.idx, static_cast<const float*>(v), s.one, s.many, x, ldx,
                   block_cols, y, ldy, xrows_, scratch_, counter_, stream, vt);
    else
        side_block(s.off32, s.idx, static_cast<const __nv_bfloat16*>(v), s.one, s.many, x, ldx,
                   block_cols, y, ldy, xrows_, scratch_, counter_, stream, vt);
}

void ReducedCsrOperator::apply(const double* x, int block_cols, double* y, cudaStream_t s) const {
    product(false, x, block_cols, y, s);
}

void ReducedCsrOperator::apply_transpose(const double* y, int block_cols, double* x,
                                         cudaStream_t s) const {
    product(true, y, block_cols, x, s);
}

void CsrOperator::apply(const double* x, int block_cols, double* y, cudaStream_t s) const {
    product(false, x, block_cols, y, s);
}

void CsrOperator::apply_transpose(const double* y, int block_cols, double* x,
                                  cudaStream_t s) const {
    product(true, y, block_cols, x, s);
}

void CsrOperator::refined(bool transpose, const double* x_hi, const double* x_lo, double* y_hi,
                          double* y_lo, int* finite, cudaStream_t stream) const {
    const Side& s = transpose ? *t_ : *a_;
    spmv_dd_kernel<<<grid_for(s.bins.warp_start[6]), kThreads, 0, stream>>>(
        s.off, s.idx, s.val, s.perm, s.bins, x_hi, x_lo, y_hi, y_lo, finite);
    AMFLS_LAUNCHED();
}

void CsrOperator::apply_refined(const double* x_hi, const double* x_lo, double* y_hi,
                                double* y_lo, int* finite, cudaStream_t s) const {
    refined(false, x_hi, x_lo, y_hi, y_lo, finite, s);
}

void CsrOperator::apply_transpose_refined(const double* y_hi, const double* y_lo, double* x_hi,
                                          double* x_lo, int* finite, cudaStream_t s) const {
    refined(true, y_hi, y_lo, x_hi, x_lo, finite, s);
}

}  // namespace amfls_gpu
