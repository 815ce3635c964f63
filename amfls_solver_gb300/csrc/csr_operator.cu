// CSR device operator: Y = A X and X = A^T Y in FP64 on sm_103a.
//
// Replaces the reference's SparseCsrOperator
// (src/algorithms/mathematics/operators/sparse_csr_operator.cpp:14-269):
//   * the constructor's one-pass validation and certified norm model
//     (offsets span the values, columns in range, no duplicate column in a
//     row, finite values; ||A|| <= min(sqrt(||A||_1 ||A||_inf), ||A||_F),
//     ||A|| >= max(max|a_ij|, max row/column 2-norm); rounding steps
//     2*max_row_nnz+2 and 2*max_col_nnz+2) runs as device kernels;
//   * apply runs a row-length-binned sub-warp SpMV: rows are grouped by
//     length and each row gets G in {1,..,32} lanes that read its nonzeros
//     contiguously and combine by a fixed butterfly, so results are
//     deterministic for a given matrix;
//   * apply_transpose does NOT scatter: it runs the same gather kernel on a
//     transpose (CSR of A^T) built once on the device with a stable sort, so
//     each column sums its entries in row order like the reference's scatter.
// Row and column sums of |a_ij| for the norm model are accumulated
// sequentially in the reference's order (rows in CSR order, columns in row
// order), so those stored sums match the reference bit for bit.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <vector>

#include "common.cuh"
#include "csr_operator.hpp"
#include "dd.cuh"
#include "epilogue.cuh"
#include "fp_bounds.cuh"

namespace amfls_gpu {

namespace {

constexpr int kThreads = 256;
constexpr int kWarpsPerBlock = kThreads / 32;
constexpr int kMaxBlocks = 152 * 8;

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

// One lane's share of a row: elements first + g t for t = 0, 1, ...,
// accumulated in that order.  Four elements' values and indices are loaded
// before their gathers so that each lane keeps several independent loads in
// flight; the streamed arrays bypass L1 and are marked evict-first so that
// the gathered vector stays in L2.
__device__ __forceinline__ double row_dot(const long long* __restrict__ off,
                                          const int* __restrict__ idx,
                                          const double* __restrict__ val,
                                          const double* __restrict__ x, int row, int first,
                                          int g) {
    const long long end = off[row + 1];
    double acc = 0.0;
    for (long long e = off[row] + first; e < end; e += 4 * g) {
        double v[4], xv[4];
        int j[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const bool in = e + u * g < end;
            v[u] = in ? __ldcs(val + e + u * g) : 0.0;
            j[u] = in ? __ldcs(idx + e + u * g) : -1;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) xv[u] = j[u] >= 0 ? __ldg(x + j[u]) : 0.0;
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (j[u] >= 0) acc = fma(v[u], xv[u], acc);
    }
    return acc;
}

__global__ void __launch_bounds__(kThreads)
spmv_binned_kernel(const long long* __restrict__ off, const int* __restrict__ idx,
                   const double* __restrict__ val, const int* __restrict__ perm, BinTable bt,
                   const double* __restrict__ x, Epilogue ep, double* partials,
                   unsigned* counter) {
    if (ep.guard && *ep.guard == 0) return;
    const int lane = threadIdx.x & 31;
    double sq_t = 0.0, sq_out = 0.0, dot = 0.0, mx_t = 0.0, mx_out = 0.0;
    int nonfin = 0;
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
        double acc = 0.0;
        if (active) acc = row_dot(off, idx, val, x, row, lane & (g - 1), g);
        for (int o = g >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (active && (lane & (g - 1)) == 0)
            epilogue_row(ep, row, acc, sq_t, sq_out, dot, mx_t, mx_out, nonfin);
    }
    finish_reduction(ep, sq_t, sq_out, dot, mx_t, mx_out, nonfin, partials, counter);
}

// Several right-hand sides: lanes share each nonzero across a chunk of up to
// 8 columns of a column-major block (x stride ldx, y stride ldy).
template <int C>
__global__ void __launch_bounds__(kThreads)
spmm_binned_kernel(const long long* __restrict__ off, const int* __restrict__ idx,
                   const double* __restrict__ val, const int* __restrict__ perm, BinTable bt,
                   const double* __restrict__ x, long long ldx, double* __restrict__ y,
                   long long ldy, int ncols) {
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
        double acc[C];
#pragma unroll
        for (int c = 0; c < C; ++c) acc[c] = 0.0;
        if (active) {
            const long long end = off[row + 1];
            long long e = off[row] + (lane & (g - 1));
            for (; e + g < end; e += 2 * g) {
                const double a0 = __ldcs(val + e), a1 = __ldcs(val + e + g);
                const int j0 = __ldcs(idx + e), j1 = __ldcs(idx + e + g);
                double x0[C], x1[C];
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    x0[c] = c < ncols ? __ldg(&x[j0 + c * ldx]) : 0.0;
                    x1[c] = c < ncols ? __ldg(&x[j1 + c * ldx]) : 0.0;
                }
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    acc[c] = fma(a0, x0[c], acc[c]);
                    acc[c] = fma(a1, x1[c], acc[c]);
                }
            }
            for (; e < end; e += g) {
                const double a = __ldcs(val + e);
                const int j = __ldcs(idx + e);
#pragma unroll
                for (int c = 0; c < C; ++c)
                    if (c < ncols) acc[c] = fma(a, __ldg(&x[j + c * ldx]), acc[c]);
            }
        }
#pragma unroll
        for (int c = 0; c < C; ++c)
            for (int o = g >> 1; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
        if (active && (lane & (g - 1)) == 0) {
#pragma unroll
            for (int c = 0; c < C; ++c)
                if (c < ncols) y[row + c * ldy] = acc[c];
        }
    }
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
    return (int)std::max<long long>(1, std::min<long long>(blocks, kMaxBlocks));
}

int setup_grid(long long items) {
    return (int)std::max<long long>(1, std::min<long long>((items + 255) / 256, 152 * 16));
}

}  // namespace

struct CsrOperator::Side {
    long long* off = nullptr;  // count+1
    int* idx = nullptr;        // nnz
    double* val = nullptr;     // nnz
    int* perm = nullptr;       // count (rows sorted by bin)
    BinTable bins{};
    int count = 0;
};

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
        s->off = nullptr;
        s->idx = nullptr;
        s->val = nullptr;
        s->perm = nullptr;
    }
    cudaFree(scratch_);
    scratch_ = nullptr;
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
    AMFLS_CUDA(cudaMalloc(&scratch_, sizeof(double) * (6 * kMaxBlocks + 64) + 64));
    counter_ = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(scratch_) +
                                           sizeof(double) * (6 * kMaxBlocks + 64));
    AMFLS_CUDA(cudaMemsetAsync(counter_, 0, 64, stream));
    AMFLS_CUDA(cudaMalloc(&A.off, sizeof(long long) * (rows_ + 1)));
    AMFLS_CUDA(cudaMalloc(&A.idx, sizeof(int) * std::max<long long>(1, nnz)));
    AMFLS_CUDA(cudaMalloc(&A.val, sizeof(double) * std::max<long long>(1, nnz)));
    AMFLS_CUDA(cudaMalloc(&T.off, sizeof(long long) * (cols_ + 1)));
    AMFLS_CUDA(cudaMalloc(&T.idx, sizeof(int) * std::max<long long>(1, nnz)));
    AMFLS_CUDA(cudaMalloc(&T.val, sizeof(double) * std::max<long long>(1, nnz)));
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

bool CsrOperator::product1(bool transpose, const double* x, const Epilogue& ep,
                           cudaStream_t stream) const {
    const Side& s = transpose ? *t_ : *a_;
    const int grid = grid_for(s.bins.warp_start[6]);
    spmv_binned_kernel<<<grid, kThreads, 0, stream>>>(
        s.off, s.idx, s.val, s.perm, s.bins, x, ep,
        ep.partials ? ep.partials : scratch_, ep.counter ? ep.counter : counter_);
    AMFLS_LAUNCHED();
    return true;
}

void CsrOperator::product(bool transpose, const double* x, int block_cols, double* y,
                          cudaStream_t stream) const {
    if (x == nullptr || y == nullptr || block_cols <= 0)
        throw std::invalid_argument("CSR product block is invalid");
    const Side& s = transpose ? *t_ : *a_;
    const long long ldx = transpose ? rows_ : cols_;
    const long long ldy = transpose ? cols_ : rows_;
    const int grid = grid_for(s.bins.warp_start[6]);
    if (block_cols == 1) {
        Epilogue ep;
        ep.out = y;
        product1(transpose, x, ep, stream);
        return;
    }
    for (int c0 = 0; c0 < block_cols; c0 += 8) {
        const int nc = std::min(8, block_cols - c0);
        spmm_binned_kernel<8><<<grid, kThreads, 0, stream>>>(
            s.off, s.idx, s.val, s.perm, s.bins, x + c0 * ldx, ldx, y + c0 * ldy, ldy, nc);
        AMFLS_LAUNCHED();
    }
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
