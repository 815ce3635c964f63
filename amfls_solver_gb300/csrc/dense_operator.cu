// Dense FP64 operator: Y = A X and X = A^T Y with A resident in HBM.
//
// Replaces DenseOperator (src/algorithms/mathematics/operators/dense_operator.cpp:20-185,
// column-major, dgemm) and RowMajorDenseOperator
// (row_major_dense_operator.cpp:106-258, row-major, the torch path).
// The product along the contiguous dimension gives each warp two outputs
// (lanes stride the contiguous index); the product across it keeps one
// output per thread (coalesced over the contiguous dimension).  Both split
// the long dimension into chunks whose partial sums a second kernel adds in
// a fixed order, so results are deterministic, and both take up to eight
// right-hand columns per pass over A.  The certified norm model and the rounding-step counts
// (2 cols + 2 for A, 2 rows + 2 for A^T) follow the reference; row and column
// sums of |a_ij| are accumulated in the reference's storage order.
// On GB300 FP64 issue rate, not HBM bandwidth, bounds these kernels
// (2 flops per 8-byte element against a ~0.18 flop/byte FP64 ridge).
#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "common.cuh"
#include "dd.cuh"
#include "dense_operator.hpp"
#include "epilogue.cuh"
#include "fp_bounds.cuh"

namespace amfls_gpu {
namespace {

constexpr int kThreads = 256;
// blocks that fill the GPU (eight per SM)
inline int target_blocks() { return grid_cap(); }

// ---- block products (s columns per pass over A, s <= 8 per launch) ----
// Both directions split the long dimension into chunks whose partial sums
// land in partial[(chunk * S + c) * outer + o]; reduce_block_kernel adds the
// chunks in a fixed order.  A is read once per group of eight columns, and
// every element read feeds S fused multiply-adds.
constexpr int kDotOutputsPerWarp = 2;

// A(o, i) at a[o * ld + i] (i contiguous): a warp owns kDotOutputsPerWarp
// outputs and strides i across its lanes.
template <int S>
__global__ void __launch_bounds__(kThreads)
dot_block_kernel(const double* __restrict__ a, long long ld, int outer, int inner, int chunk,
                 const double* __restrict__ x, long long ldx, double* partial, const int* guard) {
    constexpr int J = kDotOutputsPerWarp;
    if (guard && *guard == 0) return;
    const int lane = threadIdx.x & 31;
    const long long o0 = ((long long)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5)) * J;
    if (o0 >= outer) return;
    const int ch = blockIdx.y;
    const int i0 = ch * chunk, i1 = min(inner, i0 + chunk);
    const double* rows[J];
#pragma unroll
    for (int j = 0; j < J; ++j) rows[j] = a + min(o0 + j, (long long)outer - 1) * ld;
    double acc[J][S];
#pragma unroll
    for (int j = 0; j < J; ++j)
#pragma unroll
        for (int c = 0; c < S; ++c) acc[j][c] = 0.0;
    for (int i = i0 + lane; i < i1; i += 32) {
        double xv[S];
#pragma unroll
        for (int c = 0; c < S; ++c) xv[c] = __ldg(x + i + c * ldx);
#pragma unroll
        for (int j = 0; j < J; ++j) {
            const double av = __ldg(rows[j] + i);
#pragma unroll
            for (int c = 0; c < S; ++c) acc[j][c] = fma(av, xv[c], acc[j][c]);
        }
    }
#pragma unroll
    for (int j = 0; j < J; ++j)
#pragma unroll
        for (int c = 0; c < S; ++c) {
            const double v = warp_sum(acc[j][c]);
            if (lane == 0 && o0 + j < outer) partial[((long long)ch * S + c) * outer + o0 + j] = v;
        }
}

// A(i, o) at a[i * ld + o] (o contiguous): a thread owns one output.
template <int S>
__global__ void __launch_bounds__(kThreads)
across_block_kernel(const double* __restrict__ a, long long ld, int outer, int inner, int chunk,
                    const double* __restrict__ x, long long ldx, double* partial,
                    const int* guard) {
    if (guard && *guard == 0) return;
    const long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (o >= outer) return;
    const int ch = blockIdx.y;
    const int i0 = ch * chunk, i1 = min(inner, i0 + chunk);
    double acc[S];
#pragma unroll
    for (int c = 0; c < S; ++c) acc[c] = 0.0;
    for (int i = i0; i < i1; ++i) {
        const double av = __ldg(a + (long long)i * ld + o);
#pragma unroll
        for (int c = 0; c < S; ++c) acc[c] = fma(av, __ldg(x + i + c * ldx), acc[c]);
    }
#pragma unroll
    for (int c = 0; c < S; ++c) partial[((long long)ch * S + c) * outer + o] = acc[c];
}

__global__ void reduce_block_kernel(const double* partial, int chunks, int S, int outer,
                                    double* y, long long ldy, const int* guard) {
    if (guard && *guard == 0) return;
    const long long total = (long long)S * outer;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t / outer);
        const long long o = t % outer;
        double s = 0.0;
        for (int ch = 0; ch < chunks; ++ch) s += partial[((long long)ch * S + c) * outer + o];
        y[o + c * ldy] = s;
    }
}

// double-double variants for the validation refinement
__global__ void dd_dot_rows_kernel(const double* __restrict__ a, long long ld, int outer,
                                   int inner, const double* x_hi, const double* x_lo, double* y_hi,
                                   double* y_lo, int* finite) {
    const int lane = threadIdx.x & 31;
    for (long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; w < outer;
         w += ((long long)gridDim.x * blockDim.x) >> 5) {
        const double* row = a + w * ld;
        dd acc{0.0, 0.0};
        for (int i = lane; i < inner; i += 32)
            acc = dd_add(acc, dd_mul_d(dd{x_hi[i], x_lo ? x_lo[i] : 0.0}, row[i]));
        for (int o = 16; o > 0; o >>= 1) acc = dd_add(acc, dd_shfl_xor(acc, o));
        if (lane == 0) {
            y_hi[w] = acc.hi;
            y_lo[w] = acc.lo;
            if (!isfinite(acc.hi) || !isfinite(acc.lo)) atomicAnd(finite, 0);
        }
    }
}

__global__ void dd_sum_cols_kernel(const double* __restrict__ a, long long ld, int outer,
                                   int inner, const double* x_hi, const double* x_lo,
                                   double* y_hi, double* y_lo, int* finite) {
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < outer;
         o += (long long)gridDim.x * blockDim.x) {
        dd acc{0.0, 0.0};
        for (int i = 0; i < inner; ++i)
            acc = dd_add(acc, dd_mul_d(dd{x_hi[i], x_lo ? x_lo[i] : 0.0}, a[(long long)i * ld + o]));
        y_hi[o] = acc.hi;
        y_lo[o] = acc.lo;
        if (!isfinite(acc.hi) || !isfinite(acc.lo)) atomicAnd(finite, 0);
    }
}

// ---- norm model: sequential sums in storage order (outer loop = storage-major)
__device__ __forceinline__ void atomic_max_pos(double* addr, double v) {
    atomicMax(reinterpret_cast<unsigned long long*>(addr),
              (unsigned long long)__double_as_longlong(v));
}

// acc: [0] max outer-sum upper, [1] max two-norm lower, [2] max entry,
//      [3] max inner-sum upper, [4] nonfinite flag
__global__ void model_outer_kernel(const double* a, int outer, int inner, double* acc,
                                   double* frob_partials, unsigned* counter, double* frob_out) {
    __shared__ double scratch[32];
    double frob = 0.0;
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < outer;
         o += (long long)gridDim.x * blockDim.x) {
        double s = 0.0, q = 0.0, mx = 0.0;
        bool bad = false;
        for (int i = 0; i < inner; ++i) {
            const double m = fabs(a[o * (long long)inner + i]);
            if (!isfinite(m)) {
                bad = true;
                continue;
            }
            mx = fmax(mx, m);
            s += m;
            q = fma(m, m, q);
        }
        if (bad) atomic_max_pos(&acc[4], 1.0);
        atomic_max_pos(&acc[0], fpb::sum_upper(s, inner, true));
        atomic_max_pos(&acc[1], fpb::down_sqrt(fpb::sum_lower(q, inner)));
        atomic_max_pos(&acc[2], mx);
        frob = __dadd_ru(frob, fpb::sum_upper(q, inner, false));
    }
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
        for (unsigned b = 0; b < gridDim.x; ++b) t = __dadd_ru(t, frob_partials[b]);
        *frob_out = fpb::widen_up(t);
    }
}

// per inner index: sums over the outer dimension in order; Frobenius terms
// rounded upward per index, then summed upward by the last block
__global__ void model_inner_kernel(const double* a, int outer, int inner, double* acc,
                                   double* frob_partials, unsigned* counter, double* frob_out) {
    __shared__ double scratch[32];
    double frob = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < inner;
         i += (long long)gridDim.x * blockDim.x) {
        double s = 0.0, q = 0.0;
        for (int o = 0; o < outer; ++o) {
            const double m = fabs(a[(long long)o * inner + i]);
            if (!isfinite(m)) continue;
            s += m;
            q = fma(m, m, q);
        }
        atomic_max_pos(&acc[3], fpb::sum_upper(s, outer, true));
        atomic_max_pos(&acc[1], fpb::down_sqrt(fpb::sum_lower(q, outer)));
        frob = __dadd_ru(frob, fpb::sum_upper(q, outer, false));
    }
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
        for (unsigned b = 0; b < gridDim.x; ++b) t = __dadd_ru(t, frob_partials[b]);
        *frob_out = fpb::widen_up(t);
    }
}

__global__ void model_finish_kernel(const double* acc, const double* frob2, int row_major,
                                    double* model) {
    // row-major: outer = rows -> acc[0] is the row-sum bound (||A||_inf),
    // acc[3] the column-sum bound (||A||_1); column-major the reverse
    const double row_sum = row_major ? acc[0] : acc[3];
    const double col_sum = row_major ? acc[3] : acc[0];
    double upper = fpb::kInf;
    double lower = 0.0;
    if (acc[4] == 0.0) {
        const double one_inf = fpb::up_mul(fpb::up_sqrt(col_sum), fpb::up_sqrt(row_sum));
        upper = fmin(one_inf, fpb::up_sqrt(*frob2));
        lower = fmax(acc[2], acc[1]);
    }
    if (!isfinite(upper) || lower > upper) {
        upper = fpb::kInf;
        lower = 0.0;
    }
    model[0] = upper;
    model[1] = lower;
}

__global__ void epilogue_kernel(const double* __restrict__ t, long long n, Epilogue ep,
                                double* partials, unsigned* counter) {
    if (ep.guard && *ep.guard == 0) return;
    double sq_t = 0.0, sq_out = 0.0, dot = 0.0, mx_t = 0.0, mx_out = 0.0;
    int nonfin = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        epilogue_row(ep, (int)i, t[i], sq_t, sq_out, dot, mx_t, mx_out, nonfin);
    finish_reduction(ep, sq_t, sq_out, dot, mx_t, mx_out, nonfin, partials, counter);
}

int grid_1d(long long items) {
    return (int)std::max<long long>(1, std::min<long long>(target_blocks(), (items + 255) / 256));
}

// chunking for the block kernels: enough blocks to fill the GPU twice over
void block_chunks(bool dot, int out_n, int in_n, int& blocks_x, int& chunks, int& chunk) {
    if (dot) {
        const long long groups = (out_n + kDotOutputsPerWarp - 1) / kDotOutputsPerWarp;
        blocks_x = (int)((groups + kThreads / 32 - 1) / (kThreads / 32));
    } else {
        blocks_x = (out_n + kThreads - 1) / kThreads;
    }
    const int min_rows = dot ? 256 : 32;
    chunks = std::max(1, std::min((2 * target_blocks() + blocks_x - 1) / blocks_x,
                                  (in_n + min_rows - 1) / min_rows));
    chunk = (in_n + chunks - 1) / chunks;
    chunks = (in_n + chunk - 1) / chunk;
}

template <int S>
void launch_block(bool dot, const double* a, long long ld, int out_n, int in_n, const double* x,
                  long long ldx, double* partial, double* y, long long ldy, cudaStream_t s,
                  const int* guard = nullptr) {
    int blocks_x = 0, chunks = 0, chunk = 0;
    block_chunks(dot, out_n, in_n, blocks_x, chunks, chunk);
    const dim3 grid(blocks_x, chunks);
    if (dot)
        dot_block_kernel<S><<<grid, kThreads, 0, s>>>(a, ld, out_n, in_n, chunk, x, ldx, partial,
                                                       guard);
    else
        across_block_kernel<S><<<grid, kThreads, 0, s>>>(a, ld, out_n, in_n, chunk, x, ldx,
                                                          partial, guard);
    AMFLS_LAUNCHED();
    reduce_block_kernel<<<grid_1d((long long)S * out_n), kThreads, 0, s>>>(partial, chunks, S,
                                                                           out_n, y, ldy, guard);
    AMFLS_LAUNCHED();
}

}  // namespace

void run_epilogue(const double* t, long long n, const Epilogue& ep, double* partials,
                  unsigned* counter, cudaStream_t s) {
    epilogue_kernel<<<grid_1d(n), kThreads, 0, s>>>(t, n, ep, partials, counter);
    AMFLS_LAUNCHED();
}

DenseOperator::DenseOperator(int rows, int cols, const double* d_values, bool column_major,
                             cudaStream_t stream)
    : rows_(rows), cols_(cols), a_(d_values), column_major_(column_major) {
    if (rows <= 0 || cols <= 0 || d_values == nullptr)
        throw std::invalid_argument("dense operator input is invalid");
    const int outer = column_major ? cols : rows;
    const int inner = column_major ? rows : cols;
    double* w = nullptr;  // model workspace, freed before returning
    double model[2] = {0.0, 0.0};
    try {
        AMFLS_CUDA(cudaMalloc(&scratch_, sizeof(double) * (6 * kMaxGridCap + 64)));
        AMFLS_CUDA(cudaMalloc(&counter_, sizeof(unsigned) * 8));
        AMFLS_CUDA(cudaMemsetAsync(counter_, 0, sizeof(unsigned) * 8, stream));
        AMFLS_CUDA(cudaMalloc(&tmp_, sizeof(double) * std::max(rows, cols)));
        // partial sums of the chunked products, sized once so that products
        // can be captured into CUDA graphs
        for (int tr = 0; tr < 2; ++tr) {  // both directions, up to 8 columns per pass
            const int on = tr ? cols : rows, inn = tr ? rows : cols;
            int bx = 0, ch = 0, ck = 0;
            block_chunks(column_major == (tr == 1), on, inn, bx, ch, ck);
            partial_cap_ = std::max(partial_cap_, 8LL * ch * on);
        }
        AMFLS_CUDA(cudaMalloc(&partials_,
                              sizeof(double) * std::max<long long>(1, partial_cap_)));
        // w: acc[5] | frob(inner) | model[2] | frob(outer) | partials (inner) | partials (outer)
        const int ig = grid_1d(inner), og = grid_1d(outer);
        AMFLS_CUDA(cudaMallocAsync(&w, sizeof(double) * (9 + ig + og), stream));
        AMFLS_CUDA(cudaMemsetAsync(w, 0, sizeof(double) * (9 + ig + og), stream));
        model_outer_kernel<<<og, kThreads, 0, stream>>>(a_, outer, inner, w, w + 9 + ig,
                                                        counter_ + 2, w + 8);
        AMFLS_LAUNCHED();
        model_inner_kernel<<<ig, kThreads, 0, stream>>>(a_, outer, inner, w, w + 9, counter_,
                                                        w + 5);
        AMFLS_LAUNCHED();
        // the reference's Frobenius bound sums column square sums: the inner
        // index for row-major storage, the outer one for column-major
        model_finish_kernel<<<1, 1, 0, stream>>>(w, column_major ? w + 8 : w + 5,
                                                 column_major ? 0 : 1, w + 6);
        AMFLS_LAUNCHED();
        AMFLS_CUDA(cudaMemcpyAsync(model, w + 6, sizeof(model), cudaMemcpyDeviceToHost,
                                   stream));
        AMFLS_CUDA(cudaStreamSynchronize(stream));
        double* used = w;
        w = nullptr;
        AMFLS_CUDA(cudaFreeAsync(used, stream));
    } catch (...) {  // e.g. out of device memory part way: free what was allocated
        if (w) cudaFreeAsync(w, stream);
        release();
        throw;
    }
    model_.norm_upper = model[0];
    model_.norm_lower = model[1];
    model_.apply_steps = 2LL * cols + 2LL;
    model_.transpose_steps = 2LL * rows + 2LL;
}

DenseOperator::~DenseOperator() { release(); }

void DenseOperator::release() noexcept {
    cudaFree(partials_);
    cudaFree(tmp_);
    cudaFree(scratch_);
    cudaFree(counter_);
}

void DenseOperator::product(bool transpose, const double* x, double* y, const int* guard,
                            cudaStream_t s) const {
    // y has length rows (apply) or cols (transpose).  The contiguous
    // dimension decides the kernel: row-major rows are contiguous (apply =
    // dot of rows); column-major columns are (transpose = dot of columns).
    const int out_n = transpose ? cols_ : rows_;
    const int in_n = transpose ? rows_ : cols_;
    const bool dot = column_major_ == transpose;
    const long long ld = column_major_ ? rows_ : cols_;
    launch_block<1>(dot, a_, ld, out_n, in_n, x, in_n, partials_, y, out_n, s, guard);
}

void DenseOperator::block_product(bool transpose, const double* x, int block_cols, double* y,
                                  cudaStream_t s) const {
    const int out_n = transpose ? cols_ : rows_;
    const int in_n = transpose ? rows_ : cols_;
    const bool dot = column_major_ == transpose;
    const long long ld = column_major_ ? rows_ : cols_;
    for (int c0 = 0; c0 < block_cols; c0 += 8) {
        const int sc = std::min(8, block_cols - c0);
        const double* xs = x + (long long)c0 * in_n;
        double* ys = y + (long long)c0 * out_n;
        switch (sc) {
            case 1: launch_block<1>(dot, a_, ld, out_n, in_n, xs, in_n, partials_, ys, out_n, s); break;
            case 2: launch_block<2>(dot, a_, ld, out_n, in_n, xs, in_n, partials_, ys, out_n, s); break;
            case 3: launch_block<3>(dot, a_, ld, out_n, in_n, xs, in_n, partials_, ys, out_n, s); break;
            case 4: launch_block<4>(dot, a_, ld, out_n, in_n, xs, in_n, partials_, ys, out_n, s); break;
            case 5: launch_block<5>(dot, a_, ld, out_n, in_n, xs, in_n, partials_, ys, out_n, s); break;
            case 6: launch_block<6>(dot, a_, ld, out_n, in_n, xs, in_n, partials_, ys, out_n, s); break;
            case 7: launch_block<7>(dot, a_, ld, out_n, in_n, xs, in_n, partials_, ys, out_n, s); break;
            default: launch_block<8>(dot, a_, ld, out_n, in_n, xs, in_n, partials_, ys, out_n, s); break;
        }
    }
}

void DenseOperator::apply(const double* x, int block_cols, double* y, cudaStream_t s) const {
    if (x == nullptr || y == nullptr || block_cols <= 0)
        throw std::invalid_argument("dense apply block is invalid");
    block_product(false, x, block_cols, y, s);
}

void DenseOperator::apply_transpose(const double* y, int block_cols, double* x,
                                    cudaStream_t s) const {
    if (x == nullptr || y == nullptr || block_cols <= 0)
        throw std::invalid_argument("dense transpose block is invalid");
    block_product(true, y, block_cols, x, s);
}

bool DenseOperator::product1(bool transpose, const double* x, const Epilogue& ep,
                             cudaStream_t s) const {
    product(transpose, x, tmp_, ep.guard, s);
    run_epilogue(tmp_, transpose ? cols_ : rows_, ep, ep.partials ? ep.partials : scratch_,
                 ep.counter ? ep.counter : counter_ + 1, s);
    return true;
}

void DenseOperator::apply_refined(const double* x_hi, const double* x_lo, double* y_hi,
                                  double* y_lo, int* finite, cudaStream_t s) const {
    if (!column_major_) {
        dd_dot_rows_kernel<<<grid_1d((long long)rows_ * 32), kThreads, 0, s>>>(
            a_, cols_, rows_, cols_, x_hi, x_lo, y_hi, y_lo, finite);
        AMFLS_LAUNCHED();
    } else {
        dd_sum_cols_kernel<<<grid_1d(rows_), kThreads, 0, s>>>(a_, rows_, rows_, cols_, x_hi,
                                                               x_lo, y_hi, y_lo, finite);
        AMFLS_LAUNCHED();
    }
}

void DenseOperator::apply_transpose_refined(const double* y_hi, const double* y_lo, double* x_hi,
                                            double* x_lo, int* finite, cudaStream_t s) const {
    if (column_major_) {
        dd_dot_rows_kernel<<<grid_1d((long long)cols_ * 32), kThreads, 0, s>>>(
            a_, rows_, cols_, rows_, y_hi, y_lo, x_hi, x_lo, finite);
        AMFLS_LAUNCHED();
    } else {
        dd_sum_cols_kernel<<<grid_1d(cols_), kThreads, 0, s>>>(a_, cols_, cols_, rows_, y_hi,
                                                               y_lo, x_hi, x_lo, finite);
        AMFLS_LAUNCHED();
    }
}

}  // namespace amfls_gpu
