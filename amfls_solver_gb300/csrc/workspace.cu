// Device block Golub-Kahan workspace (see workspace.hpp for the layout).
//
// One width-one level (krylov_workspace.cpp:589-831) is the kernel chain
//   begin        decide on the device whether the level runs (can_advance,
//                depth target); reset the step audit
//   A^T u        fused SpMV^T: r = A^T u - beta v_prev, ||A^T u||, ||r||
//   V^T r        c1, per-panel partials reduced by the last block per panel
//   r -= V c1    with ||r||; its last block takes the DGKS decision
//                (second pass only if ||r_after|| < sqrt(1/2) ||r_before||,
//                krylov_workspace.cpp:152-165) and, when no second pass is
//                needed, the rank decision against the cutoff
//                64 eps max(m,n,k,1) ||A^T u|| (krylov_workspace.cpp:63-80)
//   [V^T r, r -= V c2]   only when the device flag asks for it
//   normalise    v = r / ||r|| into V's new column and a contiguous copy
//   A v          fused SpMV: y = A v - ||r|| u, ||A v||, ||y||, u.y
//   left pass    y -= (u.y) u with ||y||, u.y, y.b; DGKS and rank decision,
//                T column (alpha = ||r|| + u.y, beta = ||y||), g = u'.b
//   [left pass]  second DGKS pass when flagged
//   normalise    u' = y / ||y||
// Every kernel reads the device flag `go` and does nothing once the level
// (or an earlier one) stopped, so a whole run of levels up to the next
// checkpoint is enqueued without a host round trip.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <vector>

#include "common.cuh"
#include "vector_ops.hpp"
#include "workspace.hpp"

namespace amfls_gpu {

void keep_pool_memory() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    AMFLS_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || done[dev]) return;
    cudaMemPool_t pool;
    AMFLS_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    unsigned long long threshold = ~0ULL;
    AMFLS_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold));
    done[dev] = true;
}

void stream_wait(cudaStream_t stream) {
    struct Event {
        cudaEvent_t e = nullptr;
        int device = -1;
        ~Event() {
            if (e) cudaEventDestroy(e);
        }
    };
    thread_local Event ev;
    int dev = 0;
    AMFLS_CUDA(cudaGetDevice(&dev));
    if (!ev.e || ev.device != dev) {
        if (ev.e) cudaEventDestroy(ev.e);
        ev.e = nullptr;
        AMFLS_CUDA(cudaEventCreateWithFlags(&ev.e, cudaEventBlockingSync | cudaEventDisableTiming));
        ev.device = dev;
    }
    AMFLS_CUDA(cudaEventRecord(ev.e, stream));
    AMFLS_CUDA(cudaEventSynchronize(ev.e));
}

namespace {

constexpr int kThreads = 256;
constexpr double kEps = 2.220446049250313e-16;
constexpr int kGemvTargetBlocks = 152 * 16;

enum Hook { kHookNone = 0, kHookRightPass1 = 1, kHookRightPass2 = 2 };

__device__ inline bool dfinite(double v) { return isfinite(v); }

// Rank decision for the width-one right residual (krylov_workspace.cpp:197-310,
// scalar branch) after its final projection pass.
__device__ void decide_right(DevState* st, int m, int n) {
    const double scale = st->right_scale;
    const double after = st->norm_after;
    const int k = st->k;
    const int dim = max(max(1, m), max(n, max(k, 1)));
    const double cutoff = (scale >= 0.0 && dfinite(scale)) ? 64.0 * kEps * dim * scale
                                                           : __builtin_huge_val();
    const bool finite = dfinite(scale) && dfinite(after) && !st->coeff_nonfinite;
    const int max_rank = min(1, st->basis_limit - k);  // combined width is one
    StepAudit& a = st->audit;
    int rank = 0;
    double discarded = after, tracked = 0.0;
    bool positive = false;
    if (!finite) {
        discarded = __builtin_huge_val();
        tracked = __builtin_huge_val();  // tracked prefix = active width = 1
    } else if (max_rank == 0) {
        tracked = after;
    } else if (after > cutoff) {
        rank = 1;
        discarded = 0.0;
    } else if (after > 0.0) {
        positive = true;
        tracked = after;
    }
    a.retained_right_width = rank;
    a.right_rank_cutoff = cutoff;
    a.right_discarded_residual_norm = discarded;
    a.right_active_discarded_residual_norm = tracked;
    a.right_positive_finite_below_cutoff = positive;
    a.right_nonfinite_residual = !finite;
    a.right_rank_loss = rank < max_rank;
    a.right_basis_cap_truncation = max_rank < 1;
    const bool truncated = a.right_rank_loss && positive && tracked > 0.0;
    if (truncated || !finite) st->reliable = 0;
    st->right_rank = rank;
    if (rank == 0) {
        st->left_width = 0;
        st->active_first = st->rows_t;
        st->prev_right_first = k;
        st->prev_right_width = 0;
        st->coupling = 0.0;
        st->level_ok = 0;
        st->go = 0;
        return;
    }
    st->right_factor = after;
    st->inv_right = 1.0 / after;
    st->search_a_calls += 1;
    st->search_a_columns += 1;
}

// Rank decision of the left residual and the T / g update
// (krylov_workspace.cpp:736-830).
__device__ void decide_left(DevState* st, int m, int n, double* alpha, double* beta, double* g) {
    const double scale = st->left_scale;
    const double after = st->left_norm;
    const int dim = max(max(1, m), n);
    const double cutoff = (scale >= 0.0 && dfinite(scale)) ? 64.0 * kEps * dim * scale
                                                           : __builtin_huge_val();
    const bool finite = dfinite(scale) && dfinite(after) && dfinite(st->left_coeff);
    const int old_left = st->rows_t;
    const int max_rank = min(min(1, m - old_left), st->basis_limit + 1 - old_left);
    StepAudit& a = st->audit;
    int rank = 0;
    double discarded = after;
    bool positive = false;
    if (!finite) {
        discarded = __builtin_huge_val();
    } else if (max_rank <= 0) {
        // nothing retained, nothing tracked
    } else if (after > cutoff) {
        rank = 1;
        discarded = 0.0;
    } else if (after > 0.0) {
        positive = true;
    }
    a.retained_next_left_width = rank;
    a.left_rank_cutoff = cutoff;
    a.left_discarded_residual_norm = discarded;
    a.left_positive_finite_below_cutoff = positive;
    a.left_nonfinite_residual = !finite;
    a.left_rank_loss = rank < max_rank;
    a.left_basis_cap_truncation = max_rank < 1;
    const bool truncated = (a.left_rank_loss && positive);
    if (truncated || !finite) st->reliable = 0;
    if (!finite) {
        st->level_ok = 0;
        st->go = 0;
        return;
    }
    const int k_old = st->k;
    alpha[k_old] = st->right_factor + st->left_coeff;  // active coupling + coefficient
    beta[k_old] = rank ? after : 0.0;
    if (rank) {
        st->inv_left = 1.0 / after;
        g[old_left] = st->b_dot * st->inv_left;
    }
    st->left_rank = rank;
    st->k = k_old + 1;
    st->active_first = old_left;
    st->rows_t = old_left + rank;
    st->left_width = rank;
    st->prev_right_first = k_old;
    st->prev_right_width = 1;
    st->coupling = after;
    st->depth += 1;
    st->level_ok = 1;
    st->levels_run += 1;
    a.basis_rank_after = k_old + 1;
    if (!rank) st->go = 0;  // nothing to normalise; the process stops here
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool can_advance_dev(const DevState* st) {
    return st->reliable && (st->left_width + st->pending > 0) && st->k < st->basis_limit &&
           st->depth < st->target_depth;
}

__global__ void set_target_kernel(DevState* st, int target_depth, int iterations) {
    if (threadIdx.x != 0) return;
    st->target_depth = target_depth;
    st->iterations_left = iterations;
}

__global__ void level_begin_kernel(DevState* st) {
    if (threadIdx.x != 0) return;
    st->body_runs += 1;
    const bool go = can_advance_dev(st) && st->iterations_left > 0;
    st->iterations_left -= 1;
    st->go = go ? 1 : 0;
    if (!go) return;
    st->sub_col = st->prev_right_width > 0 ? st->prev_right_first : 0;
    st->t_mark = global_ns();
    StepAudit a;
    memset(&a, 0, sizeof(a));
    a.left_input_width = st->left_width + st->pending;
    a.basis_rank_before = st->k;
    a.basis_rank_after = st->k;
    st->audit = a;
    st->coupling_eff = (st->prev_right_width > 0 && st->left_width > 0) ? st->coupling : 0.0;
    st->second_pass = 0;
    st->right_rank = 0;
    st->left_rank = 0;
    st->coeff_nonfinite = 0;
    st->level_ok = 0;
    st->search_at_calls += 1;
    st->search_at_columns += st->left_width + st->pending;
}

// after A^T u: scale and norm_before from the fused reduction
__global__ void right_scales_kernel(DevState* st, const RedResult* red, int m, int n) {
    if (threadIdx.x != 0 || !st->go) return;
    st->at_ns += global_ns() - st->t_mark;
    const bool no_projection = st->k == 0;
    st->right_scale = red->nonfinite ? __builtin_nan("") : sqrt(red->sq_t);
    st->norm_before = red->nonfinite ? __builtin_nan("") : sqrt(red->sq_out);
    if (no_projection) {  // empty basis: no pass, the norm is the block's norm
        st->norm_after = st->norm_before;
        decide_right(st, m, n);
    }
}

// c = V^T r, masked to k columns.  grid (panels, chunks); partials [P][C][32].
__global__ void __launch_bounds__(kThreads)
vt_r_kernel(double* const* __restrict__ panels, int n, int chunk_rows,
            const double* __restrict__ r, double* __restrict__ c, double* partials,
            unsigned* panel_tickets, DevState* st, int pass) {
    if (!st->go || (pass == 2 && !st->second_pass)) return;
    const int k = st->k;  // k == 0: no projection (decided in right_scales_kernel)
    const int p = blockIdx.x, chunk = blockIdx.y, nchunks = gridDim.y;
    if (p * 32 >= k) return;  // panel beyond the current basis
    const double* __restrict__ vp = panels[p];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int q = lane & 3, rsub = lane >> 2;
    const long long row0 = (long long)chunk * chunk_rows;
    const long long row1 = min((long long)n, row0 + chunk_rows);
    double acc[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[i] = 0.0;
    for (long long base = row0 + warp * 8; base < row1; base += 64) {
        const long long row = base + rsub;
        if (row < row1) {
            const double2* src = reinterpret_cast<const double2*>(vp + row * 32 + q * 8);
            const double2 a0 = __ldg(src), a1 = __ldg(src + 1), a2 = __ldg(src + 2),
                          a3 = __ldg(src + 3);
            const double rv = __ldg(r + row);
            acc[0] = fma(a0.x, rv, acc[0]);
            acc[1] = fma(a0.y, rv, acc[1]);
            acc[2] = fma(a1.x, rv, acc[2]);
            acc[3] = fma(a1.y, rv, acc[3]);
            acc[4] = fma(a2.x, rv, acc[4]);
            acc[5] = fma(a2.y, rv, acc[5]);
            acc[6] = fma(a3.x, rv, acc[6]);
            acc[7] = fma(a3.y, rv, acc[7]);
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], 4);
        acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], 8);
        acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], 16);
    }
    __shared__ double sm[8][32];
    __shared__ bool last;
    if (lane < 4) {
#pragma unroll
        for (int i = 0; i < 8; ++i) sm[warp][lane * 8 + i] = acc[i];
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < 8; ++w) s += sm[w][threadIdx.x];
        partials[((long long)p * nchunks + chunk) * 32 + threadIdx.x] = s;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned t = atomicAdd(&panel_tickets[p], 1u);
        last = (t == (unsigned)nchunks - 1);
        if (last) panel_tickets[p] = 0u;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (threadIdx.x < 32) {
        double s = 0.0;
        for (int ch = 0; ch < nchunks; ++ch)
            s += partials[((long long)p * nchunks + ch) * 32 + threadIdx.x];
        const int col = p * 32 + threadIdx.x;
        if (col < k) {
            c[col] = s;
            if (!isfinite(s)) st->coeff_nonfinite = 1;
        }
    }
}

// out = r - V c (subtract) or out = V c; 32 rows per block, warps split the
// panels.  Sum of squares of out reduced by the last block, then `hook`.
__global__ void __launch_bounds__(kThreads)
v_c_kernel(double* const* __restrict__ panels, int n, int k_arg, const double* __restrict__ c,
           const double* r_in, double* out, int subtract, double* partials, unsigned* ticket,
           DevState* st, int hook, int m_rows, int guarded, int pass) {
    if (guarded && (!st->go || (pass == 2 && !st->second_pass) || st->k == 0)) return;
    const int k = k_arg >= 0 ? k_arg : st->k;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int q = lane & 3, rsub = lane >> 2;
    const long long row0 = (long long)blockIdx.x * 32;
    const int P = (k + 31) / 32;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int p = warp; p < P; p += 8) {
        const double* __restrict__ vp = panels[p];
        double cv[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int col = p * 32 + q * 8 + i;
            cv[i] = col < k ? c[col] : 0.0;
        }
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const long long row = row0 + s * 8 + rsub;
            if (row < n) {
                const double2* src = reinterpret_cast<const double2*>(vp + row * 32 + q * 8);
                const double2 a0 = __ldg(src), a1 = __ldg(src + 1), a2 = __ldg(src + 2),
                              a3 = __ldg(src + 3);
                double t = acc[s];
                t = fma(a0.x, cv[0], t);
                t = fma(a0.y, cv[1], t);
                t = fma(a1.x, cv[2], t);
                t = fma(a1.y, cv[3], t);
                t = fma(a2.x, cv[4], t);
                t = fma(a2.y, cv[5], t);
                t = fma(a3.x, cv[6], t);
                t = fma(a3.y, cv[7], t);
                acc[s] = t;
            }
        }
    }
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        acc[s] += __shfl_xor_sync(0xffffffffu, acc[s], 1);
        acc[s] += __shfl_xor_sync(0xffffffffu, acc[s], 2);
    }
    __shared__ double sm[8][32];
    __shared__ double red[32];
    if (q == 0) {
#pragma unroll
        for (int s = 0; s < 4; ++s) sm[warp][s * 8 + rsub] = acc[s];
    }
    __syncthreads();
    double sq = 0.0;
    if (threadIdx.x < 32) {
        const long long row = row0 + threadIdx.x;
        double y = 0.0;
#pragma unroll
        for (int w = 0; w < 8; ++w) y += sm[w][threadIdx.x];
        if (row < n) {
            const double o = subtract ? r_in[row] - y : y;
            out[row] = o;
            sq = o * o;
        }
    }
    if (hook == kHookNone) return;
    const double bs = block_sum(sq, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = bs;
    if (arrive_last(ticket, gridDim.x)) {
        double a = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) a += partials[b];
        a = block_sum(a, red);
        if (threadIdx.x == 0) {
            st->norm_after = sqrt(a);
            if (hook == kHookRightPass1) {
                const double before = st->norm_before, after = st->norm_after;
                const bool again = isfinite(before) && isfinite(after) &&
                                   after < 0.70710678118654757 * before;
                st->second_pass = again ? 1 : 0;
                if (!again) decide_right(st, m_rows, n);
            } else {
                decide_right(st, m_rows, n);
            }
        }
    }
}

__global__ void normalize_right_kernel(const double* r, int n, double* const* panels,
                                       double* vnew, DevState* st) {
    if (!st->go || !st->right_rank) return;
    const double inv = st->inv_right;
    const int k = st->k;
    double* vcol = panels[k >> 5] + (k & 31);
    if (blockIdx.x == 0 && threadIdx.x == 0) st->t_mark = global_ns();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = r[i] * inv;
        vcol[i * 32] = v;
        vnew[i] = v;
    }
}

// Left DGKS pass: y -= c u with reductions ||y||^2, u.y, y.b.
__global__ void __launch_bounds__(kThreads)
left_pass_kernel(double* y, const double* u, const double* b, int m, const RedResult* spmv_red,
                 double* partials, unsigned* ticket, DevState* st, int pass, int n_cols,
                 double* alpha, double* beta, double* g) {
    if (!st->go || (pass == 2 && !st->second_pass)) return;
    if (pass == 1 && blockIdx.x == 0 && threadIdx.x == 0) st->a_ns += global_ns() - st->t_mark;
    const double c = pass == 1 ? spmv_red->dot : st->pass_coeff;
    double sq = 0.0, du = 0.0, db = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x) {
        const double ui = u[i];
        const double v = y[i] - c * ui;
        y[i] = v;
        sq = fma(v, v, sq);
        du = fma(v, ui, du);
        db = fma(v, b[i], db);
    }
    __shared__ double red[32];
    const double s0 = block_sum(sq, red);
    const double s1 = block_sum(du, red);
    const double s2 = block_sum(db, red);
    if (threadIdx.x == 0) {
        partials[3 * blockIdx.x] = s0;
        partials[3 * blockIdx.x + 1] = s1;
        partials[3 * blockIdx.x + 2] = s2;
    }
    if (!arrive_last(ticket, gridDim.x)) return;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (unsigned blk = threadIdx.x; blk < gridDim.x; blk += blockDim.x) {
        a0 += partials[3 * blk];
        a1 += partials[3 * blk + 1];
        a2 += partials[3 * blk + 2];
    }
    a0 = block_sum(a0, red);
    a1 = block_sum(a1, red);
    a2 = block_sum(a2, red);
    if (threadIdx.x != 0) return;
    const double after = sqrt(a0);
    st->b_dot = a2;
    if (pass == 1) {
        st->left_scale = spmv_red->nonfinite ? __builtin_nan("") : sqrt(spmv_red->sq_t);
        st->norm_before = spmv_red->nonfinite ? __builtin_nan("") : sqrt(spmv_red->sq_out);
        st->left_coeff = c;
        st->left_norm = after;
        st->pass_coeff = a1;
        const double before = st->norm_before;
        const bool again = isfinite(before) && isfinite(after) &&
                           after < 0.70710678118654757 * before;
        st->second_pass = again ? 1 : 0;
        if (!again) decide_left(st, m, n_cols, alpha, beta, g);
    } else {
        st->left_coeff += c;
        st->left_norm = after;
        decide_left(st, m, n_cols, alpha, beta, g);
    }
}

__global__ void normalize_left_kernel(const double* y, double* u, int m, const DevState* st) {
    if (!st->go || !st->left_rank) return;
    const double inv = st->inv_left;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x)
        u[i] = y[i] * inv;
}

// Loop control of the captured level: continue while the next level can run.
__global__ void level_end_kernel(DevState* st, cudaGraphConditionalHandle handle) {
    if (threadIdx.x != 0) return;
    const bool more = st->go && can_advance_dev(st) && st->iterations_left > 0;
    cudaGraphSetConditional(handle, more ? 1u : 0u);
}

__global__ void scale_copy_kernel(const double* src, double* dst, long long n, double s) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i] * s;
}

// Incremental Givens QR of the lower-bidiagonal T, with sqrt(lambda) I rows
// folded in by one extra rotation per column (the damped LSQR recurrence of
// Paige and Saunders), then back substitution for y.  qr = [rho | theta |
// phi | y] (4 x cap); state = [c, s, rhobar, phibar, processed, flags].
__global__ void projected_solve_kernel(const double* alpha, const double* beta, const double* g,
                                       int k, int rows_t, double lambda, double* qr, int cap,
                                       double* state, double rcond) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double* rho = qr;
    double* theta = qr + cap;
    double* phi = qr + 2 * (long long)cap;
    double* y = qr + 3 * (long long)cap;
    double c = state[0], s = state[1], rhobar = state[2], phibar = state[3];
    int done = (int)state[4];
    const double root = sqrt(lambda);
    for (int j = done; j < k; ++j) {
        if (j == 0) {
            rhobar = alpha[0];
            phibar = g[0];
        } else {
            // the rotation of column j-1 acting on rows (j-1, j) meets column j
            theta[j] = s * alpha[j];
            rhobar = c * alpha[j];
        }
        if (lambda > 0.0) {
            const double r = hypot(rhobar, root);
            const double c1 = rhobar / r;
            phibar = c1 * phibar;
            rhobar = r;
        }
        if (j + 1 < rows_t) {
            // rotate rows (j, j+1): [phi_j; phibar_j+1] = G [phibar_j; g_j+1].
            // g = U^T b is not a multiple of e_1 once U loses orthogonality,
            // so g_j+1 enters both rotated entries.
            const double b = beta[j];
            const double r = hypot(rhobar, b);
            c = rhobar / r;
            s = b / r;
            rho[j] = r;
            phi[j] = c * phibar + s * g[j + 1];
            phibar = -s * phibar + c * g[j + 1];
        } else {
            rho[j] = rhobar;
            phi[j] = phibar;
            c = 1.0;
            s = 0.0;
        }
    }
    state[0] = c;
    state[1] = s;
    state[2] = rhobar;
    state[3] = phibar;
    state[4] = (double)k;
    // back substitution R y = phi
    int flags = 0;
    double ynext = 0.0;
    for (int j = k - 1; j >= 0; --j) {
        double num = phi[j];
        if (j + 1 < k) num -= theta[j + 1] * ynext;
        if (!(rho[j] != 0.0)) flags |= 1;
        ynext = num / rho[j];
        y[j] = ynext;
    }
    // LINPACK-style estimate of ||R^{-1}|| for the rank test the reference
    // makes with dgelsy (rcond = min(1/2, 64 eps max(rows, cols))): solve
    // R^T z = e with e_j = +-1 chosen to grow |z|, then R w = z.
    if (lambda == 0.0 && k > 0) {
        double rmax = 0.0, zprev = 0.0, znorm2 = 0.0;
        for (int j = 0; j < k; ++j) {
            const double off = j > 0 ? theta[j] : 0.0;
            rmax = fmax(rmax, fabs(rho[j]) + fabs(off));
            const double t = -off * zprev;
            const double e = t >= 0.0 ? 1.0 : -1.0;
            const double z = (e + t) / rho[j];
            zprev = z;
            znorm2 += z * z;
        }
        // ||R^{-1}|| >= ||z|| / ||e|| with ||e|| = sqrt(k)
        const double cond = rmax * sqrt(znorm2 / (double)k);
        if (!(cond * rcond < 1.0)) flags |= 2;
    }
    state[5] = (double)flags;
}

}  // namespace

// ------------------------------------------------------------ panels ----

PanelStore::PanelStore(int n, int max_panels, cudaStream_t stream)
    : n_(n), stream_(stream), table_cap_(std::max(1, max_panels)) {
    // fixed-capacity device table: its address never changes, so captured
    // kernels may keep it
    stream_alloc(&table_, sizeof(double*) * table_cap_, stream_);
    host_.reserve(table_cap_);
}

PanelStore::~PanelStore() {
    for (double* p : host_) stream_free(p, stream_);
    stream_free(table_, stream_);
}

void PanelStore::ensure_columns(int cols) {
    const int need = (cols + 31) / 32;
    if (need <= panels()) return;
    if (need > table_cap_) throw std::length_error("basis exceeds the panel table capacity");
    const int first = panels();
    while (panels() < need) {
        double* p = nullptr;
        stream_alloc(&p, sizeof(double) * 32 * static_cast<size_t>(n_), stream_);
        AMFLS_CUDA(cudaMemsetAsync(p, 0, sizeof(double) * 32 * static_cast<size_t>(n_), stream_));
        host_.push_back(p);
    }
    // host_ never reallocates (reserved to table_cap_), so the async copy
    // reads stable memory
    AMFLS_CUDA(cudaMemcpyAsync(table_ + first, host_.data() + first,
                               sizeof(double*) * (need - first), cudaMemcpyHostToDevice, stream_));
}

// --------------------------------------------------------- workspace ----

Workspace::Workspace(const DeviceOperator& op, const double* d_b, double regularization,
                     int maximum_basis_size, cudaStream_t stream, bool time_operators,
                     bool use_graphs)
    : op_(op), stream_(stream), m_(op.rows()), n_(op.cols()), reg_(regularization),
      time_ops_(time_operators), use_graphs_(use_graphs), b_(d_b) {
    if (m_ <= 0 || n_ <= 0) throw std::invalid_argument("block Golub-Kahan operator dimensions must be positive");
    if (d_b == nullptr) throw std::invalid_argument("block Golub-Kahan right-hand side must not be null");
    if (!std::isfinite(regularization) || regularization < 0.0)
        throw std::invalid_argument("block Golub-Kahan regularization must be finite and nonnegative");
    if (maximum_basis_size < 0) throw std::invalid_argument("block Golub-Kahan basis limit must be nonnegative");
    keep_pool_memory();
    const int mn = std::min(m_, n_);
    basis_limit_ = maximum_basis_size > 0 ? std::min(maximum_basis_size, mn) : mn;
    stream_alloc(&dstate_, sizeof(DevState), stream_);
    stream_alloc(&red_, sizeof(RedResult) * 4, stream_);
    // scratch: V^T r partials ((target blocks + panels) x 32), then the
    // per-block norm partials of the V c sweep (n/32 + slack)
    const long long max_panels = basis_limit_ / 32 + 2;
    vc_partials_offset_ = (kGemvTargetBlocks + max_panels) * 32 + 6 * 1216;
    const long long pcount = vc_partials_offset_ + (n_ + 31) / 32 + 1024;
    stream_alloc(&partials_, sizeof(double) * pcount, stream_);
    const long long ncounters = 64 + max_panels + 64;
    stream_alloc(&counter_, sizeof(unsigned) * ncounters, stream_);
    AMFLS_CUDA(cudaMemsetAsync(counter_, 0, sizeof(unsigned) * ncounters, stream_));
    stream_alloc(&R_, sizeof(double) * n_, stream_);
    stream_alloc(&vnew_, sizeof(double) * n_, stream_);
    stream_alloc(&Y_, sizeof(double) * m_, stream_);
    ucap_ = 1;
    stream_alloc(&U_, sizeof(double) * m_ * ucap_, stream_);
    V_ = std::make_unique<PanelStore>(n_, static_cast<int>(max_panels), stream_);
    V_->ensure_columns(1);  // panel 0 exists (zeroed) before any level runs
    AMFLS_CUDA(cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking));
    std::memset(&host_, 0, sizeof(host_));
    host_.reliable = 1;
    host_.basis_limit = basis_limit_;
    AMFLS_CUDA(cudaMemcpyAsync(dstate_, &host_, sizeof(DevState), cudaMemcpyHostToDevice, stream_));
    stream_wait(stream_);
}

Workspace::~Workspace() {
    cudaStreamSynchronize(stream_);
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (graph_) cudaGraphDestroy(graph_);
    if (capture_stream_) cudaStreamDestroy(capture_stream_);
    stream_free(dstate_, stream_);
    stream_free(red_, stream_);
    stream_free(partials_, stream_);
    stream_free(counter_, stream_);
    stream_free(R_, stream_);
    stream_free(vnew_, stream_);
    stream_free(Y_, stream_);
    stream_free(U_, stream_);
    stream_free(P_, stream_);
    stream_free(c1_, stream_);
    stream_free(c2_, stream_);
    stream_free(alpha_, stream_);
    stream_free(beta_, stream_);
    stream_free(g_, stream_);
    stream_free(qr_, stream_);
    stream_free(qr_state_, stream_);
    stream_free(U2_, stream_);
    stream_free(BR_, stream_);
    stream_free(BL_, stream_);
    stream_free(BQ_, stream_);
    stream_free(BT_, stream_);
    stream_free(small_, stream_);
    stream_free(coefs_, stream_);
    stream_free(bpart_, stream_);
    stream_free(tsqr_, stream_);
    stream_free(dflags_, stream_);
    stream_free(dnorm_, stream_);
    stream_free(d_meta_, stream_);
    stream_free(d_vals_, stream_);
    stream_free(d_pstate_, stream_);
    stream_free(d_carry_, stream_);
    stream_free(d_pwork_, stream_);
    stream_free(d_y_, stream_);
    for (cudaEvent_t e : ev_)
        if (e) cudaEventDestroy(e);
}

void Workspace::ensure_t_capacity(int cols) {
    if (cols + 2 <= tcap_ && cols <= ccap_) return;
    int cap = std::max(1024, tcap_);
    while (cap < cols + 2) cap *= 2;
    stream_wait(stream_);
    auto grow = [&](double*& p, size_t old_count, size_t new_count) {
        double* q = nullptr;
        stream_alloc(&q, sizeof(double) * new_count, stream_);
        AMFLS_CUDA(cudaMemsetAsync(q, 0, sizeof(double) * new_count, stream_));
        if (p) {
            AMFLS_CUDA(cudaMemcpyAsync(q, p, sizeof(double) * old_count, cudaMemcpyDeviceToDevice,
                                       stream_));
            stream_wait(stream_);
            stream_free(p, stream_);
        }
        p = q;
    };
    const size_t old = tcap_;
    grow(alpha_, old, cap);
    grow(beta_, old, cap);
    grow(g_, old, cap);
    grow(c1_, old, cap);
    grow(c2_, old, cap);
    // the QR arrays are laid out by capacity: rebuild them from scratch
    stream_free(qr_, stream_);
    qr_ = nullptr;
    stream_alloc(&qr_, sizeof(double) * 4 * cap, stream_);
    if (!qr_state_) stream_alloc(&qr_state_, sizeof(double) * 8, stream_);
    AMFLS_CUDA(cudaMemsetAsync(qr_state_, 0, sizeof(double) * 8, stream_));
    tcap_ = cap;
    ccap_ = cap;
    invalidate_graph();  // captured kernels hold the old buffer addresses
}

void Workspace::invalidate_graph() {
    if (graph_exec_) {
        stream_wait(stream_);
        cudaGraphExecDestroy(graph_exec_);
        graph_exec_ = nullptr;
    }
    if (graph_) {
        cudaGraphDestroy(graph_);
        graph_ = nullptr;
    }
    graph_pcap_ = 0;
}

void Workspace::initialize(const double* d_aux, int aux_cols) {
    if (initialized_) throw std::logic_error("block Golub-Kahan workspace is already initialized");
    initialized_ = true;
    // ||b|| (scaled two-pass, stands in for dnrm2)
    NormResult* nr = nullptr;
    AMFLS_CUDA(cudaMallocAsync(&nr, sizeof(NormResult), stream_));
    VectorSet set{};
    set.v[0] = b_;
    set.n[0] = m_;
    set.count = 1;
    norm_passes(set, nr, partials_, counter_ + 1, stream_);
    NormResult h{};
    AMFLS_CUDA(cudaMemcpyAsync(&h, nr, sizeof(NormResult), cudaMemcpyDeviceToHost, stream_));
    stream_wait(stream_);
    AMFLS_CUDA(cudaFreeAsync(nr, stream_));
    if (h.nonfinite[0]) throw std::invalid_argument("block Golub-Kahan right-hand side must be finite");
    b_norm_ = euclid_from(h, 0);
    ensure_t_capacity(64);
    if (std::isfinite(b_norm_) && b_norm_ > 0.0 && basis_limit_ > 0) {
        const double inv = 1.0 / b_norm_;
        scale_copy_kernel<<<std::max<long long>(1, std::min<long long>(1216, (m_ + 255) / 256)), 256, 0,
                            stream_>>>(b_, U_, m_, inv);
        AMFLS_LAUNCHED();
        AMFLS_CUDA(cudaMemcpyAsync(g_, &b_norm_, sizeof(double), cudaMemcpyHostToDevice, stream_));
        host_.left_width = 1;
        host_.rows_t = 1;
        host_.active_first = 0;
    }
    std::memset(&host_.audit, 0, sizeof(host_.audit));
    AMFLS_CUDA(cudaMemcpyAsync(dstate_, &host_, sizeof(DevState), cudaMemcpyHostToDevice, stream_));
    stream_wait(stream_);
    if (b_norm_ > 0.0 && aux_cols > 0) append_left_seed(d_aux, aux_cols);
}

// The kernels of one width-one level.  Every per-level value (k, the
// previous right column, the depth target) is read from DevState, so the
// same launches serve every level and can be captured once.
void Workspace::enqueue_level_kernels(cudaStream_t s, int pcap) {
    level_begin_kernel<<<1, 32, 0, s>>>(dstate_);
    AMFLS_LAUNCHED();
    // A^T u - beta v_prev
    Epilogue ep;
    ep.out = R_;
    ep.sub_table = V_->device_table();
    ep.sub_col = &dstate_->sub_col;
    ep.coef = &dstate_->coupling_eff;
    ep.red = &red_[0];
    ep.guard = &dstate_->go;
    ep.partials = partials_;
    ep.counter = counter_ + 2;
    if (!op_.product1(true, U_, ep, s)) throw std::runtime_error("operator has no fused device product");
    right_scales_kernel<<<1, 32, 0, s>>>(dstate_, &red_[0], m_, n_);
    AMFLS_LAUNCHED();
    const int max_chunks = (int)std::max<long long>(1, (n_ + 255) / 256);
    const int chunks = std::max(1, std::min(max_chunks, (kGemvTargetBlocks + pcap - 1) / pcap));
    const int chunk_rows = (int)(((long long)n_ + chunks - 1) / chunks);
    const dim3 tgrid(pcap, chunks);
    const int ngrid = (int)((n_ + 31) / 32);
    for (int pass = 1; pass <= 2; ++pass) {
        double* c = pass == 1 ? c1_ : c2_;
        vt_r_kernel<<<tgrid, kThreads, 0, s>>>(V_->device_table(), n_, chunk_rows, R_, c, partials_,
                                               counter_ + 64, dstate_, pass);
        AMFLS_LAUNCHED();
        v_c_kernel<<<ngrid, kThreads, 0, s>>>(
            V_->device_table(), n_, -1, c, R_, R_, 1, partials_ + vc_partials_offset_, counter_ + 3,
            dstate_, pass == 1 ? kHookRightPass1 : kHookRightPass2, m_, 1, pass);
        AMFLS_LAUNCHED();
    }
    normalize_right_kernel<<<(int)std::min<long long>(1216, (n_ + 255) / 256), 256, 0, s>>>(
        R_, n_, V_->device_table(), vnew_, dstate_);
    AMFLS_LAUNCHED();
    // y = A v - ||r|| u, with ||A v||, ||y||, u.y
    Epilogue el;
    el.out = Y_;
    el.sub = U_;
    el.sub_stride = 1;
    el.coef = &dstate_->right_factor;
    el.dot_vec = U_;
    el.red = &red_[1];
    el.guard = &dstate_->go;
    el.partials = partials_;
    el.counter = counter_ + 2;
    op_.product1(false, vnew_, el, s);
    const int lgrid = (int)std::max<long long>(1, std::min<long long>(1216, (m_ + 1023) / 1024));
    for (int pass = 1; pass <= 2; ++pass) {
        left_pass_kernel<<<lgrid, kThreads, 0, s>>>(Y_, U_, b_, m_, &red_[1], partials_,
                                                    counter_ + 4, dstate_, pass, n_, alpha_, beta_,
                                                    g_);
        AMFLS_LAUNCHED();
    }
    normalize_left_kernel<<<(int)std::min<long long>(1216, (m_ + 255) / 256), 256, 0, s>>>(
        Y_, U_, m_, dstate_);
    AMFLS_LAUNCHED();
}

void Workspace::build_graph(int pcap) {
    invalidate_graph();
    AMFLS_CUDA(cudaGraphCreate(&graph_, 0));
    cudaGraphConditionalHandle handle;
    AMFLS_CUDA(cudaGraphConditionalHandleCreate(&handle, graph_, 1, cudaGraphCondAssignDefault));
    // the params union has no default constructor: build it in zeroed storage
    alignas(cudaGraphNodeParams) unsigned char storage[sizeof(cudaGraphNodeParams)] = {};
    auto* params = reinterpret_cast<cudaGraphNodeParams*>(storage);
    params->type = cudaGraphNodeTypeConditional;
    params->conditional.handle = handle;
    params->conditional.type = cudaGraphCondTypeWhile;
    params->conditional.size = 1;
    cudaGraphNode_t node;
    AMFLS_CUDA(cudaGraphAddNode(&node, graph_, nullptr, nullptr, 0, params));
    cudaGraph_t body = params->conditional.phGraph_out[0];
    AMFLS_CUDA(cudaStreamBeginCaptureToGraph(capture_stream_, body, nullptr, nullptr, 0,
                                             cudaStreamCaptureModeRelaxed));
    const long long launches_before = launch_count();
    try {
        enqueue_level_kernels(capture_stream_, pcap);
        level_end_kernel<<<1, 32, 0, capture_stream_>>>(dstate_, handle);
        AMFLS_LAUNCHED();
    } catch (...) {
        cudaGraph_t dummy;
        cudaStreamEndCapture(capture_stream_, &dummy);
        throw;
    }
    // captured launches run once per loop iteration, counted from body_runs
    body_kernels_ = launch_count() - launches_before;
    launch_count() = launches_before;
    cudaGraph_t captured;
    AMFLS_CUDA(cudaStreamEndCapture(capture_stream_, &captured));
    AMFLS_CUDA(cudaGraphInstantiate(&graph_exec_, graph_, 0));
    graph_pcap_ = pcap;
}

void Workspace::advance_to(int target_depth) {
    if (!initialized_) throw std::logic_error("block Golub-Kahan workspace is not initialized");
    if (block_mode_) {
        while (can_advance() && host_.depth < target_depth) {
            if (!block_level()) break;
        }
        return;
    }
    int levels = target_depth - host_.depth;
    levels = std::min(levels, basis_limit_ - host_.k);
    if (levels <= 0 || !can_advance()) return;
    // all allocations for the run happen before the launch, so the device
    // runs the whole interval without the host
    ensure_t_capacity(host_.k + levels + 2);
    V_->ensure_columns(host_.k + levels + 1);
    const int pneed = (host_.k + levels + 31) / 32;
    int pcap = 4;
    while (pcap < pneed) pcap *= 2;
    set_target_kernel<<<1, 32, 0, stream_>>>(dstate_, target_depth, levels);
    AMFLS_LAUNCHED();
    if (!use_graphs_) {  // same kernels, launched one by one
        for (int i = 0; i < levels; ++i) enqueue_level_kernels(stream_, pcap);
        return;
    }
    if (!graph_exec_ || pcap > graph_pcap_) build_graph(pcap);
    AMFLS_CUDA(cudaGraphLaunch(graph_exec_, stream_));
    ++graph_launches_;
}

bool Workspace::advance_level() {
    if (!initialized_) throw std::logic_error("block Golub-Kahan workspace is not initialized");
    if (block_mode_) return block_level();
    const int before = host_.depth;
    advance_to(host_.depth + 1);
    sync();
    return host_.depth > before && host_.level_ok;
}

void Workspace::sync() {
    AMFLS_CUDA(cudaMemcpyAsync(&host_, dstate_, sizeof(DevState), cudaMemcpyDeviceToHost, stream_));
    stream_wait(stream_);
    if (use_graphs_) {  // kernels the device ran inside graph-launched intervals
        launch_count() += body_kernels_ * (host_.body_runs - counted_body_runs_);
    }
    counted_body_runs_ = host_.body_runs;
}

void Workspace::take_operator_seconds(double& a_seconds, double& at_seconds) {
    a_seconds = static_cast<double>(host_.a_ns - seen_a_ns_) * 1e-9;
    at_seconds = static_cast<double>(host_.at_ns - seen_at_ns_) * 1e-9;
    seen_a_ns_ = host_.a_ns;
    seen_at_ns_ = host_.at_ns;
}

void Workspace::solve_projected(double* d_x) {
    const int k = host_.k;
    projected_flags_ = 0;
    if (k == 0) {
        AMFLS_CUDA(cudaMemsetAsync(d_x, 0, sizeof(double) * n_, stream_));
        return;
    }
    if (block_mode_) {
        int flags = 0;
        const double* y = block_projected_y(&flags);
        v_c_kernel<<<(int)((n_ + 31) / 32), kThreads, 0, stream_>>>(
            V_->device_table(), n_, k, y, nullptr, d_x, 0, partials_, counter_ + 5, dstate_,
            kHookNone, m_, 0, 1);
        AMFLS_LAUNCHED();
        projected_flags_ = flags;
        return;
    }
    const double rcond = std::min(0.5, 64.0 * kEps * std::max(host_.rows_t, k));
    projected_solve_kernel<<<1, 32, 0, stream_>>>(alpha_, beta_, g_, k, host_.rows_t, reg_, qr_,
                                                  tcap_, qr_state_, rcond);
    AMFLS_LAUNCHED();
    const double* y = qr_ + 3 * (long long)tcap_;
    v_c_kernel<<<(int)((n_ + 31) / 32), kThreads, 0, stream_>>>(
        V_->device_table(), n_, k, y, nullptr, d_x, 0, partials_, counter_ + 5, dstate_, kHookNone,
        m_, 0, 1);
    AMFLS_LAUNCHED();
    double st[8];
    AMFLS_CUDA(cudaMemcpyAsync(st, qr_state_, sizeof(double) * 8, cudaMemcpyDeviceToHost, stream_));
    stream_wait(stream_);
    projected_flags_ = (int)st[5];
}

namespace {

__global__ void probe_fill_kernel(double* const* panels, int n, int k, double* r) {
    const long long total = (long long)n * 32;
    const int P = (k + 31) / 32;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total * P;
         i += (long long)gridDim.x * blockDim.x) {
        const int p = (int)(i / total);
        const long long e = i - (long long)p * total;
        const long long row = e / 32;
        const int col = p * 32 + (int)(e % 32);
        panels[p][e] = col < k ? (double)((row * 7 + col * 13) % 17 - 8) * 1e-3 : 0.0;
        if (p == 0 && e % 32 == 0) r[row] = (double)((row * 5) % 11 - 5) * 1e-2;
    }
}

}  // namespace

void probe_reorthogonalization(int n, int k, int reps, cudaStream_t s, double seconds[2]) {
    if (n <= 0 || k <= 0 || reps <= 0) throw std::invalid_argument("probe sizes must be positive");
    const int P = (k + 31) / 32;
    int pcap = 4;
    while (pcap < P) pcap *= 2;
    PanelStore V(n, pcap, s);
    V.ensure_columns(k);
    double *r = nullptr, *w = nullptr, *c = nullptr, *partials = nullptr;
    unsigned* counters = nullptr;
    DevState* st = nullptr;
    const long long vc_off = (long long)(kGemvTargetBlocks + pcap) * 32 + 6 * 1216;
    stream_alloc(&r, sizeof(double) * n, s);
    stream_alloc(&w, sizeof(double) * n, s);
    stream_alloc(&c, sizeof(double) * 32 * pcap, s);
    stream_alloc(&partials, sizeof(double) * (vc_off + (n + 31) / 32 + 1024), s);
    stream_alloc(&counters, sizeof(unsigned) * (64 + pcap + 64), s);
    stream_alloc(&st, sizeof(DevState), s);
    AMFLS_CUDA(cudaMemsetAsync(counters, 0, sizeof(unsigned) * (64 + pcap + 64), s));
    DevState h;
    std::memset(&h, 0, sizeof(h));
    h.k = k;
    h.go = 1;
    h.reliable = 1;
    h.basis_limit = k + 1;
    h.right_scale = 1.0;
    h.norm_before = 1e300;  // the pass never decides the level: state stays as set
    AMFLS_CUDA(cudaMemcpyAsync(st, &h, sizeof(DevState), cudaMemcpyHostToDevice, s));
    probe_fill_kernel<<<1216, 256, 0, s>>>(V.device_table(), n, k, r);
    AMFLS_LAUNCHED();
    const int max_chunks = (int)std::max<long long>(1, (n + 255) / 256);
    const int chunks = std::max(1, std::min(max_chunks, (kGemvTargetBlocks + pcap - 1) / pcap));
    const int chunk_rows = (int)(((long long)n + chunks - 1) / chunks);
    const dim3 tgrid(pcap, chunks);
    const int ngrid = (int)((n + 31) / 32);
    auto vt = [&] {
        vt_r_kernel<<<tgrid, kThreads, 0, s>>>(V.device_table(), n, chunk_rows, r, c, partials,
                                               counters + 64, st, 1);
        AMFLS_LAUNCHED();
    };
    auto vc = [&] {
        v_c_kernel<<<ngrid, kThreads, 0, s>>>(V.device_table(), n, -1, c, r, w, 0,
                                              partials + vc_off, counters + 3, st,
                                              kHookRightPass1, n, 1, 1);
        AMFLS_LAUNCHED();
    };
    cudaEvent_t e[3];
    for (auto& ev : e) AMFLS_CUDA(cudaEventCreate(&ev));
    for (int i = 0; i < 3; ++i) {  // warm-up
        vt();
        vc();
    }
    AMFLS_CUDA(cudaEventRecord(e[0], s));
    for (int i = 0; i < reps; ++i) vt();
    AMFLS_CUDA(cudaEventRecord(e[1], s));
    for (int i = 0; i < reps; ++i) vc();
    AMFLS_CUDA(cudaEventRecord(e[2], s));
    AMFLS_CUDA(cudaEventSynchronize(e[2]));
    float ms0 = 0.f, ms1 = 0.f;
    AMFLS_CUDA(cudaEventElapsedTime(&ms0, e[0], e[1]));
    AMFLS_CUDA(cudaEventElapsedTime(&ms1, e[1], e[2]));
    for (auto& ev : e) cudaEventDestroy(ev);
    seconds[0] = ms0 * 1e-3 / reps;
    seconds[1] = ms1 * 1e-3 / reps;
    stream_free(r, s);
    stream_free(w, s);
    stream_free(c, s);
    stream_free(partials, s);
    stream_free(counters, s);
    stream_free(st, s);
    stream_wait(s);
}

}  // namespace amfls_gpu
