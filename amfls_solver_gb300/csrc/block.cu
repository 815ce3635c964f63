// Block kernels for the block Golub-Kahan path (width > 1).
//
// They implement the block branches of the reference's
// orthogonalize_and_factor (src/algorithms/mathematics/krylov/
// krylov_workspace.cpp:172-195 block CGS2, :263-307 the rank-revealing SVD of
// the residual block) and the projected solve of evaluate
// (krylov_workspace.cpp:833-909):
//   * tall-skinny products X^T Y and X C for column-major blocks, and the
//     same against the panel-stored basis V;
//   * the residual block B (rows x c) is reduced to its R factor by
//     Householder TSQR (backward stable, so R's singular values are B's to
//     working accuracy, as dgesdd's are), and R's SVD comes from one-sided
//     Jacobi (high relative accuracy);
//   * the host forms q = B W_r Sigma_r^{-1} and re-orthogonalises it once by
//     Cholesky QR (q <- q U^{-1}, factor <- U Sigma_r W_r^T), which spans the
//     reference's U_r and keeps B = q factor + discarded part;
//   * T is block lower bidiagonal, so [T; sqrt(lambda) I] is reduced level by
//     level with small Householder QRs of the stacked (leftover, new,
//     damping) rows, keeping only as many leftover rows as couple to the next
//     column block.  Whenever T has full column rank this solves the same
//     projected problem as the reference's dgelsy (lambda = 0) and SVD ridge
//     filter (lambda > 0).
// Shared memory holds a factorisation when it fits; wider blocks work in a
// global-memory scratch (L2 resident) with the same code.
#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "block.hpp"
#include "common.cuh"

namespace amfls_gpu {
namespace {

constexpr int kThreads = 256;
constexpr long long kSmemDoubles = 26 * 1024;  // 208 KB of dynamic shared memory
constexpr int kColsPerCall = 64;               // column group of the panel kernels

template <typename Kernel>
void allow_smem(Kernel kernel, size_t bytes) {
    if (bytes > 48 * 1024)
        AMFLS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(bytes)));
}

int grid_for(long long work, int per_block, int cap) {
    return static_cast<int>(
        std::max<long long>(1, std::min<long long>(cap, ceil_div(work, per_block))));
}

// ------------------------------------------------------------ products ----

__global__ void __launch_bounds__(kThreads)
ts_tn_partial_kernel(const double* __restrict__ X, long long ldx, const double* __restrict__ Y,
                     long long ldy, long long m, int a, int b, int tiles_a,
                     long long rows_per_chunk, double* partials) {
    __shared__ double xs[32][33];
    __shared__ double ys[32][33];
    const int ta = blockIdx.y % tiles_a, tb = blockIdx.y / tiles_a;
    const int x0 = ta * 32, y0 = tb * 32;
    const long long r0 = blockIdx.x * rows_per_chunk;
    const long long r1 = min(m, r0 + rows_per_chunk);
    const int p = threadIdx.x & 31, q0 = threadIdx.x >> 5;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long base = r0; base < r1; base += 32) {
        for (int t = threadIdx.x; t < 1024; t += kThreads) {
            const int i = t & 31, col = t >> 5;
            const long long r = base + i;
            const bool in = r < r1;
            xs[i][col] = (in && x0 + col < a) ? X[r + (long long)(x0 + col) * ldx] : 0.0;
            ys[i][col] = (in && y0 + col < b) ? Y[r + (long long)(y0 + col) * ldy] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int i = 0; i < 32; ++i) {
            const double xv = xs[i][p];
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[u] = fma(xv, ys[i][q0 + 8 * u], acc[u]);
        }
        __syncthreads();
    }
    const long long ab = (long long)a * b;
    double* out = partials + blockIdx.x * ab;
    const int row = x0 + p;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int col = y0 + q0 + 8 * u;
        if (row < a && col < b) out[row + (long long)col * a] = acc[u];
    }
}

__global__ void sum_chunks_kernel(const double* partials, int chunks, long long count, double* C,
                                  int* nonfinite) {
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < count;
         o += (long long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < chunks; ++c) s += partials[c * count + o];
        C[o] = s;
        if (nonfinite != nullptr && !isfinite(s)) *nonfinite = 1;
    }
}

__global__ void __launch_bounds__(kThreads)
ts_nn_kernel(const double* __restrict__ X, long long ldx, const double* C, long long m, int a,
             int b, double* Y, long long ldy, double alpha, double beta, int c_in_smem) {
    extern __shared__ double cs[];
    const double* cp = C;
    if (c_in_smem) {
        for (int t = threadIdx.x; t < a * b; t += blockDim.x) cs[t] = C[t];
        __syncthreads();
        cp = cs;
    }
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < m;
         r += (long long)gridDim.x * blockDim.x) {
        for (int j0 = 0; j0 < b; j0 += 8) {
            const int nj = min(8, b - j0);
            double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            for (int i = 0; i < a; ++i) {
                const double x = X[r + (long long)i * ldx];
#pragma unroll
                for (int jj = 0; jj < 8; ++jj)
                    if (jj < nj) acc[jj] = fma(x, cp[i + (long long)(j0 + jj) * a], acc[jj]);
            }
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) {
                if (jj < nj) {
                    double* yp = Y + r + (long long)(j0 + jj) * ldy;
                    *yp = (beta == 0.0 ? 0.0 : beta * *yp) + alpha * acc[jj];
                }
            }
        }
    }
}

// grid (panels, chunks): lane = column of the panel, warp w sums R columns
// w, w + 8, ... (c <= 64); partials [panel][chunk][c][32]
__global__ void __launch_bounds__(kThreads)
panel_tn_partial_kernel(double* const* __restrict__ panels, long long n,
                        const double* __restrict__ R, long long ldr, int c,
                        long long rows_per_chunk, double* partials) {
    __shared__ double vs[32][33];
    __shared__ double rs[32][65];
    const int p = blockIdx.x, chunk = blockIdx.y, nchunks = gridDim.y;
    const double* __restrict__ vp = panels[p];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long r0 = chunk * rows_per_chunk;
    const long long r1 = min(n, r0 + rows_per_chunk);
    double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (long long base = r0; base < r1; base += 32) {
        for (int t = threadIdx.x; t < 1024; t += kThreads) {
            const int i = t >> 5, col = t & 31;
            const long long r = base + i;
            vs[i][col] = r < r1 ? vp[r * 32 + col] : 0.0;
        }
        for (int t = threadIdx.x; t < 32 * c; t += kThreads) {
            const int i = t & 31, col = t >> 5;
            const long long r = base + i;
            rs[i][col] = r < r1 ? R[r + (long long)col * ldr] : 0.0;
        }
        __syncthreads();
        for (int i = 0; i < 32; ++i) {
            const double v = vs[i][lane];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int j = warp + 8 * u;
                if (j < c) acc[u] = fma(v, rs[i][j], acc[u]);
            }
        }
        __syncthreads();
    }
    double* out = partials + ((long long)p * nchunks + chunk) * 32 * c;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const int j = warp + 8 * u;
        if (j < c) out[j * 32 + lane] = acc[u];
    }
}

__global__ void panel_tn_reduce_kernel(const double* partials, int P, int nchunks, int k, int c,
                                       double* C, long long ldc, int* nonfinite) {
    const long long total = (long long)P * 32 * c;
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < total;
         o += (long long)gridDim.x * blockDim.x) {
        const int lane = (int)(o % 32);
        const long long rest = o / 32;
        const int j = (int)(rest % c);
        const int p = (int)(rest / c);
        const int col = p * 32 + lane;
        if (col >= k) continue;
        double s = 0.0;
        for (int ch = 0; ch < nchunks; ++ch)
            s += partials[(((long long)p * nchunks + ch) * c + j) * 32 + lane];
        C[col + j * ldc] = s;
        if (nonfinite != nullptr && !isfinite(s)) *nonfinite = 1;
    }
}

// one block per 32 rows: lane = row, warp w accumulates columns w, w + 8, ...
__global__ void __launch_bounds__(kThreads)
panel_nn_kernel(double* const* __restrict__ panels, long long n, int first, int w,
                const double* __restrict__ C, int c, double* R, long long ldr, double alpha) {
    __shared__ double vs[32][33];
    const long long row0 = blockIdx.x * 32LL;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const int p0 = first / 32, p1 = (first + w - 1) / 32;
    for (int p = p0; p <= p1; ++p) {
        const double* __restrict__ vp = panels[p];
        for (int t = threadIdx.x; t < 1024; t += kThreads) {
            const int i = t >> 5, col = t & 31;
            const long long r = row0 + i;
            vs[i][col] = r < n ? vp[r * 32 + col] : 0.0;
        }
        __syncthreads();
        const int lo = max(first, p * 32), hi = min(first + w, p * 32 + 32);
        for (int col = lo; col < hi; ++col) {
            const double v = vs[lane][col - p * 32];
            const double* crow = C + (col - first);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int j = warp + 8 * u;
                if (j < c) acc[u] = fma(v, crow[(long long)j * w], acc[u]);
            }
        }
        __syncthreads();
    }
    const long long r = row0 + lane;
    if (r < n) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int j = warp + 8 * u;
            if (j < c) R[r + (long long)j * ldr] += alpha * acc[u];
        }
    }
}

__global__ void panel_append_kernel(double* const* panels, long long n, int k0, const double* Q,
                                    int r) {
    const long long total = n * r;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long i = t % n;
        const int col = k0 + (int)(t / n);
        panels[col >> 5][i * 32 + (col & 31)] = Q[t];
    }
}

// --------------------------------------------------------- Householder ----

// In-place Householder QR of the first nf columns of A (rows x nt,
// column-major, leading dimension lda, shared or global memory), applying
// each reflector to all nt columns (LAPACK dlarfg convention; R on and above
// the diagonal, zeros below).  Every thread of the block must call it.
__device__ void cta_qr(double* A, int rows, int nf, int nt, int lda, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __shared__ double s_tau, s_beta, s_scale;
    for (int j = 0; j < nf && j < rows; ++j) {
        double* col = A + (long long)j * lda;
        double part = 0.0;
        for (int i = j + 1 + threadIdx.x; i < rows; i += blockDim.x) part = fma(col[i], col[i], part);
        const double sigma = block_sum(part, red);
        if (threadIdx.x == 0) {
            const double x0 = col[j];
            if (sigma == 0.0) {
                s_tau = 0.0;
                s_beta = x0;
                s_scale = 0.0;
            } else {
                const double nrm = sqrt(fma(x0, x0, sigma));
                const double beta = x0 >= 0.0 ? -nrm : nrm;
                s_tau = (beta - x0) / beta;
                s_scale = 1.0 / (x0 - beta);
                s_beta = beta;
            }
        }
        __syncthreads();
        const double tau = s_tau, scale = s_scale, beta = s_beta;
        if (tau != 0.0) {
            for (int i = j + 1 + threadIdx.x; i < rows; i += blockDim.x) col[i] *= scale;
        }
        __syncthreads();
        if (tau != 0.0) {
            for (int l = j + 1 + warp; l < nt; l += nw) {
                double* cl = A + (long long)l * lda;
                double w = lane == 0 ? cl[j] : 0.0;  // v_j = 1
                for (int i = j + 1 + lane; i < rows; i += 32) w = fma(col[i], cl[i], w);
                w = warp_sum(w) * tau;
                if (lane == 0) cl[j] -= w;
                for (int i = j + 1 + lane; i < rows; i += 32) cl[i] = fma(-w, col[i], cl[i]);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) col[j] = beta;
        for (int i = j + 1 + threadIdx.x; i < rows; i += blockDim.x) col[i] = 0.0;
        __syncthreads();
    }
}

struct TsqrPlan {
    int cr;  // rows per leaf
    long long leaves;
    int g;  // R blocks stacked per tree node
    bool leaf_smem, tree_smem;
};

TsqrPlan tsqr_plan(long long rows, int c) {
    TsqrPlan p;
    p.cr = static_cast<int>(std::max<long long>(c, std::min<long long>(256, kSmemDoubles / c)));
    p.leaves = std::max<long long>(1, ceil_div(rows, p.cr));
    p.leaf_smem = (long long)p.cr * c <= kSmemDoubles;
    const long long cc = (long long)c * c;
    p.g = static_cast<int>(std::max<long long>(2, std::min<long long>(64, kSmemDoubles / cc)));
    p.tree_smem = p.g * cc <= kSmemDoubles;
    return p;
}

__global__ void __launch_bounds__(kThreads)
tsqr_leaf_kernel(const double* B, long long rows, int c, long long ldb, int cr, double* Rout,
                 double* gscratch) {
    extern __shared__ double sm[];
    __shared__ double red[32];
    double* A = gscratch ? gscratch + blockIdx.x * (long long)cr * c : sm;
    const long long r0 = blockIdx.x * (long long)cr;
    for (long long t = threadIdx.x; t < (long long)cr * c; t += blockDim.x) {
        const int i = (int)(t % cr), j = (int)(t / cr);
        const long long r = r0 + i;
        A[t] = r < rows ? B[r + j * ldb] : 0.0;
    }
    __syncthreads();
    cta_qr(A, cr, c, c, cr, red);
    double* out = Rout + blockIdx.x * (long long)c * c;
    for (int t = threadIdx.x; t < c * c; t += blockDim.x) {
        const int i = t % c, j = t / c;
        out[t] = i <= j ? A[i + (long long)j * cr] : 0.0;
    }
}

__global__ void __launch_bounds__(kThreads)
tsqr_tree_kernel(const double* Rin, long long nin, int c, int g, double* Rout, double* gscratch) {
    extern __shared__ double sm[];
    __shared__ double red[32];
    const int rows = g * c;
    double* A = gscratch ? gscratch + blockIdx.x * (long long)rows * c : sm;
    const long long first = blockIdx.x * (long long)g;
    const long long cnt = min((long long)g, nin - first);
    for (long long t = threadIdx.x; t < (long long)rows * c; t += blockDim.x) {
        const int i = (int)(t % rows), j = (int)(t / rows);
        const int blk = i / c, ii = i % c;
        A[t] = blk < cnt ? Rin[(first + blk) * c * c + ii + (long long)j * c] : 0.0;
    }
    __syncthreads();
    cta_qr(A, rows, c, c, rows, red);
    double* out = Rout + blockIdx.x * (long long)c * c;
    for (int t = threadIdx.x; t < c * c; t += blockDim.x) {
        const int i = t % c, j = t / c;
        out[t] = i <= j ? A[i + (long long)j * rows] : 0.0;
    }
}

// ------------------------------------------------------------- Jacobi ----

__device__ __forceinline__ void jacobi_rotation(double a, double b, double g, double& cs,
                                                double& sn) {
    const double zeta = (b - a) / (2.0 * g);
    double t;
    if (fabs(zeta) > 1e150) t = 0.5 / zeta;
    else t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(fma(zeta, zeta, 1.0)));
    cs = 1.0 / sqrt(fma(t, t, 1.0));
    sn = cs * t;
}

// One-sided (Hestenes) Jacobi on the columns of R with a round-robin
// ordering: in each round every warp rotates disjoint column pairs.
__global__ void __launch_bounds__(kThreads)
jacobi_svd_kernel(const double* R, int c, double* sigma, double* W, double* gwork) {
    extern __shared__ double sm[];
    __shared__ int s_rotated;
    double* base = gwork ? gwork : sm;
    double* M = base;
    double* V = base + (long long)c * c;
    double* nrm = V + (long long)c * c;
    int* order = reinterpret_cast<int*>(nrm + c);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (long long t = threadIdx.x; t < (long long)c * c; t += blockDim.x) {
        M[t] = R[t];
        V[t] = (t % c) == (t / c) ? 1.0 : 0.0;
    }
    __syncthreads();
    const int ce = c + (c & 1);  // even player count for the round-robin tournament
    const double tol = 2.220446049250313e-16 * sqrt((double)c);
    for (int sweep = 0; sweep < 60 && c > 1; ++sweep) {
        if (threadIdx.x == 0) s_rotated = 0;
        __syncthreads();
        for (int round = 0; round < ce - 1; ++round) {
            for (int pair = warp; pair < ce / 2; pair += nw) {
                const int pa = pair == 0 ? 0 : 1 + (pair - 1 + round) % (ce - 1);
                const int pb = 1 + (ce - 2 - pair + round) % (ce - 1);
                if (pa >= c || pb >= c) continue;
                const int p = min(pa, pb), q = max(pa, pb);
                double* mp = M + (long long)p * c;
                double* mq = M + (long long)q * c;
                double a = 0.0, b = 0.0, g = 0.0;
                for (int i = lane; i < c; i += 32) {
                    a = fma(mp[i], mp[i], a);
                    b = fma(mq[i], mq[i], b);
                    g = fma(mp[i], mq[i], g);
                }
                a = warp_sum(a);
                b = warp_sum(b);
                g = warp_sum(g);
                if (g != 0.0 && fabs(g) > tol * sqrt(a) * sqrt(b)) {
                    double cs, sn;
                    jacobi_rotation(a, b, g, cs, sn);
                    double* vp = V + (long long)p * c;
                    double* vq = V + (long long)q * c;
                    for (int i = lane; i < c; i += 32) {
                        const double x = mp[i], y = mq[i];
                        mp[i] = cs * x - sn * y;
                        mq[i] = sn * x + cs * y;
                        const double u = vp[i], v = vq[i];
                        vp[i] = cs * u - sn * v;
                        vq[i] = sn * u + cs * v;
                    }
                    if (lane == 0) s_rotated = 1;
                }
            }
            __syncthreads();
        }
        if (!s_rotated) break;
        __syncthreads();
    }
    for (int j = warp; j < c; j += nw) {
        double s = 0.0;
        for (int i = lane; i < c; i += 32)
            s = fma(M[i + (long long)j * c], M[i + (long long)j * c], s);
        s = warp_sum(s);
        if (lane == 0) nrm[j] = sqrt(s);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 0; j < c; ++j) order[j] = j;
        for (int j = 0; j < c; ++j) {  // selection sort, descending
            int best = j;
            for (int l = j + 1; l < c; ++l)
                if (nrm[order[l]] > nrm[order[best]]) best = l;
            const int tmp = order[j];
            order[j] = order[best];
            order[best] = tmp;
            sigma[j] = nrm[order[j]];
        }
    }
    __syncthreads();
    for (long long t = threadIdx.x; t < (long long)c * c; t += blockDim.x) {
        const int i = (int)(t % c), j = (int)(t / c);
        W[t] = V[i + (long long)order[j] * c];
    }
}

__global__ void __launch_bounds__(kThreads)
cholesky_kernel(const double* G, int c, double* U, double* Uinv, int* flag) {
    __shared__ double red[32];
    __shared__ double s_d;
    __shared__ int s_bad;
    for (long long t = threadIdx.x; t < (long long)c * c; t += blockDim.x) {
        U[t] = 0.0;
        Uinv[t] = 0.0;
    }
    if (threadIdx.x == 0) s_bad = 0;
    __syncthreads();
    for (int j = 0; j < c; ++j) {
        const double* uj = U + (long long)j * c;
        double part = 0.0;
        for (int k = threadIdx.x; k < j; k += blockDim.x) part = fma(uj[k], uj[k], part);
        const double ssum = block_sum(part, red);
        if (threadIdx.x == 0) {
            double d = G[j + (long long)j * c] - ssum;
            if (!(d > 0.0) || !isfinite(d)) {
                s_bad = 1;
                d = 1.0;
            }
            s_d = sqrt(d);
            U[j + (long long)j * c] = s_d;
        }
        __syncthreads();
        const double ujj = s_d;
        for (int l = j + 1 + threadIdx.x; l < c; l += blockDim.x) {
            const double* ul = U + (long long)l * c;
            double sum = G[j + (long long)l * c];
            for (int k = 0; k < j; ++k) sum -= uj[k] * ul[k];
            U[j + (long long)l * c] = sum / ujj;
        }
        __syncthreads();
    }
    for (int jj = threadIdx.x; jj < c; jj += blockDim.x) {
        double* inv = Uinv + (long long)jj * c;
        inv[jj] = 1.0 / U[jj + (long long)jj * c];
        for (int i = jj - 1; i >= 0; --i) {
            double s = 0.0;
            for (int k = i + 1; k <= jj; ++k) s = fma(U[i + (long long)k * c], inv[k], s);
            inv[i] = -s / U[i + (long long)i * c];
        }
    }
    if (threadIdx.x == 0) *flag = s_bad;
}

// ---------------------------------------------- block projected solve ----

// Single CTA.  carry = [nl, unused, h (nl), R2 (nl x aw_next, ld nl)];
// work = L (w x w) | S ((3w+1) x (2w+1)) | T2 ((3w+1) x (w+1)).
// Level j stacks, with columns [its r unknowns | rhs | the nlw new rows]:
//     [ R2 G_j        h      0 ]   leftover rows of the previous level
//     [ N_j           g_j    I ]   the new left block's rows
//     [ sqrt(l) I     0      0 ]   damping rows (lambda > 0)
// The identity columns track where the new rows go, so the next level's G
// (not known yet) can be applied afterwards: R_{j,j+1} = W_top G_{j+1} and
// the leftover block R2 comes from a QR of W_bottom.
__global__ void __launch_bounds__(kThreads)
block_projected_kernel(const int* __restrict__ meta, const double* __restrict__ vals, int first,
                       int last, double lambda, double g0, double* state, double* carry,
                       double* work, int w, double* y, int k, double rcond, int* flags) {
    __shared__ double red[32];
    double* L = work;
    double* S = L + (long long)w * w;
    double* T2 = S + (long long)(3 * w + 1) * (2 * w + 1);
    const double root = sqrt(lambda);
    if (first == 0 && threadIdx.x == 0) {
        carry[0] = 1.0;
        carry[2] = g0;   // h
        carry[3] = 1.0;  // R2 = [1]: the first row block is b / ||b||
    }
    __syncthreads();
    for (int j = first; j < last; ++j) {
        const int* mj = meta + kLevelMeta * j;
        const int r = mj[0], aw = mj[1], nlw = mj[2];
        const double* G = vals + mj[3];
        const double* N = G + (long long)aw * r;
        const double* gn = N + (long long)nlw * r;
        double* Rjj = state + mj[4];
        double* zj = Rjj + (long long)r * r;
        double* Wt = zj + r;
        double* Rc = Wt + (long long)r * nlw;
        const int nl = (int)carry[0];
        const double* h = carry + 2;
        const double* R2 = h + nl;
        for (int t = threadIdx.x; t < nl * r; t += blockDim.x) {
            const int i = t % nl, col = t / nl;
            double s = 0.0;
            for (int l = 0; l < aw; ++l) s = fma(R2[i + l * nl], G[l + (long long)col * aw], s);
            L[t] = s;
        }
        if (j > 0) {
            const int* mp = meta + kLevelMeta * (j - 1);
            const int rp = mp[0];
            const double* Wp = state + mp[4] + (long long)rp * rp + rp;
            for (int t = threadIdx.x; t < rp * r; t += blockDim.x) {
                const int i = t % rp, col = t / rp;
                double s = 0.0;
                for (int l = 0; l < aw; ++l) s = fma(Wp[i + l * rp], G[l + (long long)col * aw], s);
                Rc[t] = s;
            }
        }
        __syncthreads();
        const int drows = lambda > 0.0 ? r : 0;
        const int rows = nl + nlw + drows;
        const int cols = r + 1 + nlw;
        for (int t = threadIdx.x; t < rows * cols; t += blockDim.x) {
            const int i = t % rows, col = t / rows;
            double v = 0.0;
            if (col < r) {
                if (i < nl) v = L[i + col * nl];
                else if (i < nl + nlw) v = N[(i - nl) + (long long)col * nlw];
                else v = (i - nl - nlw) == col ? root : 0.0;
            } else if (col == r) {
                if (i < nl) v = h[i];
                else if (i < nl + nlw) v = gn[i - nl];
            } else {
                v = (i - nl) == (col - r - 1) ? 1.0 : 0.0;
            }
            S[t] = v;
        }
        __syncthreads();
        cta_qr(S, rows, r, cols, rows, red);
        const int top = min(rows, r);
        for (int t = threadIdx.x; t < r * r; t += blockDim.x) {
            const int i = t % r, col = t / r;
            Rjj[t] = (i <= col && i < top) ? S[i + col * rows] : 0.0;
        }
        for (int t = threadIdx.x; t < r; t += blockDim.x) zj[t] = t < top ? S[t + r * rows] : 0.0;
        for (int t = threadIdx.x; t < r * nlw; t += blockDim.x) {
            const int i = t % r, col = t / r;
            Wt[t] = i < top ? S[i + (r + 1 + col) * rows] : 0.0;
        }
        const int rows2 = rows - top;
        for (int t = threadIdx.x; t < rows2 * (nlw + 1); t += blockDim.x) {
            const int i = t % rows2, col = t / rows2;
            T2[t] = col < nlw ? S[(top + i) + (r + 1 + col) * rows] : S[(top + i) + r * rows];
        }
        __syncthreads();
        if (nlw > 0 && rows2 > 0) cta_qr(T2, rows2, nlw, nlw + 1, rows2, red);
        const int nl_new = min(rows2, nlw);
        double* h_new = carry + 2;
        double* R2_new = h_new + nl_new;
        for (int t = threadIdx.x; t < nl_new; t += blockDim.x) h_new[t] = T2[t + nlw * rows2];
        for (int t = threadIdx.x; t < nl_new * nlw; t += blockDim.x) {
            const int i = t % nl_new, col = t / nl_new;
            R2_new[t] = i <= col ? T2[i + col * rows2] : 0.0;
        }
        if (threadIdx.x == 0) carry[0] = (double)nl_new;
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    // back substitution over every level
    int bad = 0;
    double dmax = 0.0, dmin = __builtin_huge_val();
    int col_end = k;
    for (int j = last - 1; j >= 0; --j) {
        const int* mj = meta + kLevelMeta * j;
        const int r = mj[0];
        const int c0 = col_end - r;
        if (c0 < 0) {
            bad |= 4;
            break;
        }
        const double* Rjj = state + mj[4];
        const double* zj = Rjj + (long long)r * r;
        const double* Rc_next = nullptr;
        int r_next = 0;
        if (j + 1 < last) {
            const int* mn = meta + kLevelMeta * (j + 1);
            r_next = mn[0];
            Rc_next = state + mn[4] + (long long)r_next * r_next + r_next + (long long)r_next * mn[2];
        }
        for (int i = r - 1; i >= 0; --i) {
            double s = zj[i];
            for (int l = 0; l < r_next; ++l) s -= Rc_next[i + (long long)l * r] * y[c0 + r + l];
            for (int l = i + 1; l < r; ++l) s -= Rjj[i + (long long)l * r] * y[c0 + l];
            const double d = Rjj[i + (long long)i * r];
            dmax = fmax(dmax, fabs(d));
            dmin = fmin(dmin, fabs(d));
            if (d != 0.0) {
                y[c0 + i] = s / d;
            } else {
                bad |= 1;
                y[c0 + i] = 0.0;
            }
        }
        col_end = c0;
    }
    if (col_end != 0) bad |= 4;
    if (lambda == 0.0 && k > 0 && !(dmin >= rcond * dmax)) bad |= 2;
    *flags = bad;
}

int ts_chunks(long long m, int tiles) {
    const long long want = ceil_div(grid_cap(), tiles);
    return static_cast<int>(std::max<long long>(1, std::min<long long>(want, ceil_div(m, 256))));
}

int panel_chunks(long long n, int P) {
    const long long want = ceil_div(2432, P);
    return static_cast<int>(std::max<long long>(1, std::min<long long>(want, ceil_div(n, 256))));
}

}  // namespace

// ------------------------------------------------------------- host API ----

long long ts_tn_partial_doubles(long long m, int a, int b) {
    const int tiles = static_cast<int>(ceil_div(a, 32) * ceil_div(b, 32));
    return (long long)ts_chunks(m, tiles) * a * b;
}

void ts_tn(const double* X, long long ldx, const double* Y, long long ldy, long long m, int a,
           int b, double* C, double* partials, int* nonfinite, cudaStream_t s) {
    if (a <= 0 || b <= 0) return;
    const int tiles_a = static_cast<int>(ceil_div(a, 32));
    const int tiles = tiles_a * static_cast<int>(ceil_div(b, 32));
    const int chunks = ts_chunks(m, tiles);
    const long long rpc = std::max<long long>(1, ceil_div(m, chunks));
    ts_tn_partial_kernel<<<dim3(chunks, tiles), kThreads, 0, s>>>(X, ldx, Y, ldy, m, a, b, tiles_a,
                                                                  rpc, partials);
    AMFLS_LAUNCHED();
    const long long ab = (long long)a * b;
    sum_chunks_kernel<<<grid_for(ab, 256, grid_cap()), 256, 0, s>>>(partials, chunks, ab, C, nonfinite);
    AMFLS_LAUNCHED();
}

void ts_nn(const double* X, long long ldx, const double* C, long long m, int a, int b, double* Y,
           long long ldy, double alpha, double beta, cudaStream_t s) {
    if (b <= 0 || m <= 0) return;
    const long long ab = (long long)a * b;
    const int in_smem = ab <= 6144 ? 1 : 0;
    const size_t smem = in_smem ? sizeof(double) * std::max<long long>(1, ab) : 0;
    ts_nn_kernel<<<grid_for(m, kThreads, grid_cap()), kThreads, smem, s>>>(X, ldx, C, m, a, b, Y, ldy,
                                                                     alpha, beta, in_smem);
    AMFLS_LAUNCHED();
}

long long panel_tn_partial_doubles(long long n, int k, int c) {
    const int P = static_cast<int>(ceil_div(std::max(k, 1), 32));
    return (long long)P * panel_chunks(n, P) * 32 * std::min(c, kColsPerCall);
}

void panel_tn(double* const* panels, long long n, int k, const double* R, long long ldr, int c,
              double* C, double* partials, int* nonfinite, cudaStream_t s) {
    if (k <= 0 || c <= 0) return;
    const int P = static_cast<int>(ceil_div(k, 32));
    const int chunks = panel_chunks(n, P);
    const long long rpc = std::max<long long>(1, ceil_div(n, chunks));
    for (int c0 = 0; c0 < c; c0 += kColsPerCall) {
        const int cc = std::min(kColsPerCall, c - c0);
        panel_tn_partial_kernel<<<dim3(P, chunks), kThreads, 0, s>>>(
            panels, n, R + (long long)c0 * ldr, ldr, cc, rpc, partials);
        AMFLS_LAUNCHED();
        panel_tn_reduce_kernel<<<grid_for((long long)P * 32 * cc, 256, grid_cap()), 256, 0, s>>>(
            partials, P, chunks, k, cc, C + (long long)c0 * k, k, nonfinite);
        AMFLS_LAUNCHED();
    }
}

void panel_nn(double* const* panels, long long n, int first, int w, const double* C, int c,
              double* R, long long ldr, double alpha, cudaStream_t s) {
    if (w <= 0 || c <= 0) return;
    const long long blocks = ceil_div(n, 32);
    for (int c0 = 0; c0 < c; c0 += kColsPerCall) {
        const int cc = std::min(kColsPerCall, c - c0);
        panel_nn_kernel<<<static_cast<unsigned>(blocks), kThreads, 0, s>>>(
            panels, n, first, w, C + (long long)c0 * w, cc, R + (long long)c0 * ldr, ldr, alpha);
        AMFLS_LAUNCHED();
    }
}

void panel_append(double* const* panels, long long n, int k0, const double* Q, int r,
                  cudaStream_t s) {
    if (r <= 0) return;
    panel_append_kernel<<<grid_for(n * r, 256, 2432), 256, 0, s>>>(panels, n, k0, Q, r);
    AMFLS_LAUNCHED();
}

long long tsqr_work_doubles(long long rows, int c) {
    const TsqrPlan p = tsqr_plan(rows, c);
    const long long cc = (long long)c * c;
    long long total = 2 * p.leaves * cc;
    if (!p.leaf_smem) total += p.leaves * p.cr * c;
    if (!p.tree_smem) total += (ceil_div(p.leaves, p.g) + 1) * p.g * cc;
    return total + 64;
}

void tsqr_r(const double* B, long long rows, int c, long long ldb, double* R, double* work,
            cudaStream_t s) {
    if (c <= 0) return;
    const TsqrPlan p = tsqr_plan(rows, c);
    const long long cc = (long long)c * c;
    double* a = work;
    double* b = work + p.leaves * cc;
    double* gs = b + p.leaves * cc;
    const size_t leaf_smem = p.leaf_smem ? sizeof(double) * p.cr * c : 0;
    allow_smem(tsqr_leaf_kernel, leaf_smem);
    tsqr_leaf_kernel<<<static_cast<unsigned>(p.leaves), kThreads, leaf_smem, s>>>(
        B, rows, c, ldb, p.cr, a, p.leaf_smem ? nullptr : gs);
    AMFLS_LAUNCHED();
    const size_t tree_smem = p.tree_smem ? sizeof(double) * p.g * cc : 0;
    allow_smem(tsqr_tree_kernel, tree_smem);
    long long n = p.leaves;
    while (n > 1) {
        const long long out = ceil_div(n, p.g);
        tsqr_tree_kernel<<<static_cast<unsigned>(out), kThreads, tree_smem, s>>>(
            a, n, c, p.g, b, p.tree_smem ? nullptr : gs);
        AMFLS_LAUNCHED();
        std::swap(a, b);
        n = out;
    }
    AMFLS_CUDA(cudaMemcpyAsync(R, a, sizeof(double) * cc, cudaMemcpyDeviceToDevice, s));
}

long long jacobi_work_doubles(int c) { return 2LL * c * c + 2LL * c + 8; }

void jacobi_svd(const double* R, int c, double* sigma, double* W, double* work, cudaStream_t s) {
    if (c <= 0) return;
    const long long need = jacobi_work_doubles(c);
    const bool in_smem = need <= kSmemDoubles;
    const size_t smem = in_smem ? sizeof(double) * need : 0;
    allow_smem(jacobi_svd_kernel, smem);
    jacobi_svd_kernel<<<1, kThreads, smem, s>>>(R, c, sigma, W, in_smem ? nullptr : work);
    AMFLS_LAUNCHED();
}

void cholesky_upper(const double* G, int c, double* U, double* Uinv, int* flag, cudaStream_t s) {
    if (c <= 0) return;
    cholesky_kernel<<<1, kThreads, 0, s>>>(G, c, U, Uinv, flag);
    AMFLS_LAUNCHED();
}

long long level_state_doubles(int r, int nlw, int r_prev) {
    return (long long)r * r + r + (long long)r * nlw + (long long)r_prev * r;
}

long long projected_carry_doubles(int w) {
    const long long W = std::max(1, w);
    return 2 + W + W * W + 8;
}

long long projected_work_doubles(int w) {
    const long long W = std::max(1, w);
    return W * W + (3 * W + 1) * (2 * W + 1) + (3 * W + 1) * (W + 1) + 64;
}

void block_projected_solve(const LevelRecords& rec, int first, int last, int w, double lambda,
                           double g0, double* state, double* carry, double* work, double* y,
                           int k, double rcond, int* flags, cudaStream_t s) {
    if (last <= 0) return;
    block_projected_kernel<<<1, kThreads, 0, s>>>(rec.meta, rec.vals, first, last, lambda, g0,
                                                  state, carry, work, std::max(1, w), y, k, rcond,
                                                  flags);
    AMFLS_LAUNCHED();
}

}  // namespace amfls_gpu
