// Mixed-precision AMFLS: inner solves on a reduced-precision operator inside
// an outer FP64 residual-correction loop (iterative refinement).  No
// counterpart in the reference, whose solver is FP64 throughout; every
// termination decision is the reference's certified FP64 validation
// (candidate_validation.cpp:1176-1378) of the current x on the original
// operator, so a reduced inner product can never change what counts as
// converged.
//
// With M = [A; sqrt(lambda) I], c = [b; 0] (M = A, c = b for lambda = 0),
// x_0 = 0 and the FP64 residual s_k = M x_k - c:
//   d_k = argmin ||M~ d - s_k||   (AMFLS, lambda 0, on the reduced M~)
//   x_{k+1} = x_k - d_k
// until the FP64 certificate of x meets the tolerance, the certificate stops
// shrinking (by a factor of two after a converged inner solve; at all within
// two steps after inner solves cut by maximum_depth), or the budget is spent.  With
// maximum_depth set and a tiny inner tolerance each inner solve is one
// restart cycle of L = maximum_depth levels (restarted CG on the normal
// equations, whose latest iterate minimises the energy-norm error over its
// Krylov space): the basis, and so the cost of its sweeps, stays bounded by
// L instead of growing with the whole solve.
// When the reduced steps stop contracting (the levelling-off below) and the
// reduced operator is not the FP64 one, the remaining steps run their inner
// solves on the FP64 operator instead (a precision schedule), so the form
// reaches what FP64 inner solves reach while the early steps use the cheaper
// products.
// Each step contracts the error by about cond(M) u_low + the inner
// tolerance.  The inner AMFLS stops on a backward error relative to the
// correction problem, whose residual tends to s* = M x* - c, so when s* is
// not small (inconsistent least squares, ridge problems with small lambda)
// the gradient M^T s_k levels off near tau_in ||M|| ||s*|| (and
// u_low cond(M)^2 ||s*|| / ||M|| in x, from E^T s*): the method certifies
// small tolerances for nearly consistent problems and reports failure,
// never a false success, below that level.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <stdexcept>
#include <vector>

#include "common.cuh"
#include "controller.hpp"
#include "reduced_operator.hpp"

namespace amfls_gpu {
namespace {

// out = a + s * b
__global__ void axpy_kernel(const double* a, double s, const double* b, long long n,
                            double* out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = fma(s, b[i], a[i]);
}

int grid_for(long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, grid_cap()));
}

double certificate_of(const ValidationOutput& v, double reg) {
    return reg > 0.0 ? v.relative_energy_error_upper_bound : v.backward_error_upper_bound;
}

void accumulate(Statistics& into, const Statistics& s) {
    into.a_columns += s.a_columns;
    into.at_columns += s.at_columns;
    into.a_block_calls += s.a_block_calls;
    into.at_block_calls += s.at_block_calls;
    into.search_a_columns += s.search_a_columns;
    into.search_at_columns += s.search_at_columns;
    into.search_a_block_calls += s.search_a_block_calls;
    into.search_at_block_calls += s.search_at_block_calls;
    into.validation_a_columns += s.validation_a_columns;
    into.validation_at_columns += s.validation_at_columns;
    into.validation_a_block_calls += s.validation_a_block_calls;
    into.validation_at_block_calls += s.validation_at_block_calls;
    into.base_validation_a_columns += s.base_validation_a_columns;
    into.base_validation_at_columns += s.base_validation_at_columns;
    into.base_validation_a_block_calls += s.base_validation_a_block_calls;
    into.base_validation_at_block_calls += s.base_validation_at_block_calls;
    into.gaussian_random_columns += s.gaussian_random_columns;
    into.gaussian_random_values += s.gaussian_random_values;
    into.gaussian_random_block_requests += s.gaussian_random_block_requests;
    into.a_seconds += s.a_seconds;
    into.at_seconds += s.at_seconds;
    into.orthogonalization_seconds += s.orthogonalization_seconds;
    into.projected_solve_seconds += s.projected_solve_seconds;
    into.validation_seconds += s.validation_seconds;
    into.base_validation_seconds += s.base_validation_seconds;
    into.projected_rank_flags += s.projected_rank_flags;
    into.reduced_levels += s.reduced_levels;
    into.reduced_fallbacks += s.reduced_fallbacks;
}

void count_validation(Statistics& s, const ValidationOutput& v) {
    const int a = v.calls[0] + v.calls[2] + v.calls[4], at = v.calls[1] + v.calls[3] + v.calls[5];
    s.a_columns += a;
    s.at_columns += at;
    s.a_block_calls += a;
    s.at_block_calls += at;
    s.validation_a_columns += a;
    s.validation_at_columns += at;
    s.validation_a_block_calls += a;
    s.validation_at_block_calls += at;
    s.base_validation_a_columns += v.calls[0] + v.calls[2];
    s.base_validation_at_columns += v.calls[1] + v.calls[3];
    s.ridge_correction_a_columns += v.calls[4];
    s.ridge_correction_at_columns += v.calls[5];
}

}  // namespace

SolveResult solve_amfls_mixed(const DeviceOperator& op, const DeviceOperator& reduced,
                              const double* d_b, const SolveOptions& o, double inner_tolerance,
                              int maximum_refinements, double* d_solution, cudaStream_t stream,
                              std::vector<RefinementStep>* steps) {
    if (op.rows() <= 0 || op.cols() <= 0) throw std::invalid_argument("operator dimensions must be positive");
    if (reduced.rows() != op.rows() || reduced.cols() != op.cols())
        throw std::invalid_argument("reduced operator must have the operator's shape");
    if (d_b == nullptr || d_solution == nullptr)
        throw std::invalid_argument("right-hand side and solution cannot be null");
    if (!std::isfinite(o.regularization) || o.regularization < 0.0)
        throw std::invalid_argument("regularization must be finite and nonnegative");
    if (!std::isfinite(o.tolerance) || o.tolerance <= 0.0 || o.tolerance >= 1.0)
        throw std::invalid_argument("tolerance must lie strictly between zero and one");
    if (!std::isfinite(inner_tolerance) || inner_tolerance <= 0.0 || inner_tolerance >= 1.0)
        throw std::invalid_argument("inner tolerance must lie strictly between zero and one");
    if (maximum_refinements <= 0) throw std::invalid_argument("maximum_refinements must be positive");
    const auto t0 = std::chrono::steady_clock::now();
    const long long launches0 = launch_count();
    const double reg = o.regularization;
    const long long m = op.rows(), n = op.cols();
    const bool ridge = reg > 0.0;
    const long long ma = ridge ? m + n : m;  // rows of M

    double *res = nullptr, *dx = nullptr;
    struct Free {  // frees both buffers however the solve ends
        double** p[2];
        ~Free() {
            for (double** q : p) cudaFree(*q);
        }
    } release{{&res, &dx}};
    AMFLS_CUDA(cudaMalloc(&res, sizeof(double) * ma));
    AMFLS_CUDA(cudaMalloc(&dx, sizeof(double) * n));

    // inner operators: M~ on the reduced operator, and M on the FP64 one
    // for the steps after the reduced ones stop contracting
    const bool escalate = &reduced != &op;
    std::unique_ptr<AugmentedOperator> aug_low, aug_high;
    if (ridge) aug_low = std::make_unique<AugmentedOperator>(reduced, reg, stream);
    if (ridge && escalate) aug_high = std::make_unique<AugmentedOperator>(op, reg, stream);
    const DeviceOperator* Ml = ridge ? static_cast<const DeviceOperator*>(aug_low.get()) : &reduced;
    bool fp64_inner = !escalate;

    Validator validator(op, d_b, reg, stream);
    SolveResult out;
    out.rows = (int)m;
    out.cols = (int)n;
    // x_0 = 0: s_0 = -c
    AMFLS_CUDA(cudaMemsetAsync(d_solution, 0, sizeof(double) * n, stream));
    AMFLS_CUDA(cudaMemsetAsync(res, 0, sizeof(double) * ma, stream));
    axpy_kernel<<<grid_for(m), 256, 0, stream>>>(res, -1.0, d_b, m, res);
    AMFLS_LAUNCHED();

    SolveOptions io = o;
    io.regularization = 0.0;
    io.tolerance = inner_tolerance;
    // an inner solve cut by maximum_depth is a restart cycle: its latest
    // iterate is the best correction in the energy norm
    io.latest_at_limit = true;
    double best = __builtin_huge_val();
    double best_before_last = __builtin_huge_val();  // best certificate before the last step
    for (int k = 0; k < maximum_refinements; ++k) {
        io.stream = o.stream + (std::uint64_t)k;
        const SolveResult xr = solve_amfls(*Ml, res, io, dx, stream);
        accumulate(out.statistics, xr.statistics);
        out.depth += xr.depth;
        out.iterations += xr.iterations;
        out.basis_rank = std::max(out.basis_rank, xr.basis_rank);
        out.auxiliary_width = std::max(out.auxiliary_width, xr.auxiliary_width);
        axpy_kernel<<<grid_for(n), 256, 0, stream>>>(d_solution, -1.0, dx, n, d_solution);
        AMFLS_LAUNCHED();

        const ValidationOutput v = validator.validate(d_solution, o.tolerance);
        count_validation(out.statistics, v);
        out.v = v;
        out.status = v.status;
        out.stop_reason = v.stop_reason;
        const double cert = certificate_of(v, reg);
        TraceRow row{};
        const double fr[29] = {
            double(k), double(out.depth), fp64_inner ? 1.0 : 0.0, double(xr.basis_rank),
            double(out.statistics.a_columns), double(out.statistics.at_columns),
            double(out.statistics.a_block_calls), double(out.statistics.at_block_calls),
            v.objective, v.residual_norm, v.augmented_residual_norm, v.normal_residual_norm,
            v.operator_norm_lower_bound, v.compatible_backward_error_upper_bound,
            v.least_squares_backward_error_upper_bound, v.backward_error_upper_bound,
            v.relative_normal_residual_upper_bound, v.relative_energy_error_upper_bound,
            v.solution_norm, v.solution_energy_norm, v.augmented_operator_norm_lower_bound,
            v.energy_error_upper_bound, v.objective_gap_upper_bound,
            v.ridge_base_energy_error_upper_bound, v.ridge_corrected_energy_error_upper_bound,
            v.ridge_correction_gamma, v.ridge_correction_z_h_z,
            v.ridge_correction_two_abs_z_t_q, v.ridge_correction_q_norm_squared};
        std::copy(fr, fr + 29, row.f);
        row.i[0] = v.status;
        row.i[1] = v.stop_reason;
        row.i[2] = v.status == 0 ? 1 : 0;
        row.i[3] = v.ridge_correction_disposition;
        out.trace.push_back(row);
        if (steps)
            steps->push_back(RefinementStep{xr.status, xr.stop_reason, xr.depth, xr.basis_rank,
                                            cert});
        if (v.status == 0) break;
        // no longer contracting: an inner solve that converged (no depth
        // limit) must halve the certificate; restart cycles (stopped by
        // maximum_depth) must reduce it within two cycles (restarted Krylov
        // cycles often alternate a large and a small decrease)
        const bool cycle = xr.stop_reason == 3;
        const bool stalled = cycle ? (k > 1 && !(cert < 0.99 * best_before_last))
                                   : (k > 0 && !(cert < 0.5 * best));
        best_before_last = best;
        best = std::min(best, cert);
        if (stalled) {
            if (fp64_inner) break;
            // precision schedule: the reduced products have contracted as
            // far as they can; the remaining steps solve on the FP64
            // operator (same restart cycles and sweeps)
            fp64_inner = true;
            Ml = ridge ? static_cast<const DeviceOperator*>(aug_high.get()) : &op;
            best_before_last = __builtin_huge_val();
            best = cert;
        }
        // s_{k+1} = M x_{k+1} - c in FP64 (A x - b, then sqrt(lambda) x)
        Epilogue ep;
        ep.out = res;
        ep.minus_vec = d_b;
        if (!op.product1(false, d_solution, ep, stream)) {
            op.apply(d_solution, 1, res, stream);
            axpy_kernel<<<grid_for(m), 256, 0, stream>>>(res, -1.0, d_b, m, res);
            AMFLS_LAUNCHED();
        }
        if (ridge) {
            AMFLS_CUDA(cudaMemsetAsync(res + m, 0, sizeof(double) * n, stream));
            axpy_kernel<<<grid_for(n), 256, 0, stream>>>(res + m, std::sqrt(reg), d_solution, n,
                                                         res + m);
            AMFLS_LAUNCHED();
        }
    }
    stream_wait(stream);
    out.statistics.total_seconds =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    out.statistics.kernel_launches = launch_count() - launches0;
    return out;
}

}  // namespace amfls_gpu
