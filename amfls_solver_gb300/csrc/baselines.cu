// Scalar LSQR and LSMR over the device operators.
//
// Restates src/algorithms/lsqr/lsqr.cpp:84-281 and
// src/algorithms/lsmr/lsmr.cpp:112-351 (Fong and Saunders 2011, section 5.2,
// damp^2 = regularization): the recurrences run on the host in double, the
// vectors stay on the device (products through the operator, elementwise
// updates and norms as kernels), and every checkpoint of the reference's
// CertificateCheckpointSchedule certifies the current iterate with the
// device validation, exactly where the reference validates.  The norms are
// the scaled two-pass norms that stand in for dnrm2 elsewhere in the
// library, and the vector updates contract to FMAs, so iterates agree with
// the reference's to rounding rather than bit for bit.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <initializer_list>
#include <stdexcept>
#include <utility>
#include <vector>

#include "baselines.hpp"
#include "common.cuh"
#include "solve_common.hpp"
#include "validation.hpp"
#include "vector_ops.hpp"

namespace amfls_gpu {
namespace {

using Clock = std::chrono::steady_clock;

__global__ void combine_kernel(double* out, const double* a, double c, const double* b,
                               long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = a[i] + c * b[i];
}

__global__ void scale_kernel(double* v, double f, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        v[i] *= f;
}

int grid_for(long long n) {
    return (int)std::max<long long>(1, std::min<long long>(grid_cap(), (n + 255) / 256));
}

// Device vectors, elementwise kernels, norms and the search-product
// bookkeeping of one solve, all on one stream.
class Run {
public:
    Run(const DeviceOperator& op, cudaStream_t s) : op_(op), s_(s) {
        stream_alloc(&partials_, sizeof(double) * 2 * kMaxVectors * kMaxGridCap, s_);
        stream_alloc(&counter_, sizeof(unsigned), s_);
        stream_alloc(&norms_, sizeof(NormResult), s_);
        AMFLS_CUDA(cudaMemsetAsync(counter_, 0, sizeof(unsigned), s_));
        for (auto& e : ev_) AMFLS_CUDA(cudaEventCreate(&e));
    }
    ~Run() {
        cudaStreamSynchronize(s_);
        for (double* p : vecs_) stream_free(p, s_);
        stream_free(partials_, s_);
        stream_free(counter_, s_);
        stream_free(norms_, s_);
        for (auto e : ev_) cudaEventDestroy(e);
    }
    Run(const Run&) = delete;
    Run& operator=(const Run&) = delete;

    double* vec(long long n) {
        double* p = nullptr;
        stream_alloc(&p, sizeof(double) * std::max<long long>(1, n), s_);
        vecs_.push_back(p);
        return p;
    }
    void zero(double* v, long long n) {
        AMFLS_CUDA(cudaMemsetAsync(v, 0, sizeof(double) * n, s_));
    }
    void copy(double* dst, const double* src, long long n) {
        AMFLS_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, s_));
    }
    // out = a + c b (out may alias a or b)
    void combine(double* out, const double* a, double c, const double* b, long long n) {
        combine_kernel<<<grid_for(n), 256, 0, s_>>>(out, a, c, b, n);
        AMFLS_LAUNCHED();
    }
    void scale(double* v, double f, long long n) {
        scale_kernel<<<grid_for(n), 256, 0, s_>>>(v, f, n);
        AMFLS_LAUNCHED();
    }
    // Norms and finiteness of up to kMaxVectors vectors (synchronises); the
    // search products enqueued before are timed here.
    NormResult norms(std::initializer_list<std::pair<const double*, long long>> list) {
        VectorSet set{};
        for (const auto& [p, n] : list) {
            set.v[set.count] = p;
            set.n[set.count] = n;
            ++set.count;
        }
        norm_passes(set, norms_, partials_, counter_, s_);
        NormResult h{};
        AMFLS_CUDA(cudaMemcpyAsync(&h, norms_, sizeof(NormResult), cudaMemcpyDeviceToHost, s_));
        stream_wait(s_);
        settle();
        return h;
    }
    // apply_search / apply_transpose_search (lsqr.cpp:20-50)
    void apply(const double* x, double* y) {
        AMFLS_CUDA(cudaEventRecord(ev_[0], s_));
        op_.apply(x, 1, y, s_);
        AMFLS_CUDA(cudaEventRecord(ev_[1], s_));
        pending_a_ = true;
        ++stats.a_columns;
        ++stats.a_block_calls;
        ++stats.search_a_columns;
        ++stats.search_a_block_calls;
    }
    void apply_transpose(const double* y, double* x) {
        AMFLS_CUDA(cudaEventRecord(ev_[2], s_));
        op_.apply_transpose(y, 1, x, s_);
        AMFLS_CUDA(cudaEventRecord(ev_[3], s_));
        pending_at_ = true;
        ++stats.at_columns;
        ++stats.at_block_calls;
        ++stats.search_at_columns;
        ++stats.search_at_block_calls;
    }
    Statistics stats;

private:
    void settle() {
        float ms = 0.0f;
        if (pending_a_) {
            AMFLS_CUDA(cudaEventElapsedTime(&ms, ev_[0], ev_[1]));
            stats.a_seconds += 1e-3 * ms;
            pending_a_ = false;
        }
        if (pending_at_) {
            AMFLS_CUDA(cudaEventElapsedTime(&ms, ev_[2], ev_[3]));
            stats.at_seconds += 1e-3 * ms;
            pending_at_ = false;
        }
    }
    const DeviceOperator& op_;
    cudaStream_t s_;
    double* partials_ = nullptr;
    unsigned* counter_ = nullptr;
    NormResult* norms_ = nullptr;
    std::vector<double*> vecs_;
    cudaEvent_t ev_[4] = {};
    bool pending_a_ = false, pending_at_ = false;
};

// validate_common_inputs (candidate_validation.cpp:570-592) and the
// iteration limit's check; the right-hand side's finiteness is checked with
// its norm.
int check_inputs(const DeviceOperator& op, const double* d_b, const BaselineOptions& o) {
    if (op.rows() <= 0 || op.cols() <= 0)
        throw std::invalid_argument("operator dimensions must be positive");
    if (d_b == nullptr) throw std::invalid_argument("right-hand side cannot be null");
    if (!std::isfinite(o.regularization) || o.regularization < 0.0)
        throw std::invalid_argument("regularization must be finite and nonnegative");
    if (!std::isfinite(o.tolerance) || o.tolerance <= 0.0 || o.tolerance >= 1.0)
        throw std::invalid_argument("tolerance must lie strictly between zero and one");
    if (o.maximum_iterations < 0)
        throw std::invalid_argument("maximum_iterations must be nonnegative");
    return o.maximum_iterations > 0 ? o.maximum_iterations : std::min(op.rows(), op.cols());
}

// The certified candidates of one solve: validate_iterate (lsqr.cpp:59-78)
// with its trace record, and the result at the end.
class Candidates {
public:
    Candidates(const DeviceOperator& op, const double* d_b, const BaselineOptions& o, Run& run,
               cudaStream_t s)
        : validator_(op, d_b, o.regularization, s), sched_(o.regularization, o.tolerance),
          tol_(o.tolerance), run_(run) {
        out_.rows = op.rows();
        out_.cols = op.cols();
    }
    // Certifies d_x as the iterate of `it`; returns its validation.
    const ValidationOutput& evaluate(const double* d_x, int it) {
        v_ = validator_.validate(d_x, tol_);
        account_validation(run_.stats, v_);
        sched_.record(it, v_);
        TraceRow row;
        fill_trace_row(row, v_, run_.stats, 0, it, 0, it);
        out_.trace.push_back(row);
        it_ = it;
        status_ = v_.status;
        reason_ = v_.stop_reason;
        return v_;
    }
    bool should_evaluate(int it) const { return sched_.should_evaluate(it); }
    bool failed() const { return failed_numerically(v_); }
    bool success() const { return status_ == 0; }
    void set_outcome(int status, int reason) {
        status_ = status;
        reason_ = reason;
    }
    SolveResult finish(const double* d_x, double* d_solution, Clock::time_point t0,
                       long long launches0, cudaStream_t s) {
        out_.iterations = out_.depth = out_.basis_rank = it_;
        out_.auxiliary_width = 0;
        out_.v = v_;
        out_.status = status_;
        out_.stop_reason = reason_;
        AMFLS_CUDA(cudaMemcpyAsync(d_solution, d_x, sizeof(double) * out_.cols,
                                   cudaMemcpyDeviceToDevice, s));
        stream_wait(s);
        run_.stats.total_seconds = std::chrono::duration<double>(Clock::now() - t0).count();
        run_.stats.kernel_launches = launch_count() - launches0;
        out_.statistics = run_.stats;
        return std::move(out_);
    }

private:
    Validator validator_;
    CheckpointSchedule sched_;
    double tol_;
    Run& run_;
    SolveResult out_;
    ValidationOutput v_{};
    int it_ = 0, status_ = 1, reason_ = 3;
};

bool finite_all(std::initializer_list<double> values) {
    for (double v : values)
        if (!std::isfinite(v)) return false;
    return true;
}

// symmetric_givens (lsmr.cpp:17-27)
struct Givens {
    double c, s, r;
};
Givens givens(double a, double b) {
    const double r = std::hypot(a, b);
    if (r == 0.0) return {1.0, 0.0, 0.0};
    return {a / r, b / r, r};
}

}  // namespace

SolveResult solve_lsqr(const DeviceOperator& op, const double* d_b, const BaselineOptions& o,
                       double* d_solution, cudaStream_t stream) {
    const int max_it = check_inputs(op, d_b, o);
    const auto t0 = Clock::now();
    const long long launches0 = launch_count();
    const long long m = op.rows(), n = op.cols();
    Run run(op, stream);
    double* u = run.vec(m);
    double* av = run.vec(m);
    double* v = run.vec(n);
    double* atu = run.vec(n);
    double* w = run.vec(n);
    double* x = run.vec(n);

    run.copy(u, d_b, m);
    NormResult nr = run.norms({{u, m}});
    if (nr.nonfinite[0]) throw std::invalid_argument("right-hand side must be finite");
    double beta = euclid_from(nr, 0);
    run.zero(x, n);
    if (beta > 0.0) run.scale(u, 1.0 / beta, m);
    run.apply_transpose(u, v);
    double alpha = euclid_from(run.norms({{v, n}}), 0);
    if (alpha > 0.0) run.scale(v, 1.0 / alpha, n);
    run.copy(w, v, n);
    double rhobar = alpha, phibar = beta;
    const double damp = std::sqrt(o.regularization);
    Candidates cand(op, d_b, o, run, stream);

    if (!std::isfinite(beta) || !std::isfinite(alpha) || alpha == 0.0) {
        cand.evaluate(x, 0);
        if (cand.failed() || cand.success() || alpha == 0.0)
            return cand.finish(x, d_solution, t0, launches0, stream);
    }
    for (int it = 1; it <= max_it; ++it) {
        run.apply(v, av);
        run.combine(av, av, -alpha, u, m);
        beta = euclid_from(run.norms({{av, m}}), 0);
        if (beta > 0.0) run.scale(av, 1.0 / beta, m);

        // x_k needs beta_{k+1} only: it is formed (and certified at a
        // checkpoint) before the transpose half-step
        const double rhobar1 = std::hypot(rhobar, damp);
        const double cs1 = rhobar1 == 0.0 ? 1.0 : rhobar / rhobar1;
        phibar *= cs1;
        const double rho = std::hypot(rhobar1, beta);
        const double cs = rho == 0.0 ? 1.0 : rhobar1 / rho;
        const double sn = rho == 0.0 ? 0.0 : beta / rho;
        const double phi = cs * phibar;
        phibar = sn * phibar;
        bool finite = finite_all({beta, rhobar1, cs1, rho, cs, sn, phi, phibar});
        if (rho != 0.0) {
            const double update = phi / rho;
            finite = finite && std::isfinite(update);
            run.combine(x, x, update, w, n);
        }
        finite = finite && run.norms({{x, n}}).nonfinite[0] == 0;
        std::swap(u, av);

        const bool breakdown = beta == 0.0;
        bool evaluated = false;
        if (cand.should_evaluate(it) || breakdown || !finite || it == max_it) {
            cand.evaluate(x, it);
            evaluated = true;
            if (cand.failed() || cand.success()) break;
            if (!finite) {
                cand.set_outcome(4, 7);
                break;
            }
            if (breakdown) {
                cand.set_outcome(1, 2);
                break;
            }
            if (it == max_it) {
                cand.set_outcome(1, 3);
                break;
            }
        }

        run.apply_transpose(u, atu);
        run.combine(atu, atu, -beta, v, n);
        const NormResult na = run.norms({{atu, n}});
        const double next_alpha = euclid_from(na, 0);
        bool cont = std::isfinite(next_alpha) && na.nonfinite[0] == 0;
        if (next_alpha > 0.0 && std::isfinite(next_alpha)) run.scale(atu, 1.0 / next_alpha, n);
        const double theta = sn * next_alpha;
        const double next_rhobar = -cs * next_alpha;
        const double recurrence = theta / rho;
        cont = cont && finite_all({theta, next_rhobar, recurrence});
        if (cont && next_alpha > 0.0) {
            run.combine(w, atu, -recurrence, w, n);
            cont = run.norms({{w, n}}).nonfinite[0] == 0;
        }
        if (!cont || next_alpha == 0.0) {
            if (!evaluated) {
                cand.evaluate(x, it);
                if (cand.failed() || cand.success()) break;
            }
            cand.set_outcome(cont ? 1 : 4, cont ? 2 : 7);
            break;
        }
        alpha = next_alpha;
        rhobar = next_rhobar;
        std::swap(v, atu);
    }
    return cand.finish(x, d_solution, t0, launches0, stream);
}

SolveResult solve_lsmr(const DeviceOperator& op, const double* d_b, const BaselineOptions& o,
                       double* d_solution, cudaStream_t stream) {
    const int max_it = check_inputs(op, d_b, o);
    const auto t0 = Clock::now();
    const long long launches0 = launch_count();
    const long long m = op.rows(), n = op.cols();
    Run run(op, stream);
    double* u = run.vec(m);
    double* av = run.vec(m);
    double* v = run.vec(n);
    double* atu = run.vec(n);
    double* x = run.vec(n);
    double* h = run.vec(n);
    double* hbar = run.vec(n);
    double* nx = run.vec(n);
    double* nh = run.vec(n);
    double* nhbar = run.vec(n);

    run.copy(u, d_b, m);
    NormResult nr = run.norms({{u, m}});
    if (nr.nonfinite[0]) throw std::invalid_argument("right-hand side must be finite");
    double beta = euclid_from(nr, 0);
    if (beta > 0.0 && std::isfinite(beta)) run.scale(u, 1.0 / beta, m);
    run.apply_transpose(u, v);
    double alpha = euclid_from(run.norms({{v, n}}), 0);
    if (alpha > 0.0 && std::isfinite(alpha)) run.scale(v, 1.0 / alpha, n);
    run.zero(x, n);
    run.copy(h, v, n);
    run.zero(hbar, n);
    double alphabar = alpha, zetabar = alpha * beta;
    double rho = 1.0, rhobar = 1.0, cbar = 1.0, sbar = 0.0;
    const double damp = std::sqrt(o.regularization);
    Candidates cand(op, d_b, o, run, stream);

    bool initial_breakdown = !std::isfinite(beta) || !std::isfinite(alpha);
    if (initial_breakdown || alpha == 0.0) {
        cand.evaluate(x, 0);
        initial_breakdown = initial_breakdown || cand.failed();
        if (initial_breakdown)
            cand.set_outcome(4, 7);
        else if (alpha == 0.0 && !cand.success())
            cand.set_outcome(1, 2);
        if (cand.success() || initial_breakdown || alpha == 0.0)
            return cand.finish(x, d_solution, t0, launches0, stream);
    }
    for (int it = 1; it <= max_it; ++it) {
        run.apply(v, av);
        bool valid = run.norms({{av, m}}).nonfinite[0] == 0;
        run.combine(av, av, -alpha, u, m);
        beta = euclid_from(run.norms({{av, m}}), 0);
        valid = valid && std::isfinite(beta);
        if (beta > 0.0 && std::isfinite(beta)) run.scale(av, 1.0 / beta, m);
        // at an exact beta breakdown A^T u_{k+1} = 0 without a product
        if (beta == 0.0) {
            run.zero(atu, n);
            alpha = 0.0;
        } else {
            run.apply_transpose(av, atu);
            run.combine(atu, atu, -beta, v, n);
            alpha = euclid_from(run.norms({{atu, n}}), 0);
            valid = valid && std::isfinite(alpha);
            if (alpha > 0.0 && std::isfinite(alpha)) run.scale(atu, 1.0 / alpha, n);
        }

        // damping, bidiagonal QR and MINRES rotations in the order of
        // Fong and Saunders' section 5.2
        const Givens damping = givens(alphabar, damp);
        const double rho_old = rho;
        const Givens bidiagonal = givens(damping.r, beta);
        rho = bidiagonal.r;
        const double theta_new = bidiagonal.s * alpha;
        alphabar = bidiagonal.c * alpha;
        const double rhobar_old = rhobar;
        const double theta_bar = sbar * rho;
        const double rho_temp = cbar * rho;
        const Givens minres = givens(rho_temp, theta_new);
        cbar = minres.c;
        sbar = minres.s;
        rhobar = minres.r;
        const double zeta = cbar * zetabar;
        zetabar = -sbar * zetabar;
        const double hbar_den = rho_old * rhobar_old;
        const double sol_den = rho * rhobar;
        valid = valid &&
                finite_all({damping.c, damping.s, damping.r, bidiagonal.c, bidiagonal.s, rho,
                            theta_new, alphabar, theta_bar, rho_temp, minres.c, minres.s, rhobar,
                            zeta, zetabar, hbar_den, sol_den}) &&
                hbar_den != 0.0 && sol_den != 0.0 && rho != 0.0;
        if (valid) {
            const double hbar_rec = theta_bar * rho / hbar_den;
            const double sol_update = zeta / sol_den;
            const double h_rec = theta_new / rho;
            valid = finite_all({hbar_rec, sol_update, h_rec});
            run.combine(nhbar, h, -hbar_rec, hbar, n);
            run.combine(nx, x, sol_update, nhbar, n);
            run.combine(nh, atu, -h_rec, h, n);
            const NormResult nn = run.norms({{nhbar, n}, {nx, n}, {nh, n}});
            valid = valid && nn.nonfinite[0] == 0 && nn.nonfinite[1] == 0 && nn.nonfinite[2] == 0;
            if (valid) {
                std::swap(hbar, nhbar);
                std::swap(x, nx);
                std::swap(h, nh);
            }
        }
        std::swap(u, av);
        std::swap(v, atu);

        const bool exact = alpha == 0.0 || beta == 0.0;
        if (!(cand.should_evaluate(it) || !valid || exact || it == max_it)) continue;
        // the baseline protocol recomputes both residuals (no recurrence estimates)
        cand.evaluate(x, it);
        if (cand.failed()) break;
        if (!valid) {
            cand.set_outcome(4, 7);
            break;
        }
        if (cand.success()) break;
        if (exact) {
            cand.set_outcome(1, 2);
            break;
        }
        if (it == max_it) cand.set_outcome(1, 3);
    }
    return cand.finish(x, d_solution, t0, launches0, stream);
}

}  // namespace amfls_gpu
