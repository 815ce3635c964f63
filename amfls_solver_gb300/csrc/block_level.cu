// Block (width > 1) levels of the device block Golub-Kahan workspace.
//
// Restates, with device kernels for every O(rows) operation and host
// decisions on small matrices:
//   orthogonalize_and_factor  krylov_workspace.cpp:82-310
//   append_left_seed          krylov_workspace.cpp:505-587
//   advance_level             krylov_workspace.cpp:589-831
// A block level synchronises with the host a few times (rank decisions on
// the singular values of each residual block).  The first time a block
// appears, the width-one history (alpha, beta, g on the device) is turned
// into level records, and from then on the projected operator T is kept as
// records: per level G (aw x r, rows of the previous left block), N
// (nlw x r, rows of the new left block) and g (the new rows' U^T b).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <vector>

#include "block.hpp"
#include "common.cuh"
#include "workspace.hpp"

namespace amfls_gpu {
namespace {

constexpr double kEps = std::numeric_limits<double>::epsilon();
constexpr double kInf = std::numeric_limits<double>::infinity();

// krylov_workspace.cpp:63-80
double rank_revealing_cutoff(double scale, int rows, int cols, int basis_cols, int block_cols) {
    if (!(scale >= 0.0) || !std::isfinite(scale)) return kInf;
    const int dim = std::max({1, rows, cols, basis_cols, block_cols});
    return 64.0 * kEps * dim * scale;
}

// krylov_workspace.cpp:965-979
bool truncated_or_broken(const StepAudit& a) {
    const bool truncation =
        (a.right_rank_loss && a.right_positive_finite_below_cutoff &&
         a.right_active_discarded_residual_norm > 0.0) ||
        (a.left_rank_loss && a.left_positive_finite_below_cutoff);
    return truncation || a.right_nonfinite_residual || a.left_nonfinite_residual;
}

// Grow a device buffer to hold `need` elements; `keep` elements of the old
// contents survive (copy and free are ordered on the stream).
template <typename T>
void grow(T*& p, long long& cap, long long need, long long keep, cudaStream_t s) {
    if (need <= cap) return;
    long long c = std::max<long long>(need, cap + cap / 2);
    T* q = nullptr;
    stream_alloc(&q, sizeof(T) * c, s);
    if (p) {
        if (keep > 0)
            AMFLS_CUDA(cudaMemcpyAsync(q, p, sizeof(T) * std::min(keep, cap),
                                       cudaMemcpyDeviceToDevice, s));
        stream_free(p, s);
    }
    p = q;
    cap = c;
}

}  // namespace

void Workspace::push_state() {
    AMFLS_CUDA(cudaMemcpyAsync(dstate_, &host_, sizeof(DevState), cudaMemcpyHostToDevice, stream_));
    stream_wait(stream_);
}

void Workspace::upload(double* dst, const std::vector<double>& src) {
    if (src.empty()) return;
    AMFLS_CUDA(cudaMemcpyAsync(dst, src.data(), sizeof(double) * src.size(),
                               cudaMemcpyHostToDevice, stream_));
    // the host vector may die right after: make the copy complete
    stream_wait(stream_);
}

double Workspace::device_norm(const double* x, long long count) {
    if (count <= 0) return 0.0;
    VectorSet set{};
    set.v[0] = x;
    set.n[0] = count;
    set.count = 1;
    norm_passes(set, dnorm_, partials_, counter_ + 1, stream_);
    NormResult h{};
    AMFLS_CUDA(cudaMemcpyAsync(&h, dnorm_, sizeof(NormResult), cudaMemcpyDeviceToHost, stream_));
    stream_wait(stream_);
    return euclid_from(h, 0);
}

double Workspace::timed_apply(bool transpose, const double* in, int cols, double* out) {
    AMFLS_CUDA(cudaEventRecord(ev_[0], stream_));
    if (transpose) op_.apply_transpose(in, cols, out, stream_);
    else op_.apply(in, cols, out, stream_);
    AMFLS_CUDA(cudaEventRecord(ev_[1], stream_));
    AMFLS_CUDA(cudaEventSynchronize(ev_[1]));
    float ms = 0.0f;
    AMFLS_CUDA(cudaEventElapsedTime(&ms, ev_[0], ev_[1]));
    return static_cast<double>(ms) * 1e-3;
}

void Workspace::ensure_u_capacity(int cols) {
    if (cols <= ucap_ && U2_ != nullptr) return;
    const int cap = std::max({cols, 2 * ucap_, 4});
    const long long keep = (long long)m_ * (host_.left_width + host_.pending);
    double* u = nullptr;
    double* u2 = nullptr;
    stream_alloc(&u, sizeof(double) * m_ * (size_t)cap, stream_);
    stream_alloc(&u2, sizeof(double) * m_ * (size_t)cap, stream_);
    if (keep > 0)
        AMFLS_CUDA(cudaMemcpyAsync(u, U_, sizeof(double) * keep, cudaMemcpyDeviceToDevice, stream_));
    stream_wait(stream_);
    stream_free(U_, stream_);
    stream_free(U2_, stream_);
    U_ = u;
    U2_ = u2;
    ucap_ = cap;
    invalidate_graph();  // captured width-one kernels hold the old U
}

void Workspace::ensure_block_capacity(int width) {
    if (width > bcap_) {
        const int cap = std::max(width, 2 * bcap_);
        stream_wait(stream_);
        for (double** p : {&BR_, &BL_, &BQ_, &BT_}) {
            stream_free(*p, stream_);
            *p = nullptr;
        }
        const size_t rows_max = std::max(m_, n_);
        stream_alloc(&BR_, sizeof(double) * n_ * (size_t)cap, stream_);
        stream_alloc(&BL_, sizeof(double) * m_ * (size_t)cap, stream_);
        stream_alloc(&BQ_, sizeof(double) * n_ * (size_t)cap, stream_);
        stream_alloc(&BT_, sizeof(double) * rows_max * (size_t)cap, stream_);
        bcap_ = cap;
    }
    const long long c = std::max(width, 1);
    grow(small_, small_cap_, 10 * c * c + 8 * c + jacobi_work_doubles((int)c) + 256, 0, stream_);
    if (!dflags_) {
        stream_alloc(&dflags_, sizeof(int) * 8, stream_);
        AMFLS_CUDA(cudaMemsetAsync(dflags_, 0, sizeof(int) * 8, stream_));
    }
    if (!dnorm_) stream_alloc(&dnorm_, sizeof(NormResult), stream_);
    if (!ev_[0]) {
        AMFLS_CUDA(cudaEventCreate(&ev_[0]));
        AMFLS_CUDA(cudaEventCreate(&ev_[1]));
    }
}

void Workspace::enter_block_mode() {
    if (block_mode_) return;
    sync();
    ensure_block_capacity(1);
    const int k = host_.k;
    if (host_.depth != k) throw std::logic_error("width-one history is inconsistent");
    if (k > 0) {
        std::vector<double> al(k), be(k), g(std::max(1, host_.rows_t));
        AMFLS_CUDA(cudaMemcpyAsync(al.data(), alpha_, sizeof(double) * k, cudaMemcpyDeviceToHost, stream_));
        AMFLS_CUDA(cudaMemcpyAsync(be.data(), beta_, sizeof(double) * k, cudaMemcpyDeviceToHost, stream_));
        AMFLS_CUDA(cudaMemcpyAsync(g.data(), g_, sizeof(double) * host_.rows_t, cudaMemcpyDeviceToHost,
                                   stream_));
        stream_wait(stream_);
        for (int j = 0; j < k; ++j) {
            const int nlw = be[j] != 0.0 ? 1 : 0;
            rec_meta_.insert(rec_meta_.end(), {1, 1, nlw, (int)rec_vals_.size(), (int)rec_state_size_});
            rec_vals_.push_back(al[j]);
            if (nlw) {
                rec_vals_.push_back(be[j]);
                rec_vals_.push_back(g[j + 1]);
            }
            rec_state_size_ += level_state_doubles(1, nlw, rec_last_r_);
            rec_last_r_ = 1;
        }
    }
    coupling_.clear();
    if (host_.left_width > 0 && host_.prev_right_width > 0) coupling_.push_back(host_.coupling);
    block_mode_ = true;
}

Workspace::Factor Workspace::orthogonalize_and_factor(double* B, int cols, const Basis& basis,
                                                      int max_rank, double scale, int tracked,
                                                      bool retain, double* q_out) {
    const long long rows = basis.panels ? n_ : m_;
    const int kb = basis.cols;
    Factor F;
    if (retain) F.coefficients.assign((size_t)kb * cols, 0.0);
    double resid = 0.0;
    bool coeff_finite = true;
    int passes = 0;
    double* C[2] = {nullptr, nullptr};
    if (kb > 0 && cols > 0) {
        grow(coefs_, coefs_cap_, 2LL * kb * cols, 0, stream_);
        C[0] = coefs_;
        C[1] = coefs_ + (long long)kb * cols;
        const long long part = basis.panels ? panel_tn_partial_doubles(n_, kb, cols)
                                            : ts_tn_partial_doubles(m_, kb, cols);
        grow(bpart_, bpart_cap_, part, 0, stream_);
        AMFLS_CUDA(cudaMemsetAsync(dflags_, 0, sizeof(int), stream_));
    }
    auto project = [&](double* c) {  // c = basis^T B; B -= basis c
        if (basis.panels) {
            panel_tn(V_->device_table(), n_, kb, B, rows, cols, c, bpart_, dflags_, stream_);
            panel_nn(V_->device_table(), n_, 0, kb, c, cols, B, rows, -1.0, stream_);
        } else {
            ts_tn(basis.mat, m_, B, m_, m_, kb, cols, c, bpart_, dflags_, stream_);
            ts_nn(basis.mat, m_, c, m_, kb, cols, B, m_, -1.0, 1.0, stream_);
        }
        ++passes;
    };
    if (cols == 1 && kb > 0) {
        // scalar DGKS (krylov_workspace.cpp:110-170)
        const double before = device_norm(B, rows);
        project(C[0]);
        resid = device_norm(B, rows);
        if (std::isfinite(before) && std::isfinite(resid) && resid < std::sqrt(0.5) * before) {
            project(C[1]);
            resid = device_norm(B, rows);
        }
    } else {
        // block CGS2 (krylov_workspace.cpp:172-195)
        if (kb > 0) {
            project(C[0]);
            project(C[1]);
        }
        resid = device_norm(B, rows * cols);
    }
    if (passes > 0) {
        int nf = 0;
        AMFLS_CUDA(cudaMemcpyAsync(&nf, dflags_, sizeof(int), cudaMemcpyDeviceToHost, stream_));
        std::vector<double> h;
        if (retain) h.resize((size_t)passes * kb * cols);
        if (retain)
            AMFLS_CUDA(cudaMemcpyAsync(h.data(), coefs_, sizeof(double) * h.size(),
                                       cudaMemcpyDeviceToHost, stream_));
        stream_wait(stream_);
        coeff_finite = nf == 0;
        if (retain) {
            const size_t cnt = (size_t)kb * cols;
            for (int p = 0; p < passes; ++p)
                for (size_t i = 0; i < cnt; ++i) F.coefficients[i] += h[p * cnt + i];
            for (double v : F.coefficients)
                if (!std::isfinite(v)) coeff_finite = false;
        }
    }
    F.cutoff = rank_revealing_cutoff(scale, m_, n_, kb, cols);
    const bool finite = std::isfinite(scale) && std::isfinite(resid) && coeff_finite;
    if (!finite) {
        F.nonfinite = true;
        F.discarded = kInf;
        F.tracked = tracked > 0 ? kInf : 0.0;
        return F;
    }
    if (max_rank == 0 || cols == 0) {
        if (tracked > 0) F.tracked = device_norm(B, rows * tracked);
        return F;
    }
    double* sm = small_;
    if (cols == 1) {
        if (resid > F.cutoff) {
            const double inv = 1.0 / resid;
            AMFLS_CUDA(cudaMemcpyAsync(sm, &inv, sizeof(double), cudaMemcpyHostToDevice, stream_));
            ts_nn(B, rows, sm, rows, 1, 1, q_out, rows, 1.0, 0.0, stream_);
            stream_wait(stream_);
            F.rank = 1;
            F.factor = {resid};
        } else if (resid > 0.0 && resid <= F.cutoff) {
            F.positive_below = true;
            if (tracked == 1) F.tracked = resid;
        }
        return F;
    }
    // rank-revealing SVD of the residual block (krylov_workspace.cpp:263-307)
    const long long cc = (long long)cols * cols;
    double* Rf = sm;
    double* sig = Rf + cc;
    double* W = sig + cols;
    double* jw = W + cc;
    grow(tsqr_, tsqr_cap_, tsqr_work_doubles(rows, cols), 0, stream_);
    tsqr_r(B, rows, cols, rows, Rf, tsqr_, stream_);
    jacobi_svd(Rf, cols, sig, W, jw, stream_);
    std::vector<double> hs(cols), hw(cc);
    AMFLS_CUDA(cudaMemcpyAsync(hs.data(), sig, sizeof(double) * cols, cudaMemcpyDeviceToHost, stream_));
    AMFLS_CUDA(cudaMemcpyAsync(hw.data(), W, sizeof(double) * cc, cudaMemcpyDeviceToHost, stream_));
    stream_wait(stream_);
    // a rows x cols block has min(rows, cols) singular values
    const int nsv = (int)std::min<long long>(rows, cols);
    int rank = 0;
    while (rank < nsv && rank < max_rank && std::isfinite(hs[rank]) && hs[rank] > F.cutoff) ++rank;
    if (rank < nsv && rank < max_rank) {
        const double first = hs[rank];
        F.positive_below = std::isfinite(first) && first > 0.0 && first <= F.cutoff;
    }
    if (rank > 0) {
        // q = B W_r Sigma_r^{-1}, then one Cholesky QR pass
        std::vector<double> M((size_t)cols * rank);
        for (int j = 0; j < rank; ++j)
            for (int i = 0; i < cols; ++i) M[i + (size_t)j * cols] = hw[i + (size_t)j * cols] / hs[j];
        double* dM = jw;  // the Jacobi scratch is free again
        double* dG = dM + (long long)cols * rank;
        double* dU = dG + (long long)rank * rank;
        double* dUi = dU + (long long)rank * rank;
        upload(dM, M);
        ts_nn(B, rows, dM, rows, cols, rank, BT_, rows, 1.0, 0.0, stream_);
        grow(bpart_, bpart_cap_, ts_tn_partial_doubles(rows, rank, rank), 0, stream_);
        ts_tn(BT_, rows, BT_, rows, rows, rank, rank, dG, bpart_, nullptr, stream_);
        cholesky_upper(dG, rank, dU, dUi, dflags_ + 1, stream_);
        std::vector<double> hu((size_t)rank * rank);
        int chol_bad = 0;
        AMFLS_CUDA(cudaMemcpyAsync(hu.data(), dU, sizeof(double) * hu.size(), cudaMemcpyDeviceToHost,
                                   stream_));
        AMFLS_CUDA(cudaMemcpyAsync(&chol_bad, dflags_ + 1, sizeof(int), cudaMemcpyDeviceToHost,
                                   stream_));
        stream_wait(stream_);
        if (chol_bad) {
            // keep q = B W_r Sigma_r^{-1} as it is (U = I)
            AMFLS_CUDA(cudaMemcpyAsync(q_out, BT_, sizeof(double) * rows * rank,
                                       cudaMemcpyDeviceToDevice, stream_));
            std::fill(hu.begin(), hu.end(), 0.0);
            for (int i = 0; i < rank; ++i) hu[i + (size_t)i * rank] = 1.0;
        } else {
            ts_nn(BT_, rows, dUi, rows, rank, rank, q_out, rows, 1.0, 0.0, stream_);
        }
        // factor = U Sigma_r W_r^T (rank x cols)
        F.factor.assign((size_t)rank * cols, 0.0);
        for (int c = 0; c < cols; ++c)
            for (int i = 0; i < rank; ++i) {
                double s = 0.0;
                for (int l = i; l < rank; ++l)
                    s += hu[i + (size_t)l * rank] * hs[l] * hw[c + (size_t)l * cols];
                F.factor[i + (size_t)c * rank] = s;
            }
        F.rank = rank;
    }
    for (int idx = rank; idx < nsv; ++idx) {
        F.discarded = std::hypot(F.discarded, hs[idx]);
        double weight = 0.0;
        for (int c = 0; c < tracked; ++c) weight = std::hypot(weight, hw[c + (size_t)idx * cols]);
        F.tracked = std::hypot(F.tracked, hs[idx] * weight);
    }
    stream_wait(stream_);
    return F;
}

int Workspace::append_left_seed(const double* d_seed, int cols) {
    if (!initialized_) throw std::logic_error("block Golub-Kahan workspace is not initialized");
    if (cols < 0) throw std::invalid_argument("injected left block has a negative width");
    if (cols > 0 && d_seed == nullptr) throw std::invalid_argument("injected left block is null");
    sync();
    if (!host_.reliable)
        throw std::logic_error("cannot continue block Golub-Kahan after numerical truncation");
    enter_block_mode();
    if (pending_requested_ == 0 && host_.pending == 0) std::memset(&host_.audit, 0, sizeof(StepAudit));
    if (cols > std::numeric_limits<int>::max() - pending_requested_)
        throw std::overflow_error("pending block Golub-Kahan width exceeds LP64 limits");
    pending_requested_ += cols;
    host_.audit.requested_injected_columns = pending_requested_;
    host_.audit.retained_injected_columns = pending_retained_;
    if (cols == 0) {
        push_state();
        return 0;
    }
    const int lw = host_.left_width, p = host_.pending;
    const int available = std::max(0, basis_limit_ - host_.k - lw - p);
    const int max_rank = std::min({available, m_ - lw - p, cols});
    if (max_rank <= 0) {
        push_state();
        return 0;
    }
    ensure_block_capacity(cols);
    ensure_u_capacity(lw + p + max_rank);
    AMFLS_CUDA(cudaMemcpyAsync(BL_, d_seed, sizeof(double) * m_ * (size_t)cols,
                               cudaMemcpyDeviceToDevice, stream_));
    const double scale = device_norm(BL_, (long long)m_ * cols);
    const Factor F = orthogonalize_and_factor(BL_, cols, Basis{false, U_, lw + p}, max_rank, scale, 0,
                                              false, U_ + (size_t)m_ * (lw + p));
    if (F.rank > 0) {
        host_.pending += F.rank;
        pending_retained_ += F.rank;
        host_.audit.retained_injected_columns = pending_retained_;
    }
    push_state();
    return F.rank;
}

bool Workspace::block_level() {
    StepAudit a;
    std::memset(&a, 0, sizeof(a));
    a.requested_injected_columns = pending_requested_;
    a.retained_injected_columns = pending_retained_;
    a.basis_rank_before = host_.k;
    a.basis_rank_after = host_.k;
    a.left_input_width = host_.left_width + host_.pending;
    host_.audit = a;
    host_.level_ok = 0;
    if (!can_advance()) {
        push_state();
        return false;
    }
    if (host_.rows_t != host_.active_first + host_.left_width)
        throw std::logic_error("block Golub-Kahan active left frontier is inconsistent");
    const int aw = host_.left_width, cw = aw + host_.pending;
    const int old_right = host_.k, old_left = host_.rows_t;
    ensure_block_capacity(cw);
    ensure_u_capacity(cw);

    // right half-step: A^T [U P] - V_prev coupling^T, projected off V
    const double t_at = timed_apply(true, U_, cw, BR_);
    host_.at_ns += static_cast<unsigned long long>(t_at * 1e9);
    host_.search_at_calls += 1;
    host_.search_at_columns += cw;
    host_.pending = 0;
    pending_requested_ = 0;
    pending_retained_ = 0;
    const double right_scale = device_norm(BR_, (long long)n_ * cw);
    if (host_.prev_right_width > 0 && aw > 0) {
        const int pw = host_.prev_right_width;
        if (coupling_.size() != (size_t)aw * pw)
            throw std::logic_error("block Golub-Kahan frontier coupling dimensions are invalid");
        std::vector<double> ct((size_t)pw * aw);
        for (int j = 0; j < aw; ++j)
            for (int l = 0; l < pw; ++l) ct[l + (size_t)j * pw] = coupling_[j + (size_t)l * aw];
        upload(small_, ct);
        panel_nn(V_->device_table(), n_, host_.prev_right_first, pw, small_, aw, BR_, n_, -1.0,
                 stream_);
    }
    const int max_right = std::min(cw, basis_limit_ - host_.k);
    V_->ensure_columns(host_.k + std::max(1, max_right));
    const Factor F = orthogonalize_and_factor(BR_, cw, Basis{true, nullptr, host_.k}, max_right,
                                              right_scale, aw, false, BQ_);
    StepAudit& au = host_.audit;
    au.retained_right_width = F.rank;
    au.right_rank_cutoff = F.cutoff;
    au.right_discarded_residual_norm = F.discarded;
    au.right_active_discarded_residual_norm = F.tracked;
    au.right_positive_finite_below_cutoff = F.positive_below;
    au.right_nonfinite_residual = F.nonfinite;
    au.right_rank_loss = F.rank < max_right;
    au.right_basis_cap_truncation = max_right < cw;
    if (truncated_or_broken(au)) host_.reliable = 0;
    const int r = F.rank;
    if (r == 0) {
        host_.left_width = 0;
        host_.active_first = old_left;
        host_.prev_right_first = host_.k;
        host_.prev_right_width = 0;
        coupling_.clear();
        push_state();
        return false;
    }

    // left half-step: A q - U Fa^T, projected off U
    const double t_a = timed_apply(false, BQ_, r, BL_);
    host_.a_ns += static_cast<unsigned long long>(t_a * 1e9);
    host_.search_a_calls += 1;
    host_.search_a_columns += r;
    const double left_scale = device_norm(BL_, (long long)m_ * r);
    if (aw > 0) {
        std::vector<double> ct((size_t)aw * r);  // Fa^T, Fa = factor[:, :aw]
        for (int i = 0; i < aw; ++i)
            for (int c = 0; c < r; ++c) ct[i + (size_t)c * aw] = F.factor[c + (size_t)i * r];
        upload(small_, ct);
        ts_nn(U_, m_, small_, m_, aw, r, BL_, m_, -1.0, 1.0, stream_);
    }
    const int max_left = std::min({r, m_ - old_left, basis_limit_ + 1 - old_left});
    const Factor FL = orthogonalize_and_factor(BL_, r, Basis{false, U_, aw}, max_left, left_scale, 0,
                                               true, U2_);
    au.retained_next_left_width = FL.rank;
    au.left_rank_cutoff = FL.cutoff;
    au.left_discarded_residual_norm = FL.discarded;
    au.left_positive_finite_below_cutoff = FL.positive_below;
    au.left_nonfinite_residual = FL.nonfinite;
    au.left_rank_loss = FL.rank < max_left;
    au.left_basis_cap_truncation = max_left < r;
    if (truncated_or_broken(au)) host_.reliable = 0;
    if (FL.nonfinite) {  // V, T, g and depth stay at the previous level
        push_state();
        return false;
    }
    const int nlw = FL.rank;
    panel_append(V_->device_table(), n_, host_.k, BQ_, r, stream_);
    host_.k += r;

    // level record: G = Fa^T + left coefficients, N = left factor, g = q^T b
    std::vector<double> gnew(nlw);
    if (nlw > 0) {
        grow(bpart_, bpart_cap_, ts_tn_partial_doubles(m_, nlw, 1), 0, stream_);
        ts_tn(U2_, m_, b_, m_, m_, nlw, 1, small_, bpart_, nullptr, stream_);
        AMFLS_CUDA(cudaMemcpyAsync(gnew.data(), small_, sizeof(double) * nlw, cudaMemcpyDeviceToHost,
                                   stream_));
        stream_wait(stream_);
    }
    rec_meta_.insert(rec_meta_.end(), {r, aw, nlw, (int)rec_vals_.size(), (int)rec_state_size_});
    for (int c = 0; c < r; ++c)
        for (int i = 0; i < aw; ++i) {
            const double coef = FL.coefficients.empty() ? 0.0 : FL.coefficients[i + (size_t)c * aw];
            rec_vals_.push_back(F.factor[c + (size_t)i * r] + coef);
        }
    rec_vals_.insert(rec_vals_.end(), FL.factor.begin(), FL.factor.end());
    rec_vals_.insert(rec_vals_.end(), gnew.begin(), gnew.end());
    rec_state_size_ += level_state_doubles(r, nlw, rec_last_r_);
    rec_last_r_ = r;
    rec_width_ = std::max({rec_width_, r, aw, nlw});

    std::swap(U_, U2_);
    host_.left_width = nlw;
    host_.active_first = old_left;
    host_.rows_t = old_left + nlw;
    host_.prev_right_first = old_right;
    host_.prev_right_width = r;
    coupling_ = FL.factor;
    host_.depth += 1;
    host_.level_ok = 1;
    host_.levels_run += 1;
    au.basis_rank_after = host_.k;
    push_state();
    return true;
}

const double* Workspace::block_projected_y(int* flags) {
    const int levels = static_cast<int>(rec_meta_.size() / kLevelMeta);
    const int k = host_.k;
    // records are append-only: upload the new tail
    const long long nmeta = (long long)rec_meta_.size();
    const long long nvals = (long long)rec_vals_.size();
    if (nmeta > d_meta_cap_) {
        grow(d_meta_, d_meta_cap_, nmeta, 0, stream_);
        d_meta_uploaded_ = 0;
    }
    if (nvals > d_vals_cap_) {
        grow(d_vals_, d_vals_cap_, nvals, 0, stream_);
        d_vals_uploaded_ = 0;
    }
    if (nmeta > d_meta_uploaded_)
        AMFLS_CUDA(cudaMemcpyAsync(d_meta_ + d_meta_uploaded_, rec_meta_.data() + d_meta_uploaded_,
                                   sizeof(int) * (nmeta - d_meta_uploaded_), cudaMemcpyHostToDevice,
                                   stream_));
    if (nvals > d_vals_uploaded_)
        AMFLS_CUDA(cudaMemcpyAsync(d_vals_ + d_vals_uploaded_, rec_vals_.data() + d_vals_uploaded_,
                                   sizeof(double) * (nvals - d_vals_uploaded_),
                                   cudaMemcpyHostToDevice, stream_));
    d_meta_uploaded_ = (int)nmeta;
    d_vals_uploaded_ = nvals;
    // the state and carry of levels already reduced are kept (copied on growth)
    grow(d_pstate_, d_pstate_cap_, std::max<long long>(1, rec_state_size_), d_pstate_cap_, stream_);
    grow(d_carry_, d_carry_cap_, projected_carry_doubles(rec_width_), d_carry_cap_, stream_);
    grow(d_pwork_, d_pwork_cap_, projected_work_doubles(rec_width_), 0, stream_);
    grow(d_y_, d_y_cap_, std::max(1, k), 0, stream_);
    const double rcond = std::min(0.5, 64.0 * kEps * std::max(host_.rows_t, k));
    block_projected_solve(LevelRecords{d_meta_, d_vals_}, rec_solved_, levels, rec_width_, reg_,
                          b_norm_, d_pstate_, d_carry_, d_pwork_, d_y_, k, rcond, dflags_ + 2,
                          stream_);
    rec_solved_ = levels;
    AMFLS_CUDA(cudaMemcpyAsync(flags, dflags_ + 2, sizeof(int), cudaMemcpyDeviceToHost, stream_));
    stream_wait(stream_);
    return d_y_;
}

}  // namespace amfls_gpu
