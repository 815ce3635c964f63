// AMFLS controller, width controller and checkpoint cadence (host C++20).
//
// Restates, step for step, the reference's decision logic:
//   solve_amfls ..................... src/algorithms/amfls/amfls.cpp:57-661
//   default_epochs / next checkpoint  amfls.cpp:25-45
//   ProgressHistory & record ........ src/algorithms/amfls/amfls_internal.hpp:14-144
//   next_dyadic_active_width_increment amfls_internal.hpp:151-181
//   maximum_feedback_feasible_width_increment :193-207
//   WidthDecision / cost gate ....... amfls_internal.hpp:209-325
//   make_horizon_width_candidate .... amfls_internal.hpp:332-392
//   make_initial_width_candidate .... amfls_internal.hpp:399-552
//   MatchedHorizonPlan helpers ...... amfls_internal.hpp:554-674
//   CertificateCheckpointSchedule ... krylov/certificate_checkpoint_schedule.hpp:15-131
//   solve_fixed_rbgk ................ src/algorithms/fixed_rbgk/fixed_rbgk.cpp:18-209
// The decisions are the reference's; what differs is where the work runs:
// levels between checkpoints are enqueued on the GPU without host round
// trips (the device decides when the process must stop), and the measured
// seconds that feed the width decisions are CUDA-event device times.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>

#include "common.cuh"
#include "controller.hpp"
#include "gaussian.hpp"
#include "solve_common.hpp"
#include "workspace.hpp"

namespace amfls_gpu {
namespace {

using Clock = std::chrono::steady_clock;
constexpr double kInf = std::numeric_limits<double>::infinity();
constexpr int kIntMax = std::numeric_limits<int>::max();
constexpr double kDblMax = std::numeric_limits<double>::max();
using LD = long double;

double seconds_since(Clock::time_point t) {
    return std::chrono::duration<double>(Clock::now() - t).count();
}

// ------------------------------------------------------ width controller

struct History {
    double contr[2] = {0.0, 0.0};
    double level_contr[2] = {0.0, 0.0};
    int levels[2] = {0, 0};
    double op_s[2] = {kInf, kInf};
    double local_s[2] = {kInf, kInf};
    int count = 0;
    double prior_contr = 0.0;
    int prior_levels = 0;
    int width = -1;
};

void record_progress(History& h, double prev, double cur, int start_w, int end_w, int levels,
                     double op_s, double local_s) {
    if (start_w <= 0 || end_w <= 0 || start_w != end_w) {
        h = History{};
        return;
    }
    if (h.width != start_w) {
        h = History{};
        h.width = start_w;
    }
    if (levels <= 0 || !(prev > 0.0) || !(cur > 0.0) || !std::isfinite(prev) ||
        !std::isfinite(cur))
        return;
    const LD progress = prev > cur ? std::log(static_cast<LD>(prev)) - std::log(static_cast<LD>(cur))
                                   : 0.0L;
    if (!(progress >= 0.0L) || !std::isfinite(progress)) return;
    const LD lvl = progress / static_cast<LD>(levels);
    const double lvl_d = lvl > 0.0L && std::isfinite(lvl)
                             ? static_cast<double>(std::min(lvl, static_cast<LD>(kDblMax)))
                             : 0.0;
    const bool fin = op_s >= 0.0 && local_s >= 0.0 && std::isfinite(op_s) &&
                     std::isfinite(local_s) && op_s + local_s > 0.0 &&
                     std::isfinite(op_s + local_s);
    const double lop = fin ? op_s / levels : kInf;
    const double lloc = fin ? local_s / levels : kInf;
    if (h.count < 2) {
        const int i = h.count++;
        h.contr[i] = static_cast<double>(progress);
        h.level_contr[i] = lvl_d;
        h.levels[i] = levels;
        h.op_s[i] = lop;
        h.local_s[i] = lloc;
    } else {
        const LD pooled = static_cast<LD>(h.prior_contr) + static_cast<LD>(h.contr[0]);
        if (h.prior_levels > kIntMax - h.levels[0] || !std::isfinite(pooled) ||
            pooled > static_cast<LD>(kDblMax)) {
            h.prior_contr = kInf;
            h.prior_levels = kIntMax;
        } else {
            h.prior_contr = static_cast<double>(pooled);
            h.prior_levels += h.levels[0];
        }
        h.contr[0] = h.contr[1];
        h.contr[1] = static_cast<double>(progress);
        h.level_contr[0] = h.level_contr[1];
        h.level_contr[1] = lvl_d;
        h.levels[0] = h.levels[1];
        h.levels[1] = levels;
        h.op_s[0] = h.op_s[1];
        h.op_s[1] = lop;
        h.local_s[0] = h.local_s[1];
        h.local_s[1] = lloc;
    }
}

int next_dyadic_increment(int active, int generated, int max_generated, int available) {
    if (active <= 0 || generated < 0 || max_generated <= generated || active > generated + 1 ||
        available <= 0)
        return 0;
    const long long max_active = static_cast<long long>(active) + max_generated - generated;
    const long long cur = active;
    const long long nxt = cur > max_active / 2 ? max_active : std::min(2 * cur, max_active);
    if (nxt <= cur) return 0;
    const long long req = nxt - cur;
    return req <= available && req <= kIntMax ? static_cast<int>(req) : 0;
}

int ceil_ratio(int a, int b) { return a <= 0 || b <= 0 ? 0 : 1 + (a - 1) / b; }

int feedback_feasible_increment(int rank, int limit, int frontier, int levels) {
    if (rank < 0 || limit < rank || frontier < 0 || levels <= 0) return 0;
    return std::max(0, (limit - rank) / levels - frontier);
}

struct Decision {
    double recent = 0.0, prior = 0.0, remaining = 0.0;
    int forecast = 0, incumbent_levels = 0, target_levels = 0, target_remaining = 0;
    int matched_horizon = 0;
    double inc_s = kInf, tgt_s = kInf;
    bool history_mature = false, prior_mature = false, recent_slowdown = false;
    bool persistent_slowdown = false, stalled = false, long_horizon = false, necessary = false;
    bool costs_mature = false, width_depth_ok = true, pass_reduction = false, feasible = false;
    bool finite_cert = false, finite_boundary = false, candidate = false;
};

void cost_gate(Decision& d, int aw, int tw, const double* lop, const double* lloc, int count,
               double inc_cost, double tgt_cost) {
    if (d.incumbent_levels <= 0 || d.target_levels <= 0 || aw <= 0 || tw <= aw || count != 2 ||
        !(inc_cost > 0.0) || !(tgt_cost > 0.0) || !std::isfinite(inc_cost) ||
        !std::isfinite(tgt_cost))
        return;
    const LD wr = static_cast<LD>(tw) / static_cast<LD>(aw);
    const LD wr2 = wr * wr;
    const LD ratio = static_cast<LD>(tgt_cost) / static_cast<LD>(inc_cost);
    const LD inc_op_cost = static_cast<LD>(d.incumbent_levels) * static_cast<LD>(inc_cost);
    const LD tgt_op_cost = static_cast<LD>(d.target_levels) * static_cast<LD>(tgt_cost);
    LD best_inc = std::numeric_limits<LD>::infinity(), worst_tgt = 0.0L;
    bool ok = true;
    for (int i = 0; i < count; ++i) {
        const LD o = lop[i], l = lloc[i];
        if (!(o >= 0.0L) || !(l >= 0.0L) || !std::isfinite(o) || !std::isfinite(l) ||
            !(o + l > 0.0L)) {
            ok = false;
            break;
        }
        const LD inc = static_cast<LD>(d.incumbent_levels) * (o + l);
        const LD tl = l * wr2;
        const LD tgt = static_cast<LD>(d.target_levels) * (o * ratio + tl) + tl;
        if (!std::isfinite(inc) || !std::isfinite(tgt)) {
            ok = false;
            break;
        }
        best_inc = std::min(best_inc, inc);
        worst_tgt = std::max(worst_tgt, tgt);
    }
    if (ok) {
        ok = best_inc <= static_cast<LD>(kDblMax) && worst_tgt <= static_cast<LD>(kDblMax);
        if (ok) {
            d.inc_s = static_cast<double>(best_inc);
            d.tgt_s = static_cast<double>(worst_tgt);
        }
    }
    d.costs_mature = ok;
    d.pass_reduction = d.width_depth_ok && d.target_levels < d.incumbent_levels &&
                       tgt_op_cost < inc_op_cost && d.costs_mature && d.tgt_s < d.inc_s;
}

Decision horizon_candidate(int inc, int horizon, int depth, int max_depth, int rank, int limit,
                           int aw, const double* lop, const double* lloc, int count,
                           double inc_cost, double tgt_cost, bool balance) {
    Decision d;
    d.feasible = inc > 0 && aw > 0 && inc <= kIntMax - aw;
    d.finite_boundary = depth >= 0 && max_depth >= depth && rank >= 0 && limit >= rank && aw > 0 &&
                        horizon > 0 && horizon <= limit - rank;
    if (!d.feasible || !d.finite_boundary) return d;
    const int tw = aw + inc;
    d.target_remaining = std::min(max_depth - depth, (limit - rank) / tw);
    const long long cap = static_cast<long long>(d.target_remaining) * tw;
    d.matched_horizon = static_cast<int>(std::min<long long>(horizon, cap));
    d.incumbent_levels = ceil_ratio(d.matched_horizon, aw);
    d.target_levels = ceil_ratio(d.matched_horizon, tw);
    if (d.target_levels < 2) return d;
    d.width_depth_ok = !balance || d.target_levels > tw;
    cost_gate(d, aw, tw, lop, lloc, count, inc_cost, tgt_cost);
    d.candidate = d.pass_reduction;
    return d;
}

Decision initial_candidate(int inc, double cert, double tol, int depth, int max_depth, int rank,
                           int limit, int aw, const History& h, double inc_cost, double tgt_cost) {
    Decision d;
    d.finite_cert = cert > 0.0 && tol > 0.0 && cert > tol && std::isfinite(cert) &&
                    std::isfinite(tol);
    d.history_mature = h.width == aw && h.count >= 2;
    if (!d.finite_cert || !d.history_mature || depth < 0 || max_depth < depth || rank < 0 ||
        limit < rank || aw <= 0 || inc <= 0 || inc > kIntMax - aw)
        return d;
    const long long recent_levels = static_cast<long long>(h.levels[0]) + h.levels[1];
    const LD recent_progress = static_cast<LD>(h.contr[0]) + static_cast<LD>(h.contr[1]);
    if (recent_levels <= 0 || !(recent_progress >= 0.0L) || !std::isfinite(recent_progress))
        return d;
    d.stalled = recent_progress == 0.0L;
    d.recent = d.stalled ? 0.0 : static_cast<double>(recent_progress / static_cast<LD>(recent_levels));
    d.remaining = std::log(cert) - std::log(tol);
    if ((!d.stalled && (!(d.recent > 0.0) || !std::isfinite(d.recent))) ||
        !(d.remaining > 0.0) || !std::isfinite(d.remaining))
        return d;
    if (!d.stalled) {
        const LD raw = static_cast<LD>(d.remaining) / static_cast<LD>(d.recent);
        if (!(raw > 0.0L) || !std::isfinite(raw)) return d;
        d.forecast = raw >= static_cast<LD>(kIntMax)
                         ? kIntMax
                         : std::max(1, static_cast<int>(std::ceil(raw)));
    }
    d.prior_mature = h.prior_levels > 0 && h.prior_contr > 0.0 && std::isfinite(h.prior_contr);
    if (d.prior_mature) {
        d.prior = h.prior_contr / static_cast<double>(h.prior_levels);
        d.persistent_slowdown = std::isfinite(d.prior) && h.level_contr[0] > 0.0 &&
                                h.level_contr[1] > 0.0 && h.level_contr[0] < d.prior &&
                                h.level_contr[1] < d.prior;
    }
    const int remaining_basis = limit - rank;
    const int tw = aw + inc;
    const int tr = std::min(max_depth - depth, remaining_basis / tw);
    const long long raw_h = d.stalled ? static_cast<long long>(tw) * tr
                                      : static_cast<long long>(aw) * d.forecast;
    const int horizon = static_cast<int>(std::min<long long>(raw_h, remaining_basis));
    Decision c = horizon_candidate(inc, horizon, depth, max_depth, rank, limit, aw, h.op_s,
                                   h.local_s, 2, inc_cost, tgt_cost, false);
    c.finite_cert = d.finite_cert;
    c.history_mature = d.history_mature;
    c.prior_mature = d.prior_mature;
    c.persistent_slowdown = d.persistent_slowdown;
    c.stalled = d.stalled;
    c.recent = d.recent;
    c.prior = d.prior;
    c.remaining = d.remaining;
    c.forecast = d.forecast;
    c.long_horizon = c.target_remaining > 0 && (c.stalled || d.forecast > c.target_remaining);
    const bool positive = h.level_contr[0] > 0.0 && h.level_contr[1] > 0.0;
    c.recent_slowdown = positive && h.level_contr[1] < 0.5 * h.level_contr[0];
    const bool established_stall = c.stalled && (aw > 1 || c.prior_mature);
    const bool scalar_needed = aw == 1 && positive &&
                               (c.recent_slowdown ||
                                (c.prior_mature && (c.persistent_slowdown || c.long_horizon)));
    const bool block_needed = aw > 1 && (positive || established_stall) &&
                              (c.persistent_slowdown || c.long_horizon || c.pass_reduction);
    c.necessary = scalar_needed || block_needed;
    c.candidate = c.candidate && c.necessary;
    return c;
}

struct Plan {
    int end = -1, origin = -1, width = -1;
    double start_cert = kInf;
    double op_s[2] = {kInf, kInf};
    double local_s[2] = {kInf, kInf};
    int count = 0;
};

int remaining_horizon(const Plan& p, int rank) {
    if (p.end < 0 || rank < 0 || rank >= p.end) return 0;
    return p.end - rank;
}

bool extend_to_limit(Plan& p, int rank, int limit) {
    if (p.end < 0 || rank < 0 || limit <= rank || rank < p.end) return false;
    p.end = limit;
    return true;
}

bool horizon_stalled(const Plan& p, double cert) {
    return p.start_cert > 0.0 && cert > 0.0 && std::isfinite(p.start_cert) &&
           std::isfinite(cert) && std::log(p.start_cert) - std::log(cert) < std::log(2.0);
}

bool start_plan(Plan& p, int rank, int limit, int horizon, int origin, int target, double cert) {
    if (rank < 0 || limit < rank || horizon <= 0 || horizon > limit - rank || origin <= 0 ||
        target <= 0 || !(cert > 0.0) || !std::isfinite(cert)) {
        p = Plan{};
        return false;
    }
    p = Plan{};
    p.end = rank + horizon;
    p.origin = origin;
    p.width = target;
    p.start_cert = cert;
    return true;
}

void reset_plan_costs(Plan& p, int width) {
    p.width = width;
    p.op_s[0] = p.op_s[1] = kInf;
    p.local_s[0] = p.local_s[1] = kInf;
    p.count = 0;
}

bool record_plan_cost(Plan& p, int start_w, int end_w, int levels, double op_s, double local_s) {
    if (p.end < 0 || start_w <= 0 || start_w != end_w || start_w != p.width || levels <= 0 ||
        op_s < 0.0 || local_s < 0.0 || !std::isfinite(op_s) || !std::isfinite(local_s) ||
        !(op_s + local_s > 0.0) || p.count >= 2)
        return false;
    p.op_s[p.count] = op_s / levels;
    p.local_s[p.count] = local_s / levels;
    ++p.count;
    return true;
}

int default_epochs(int dim) {
    int epochs = 1, covered = 1;
    while (covered < dim && epochs < 30) {
        covered *= 2;
        ++epochs;
    }
    return epochs;
}

bool step_truncated(const StepAudit& a) {
    return (a.right_rank_loss && a.right_positive_finite_below_cutoff &&
            a.right_active_discarded_residual_norm > 0.0) ||
           (a.left_rank_loss && a.left_positive_finite_below_cutoff);
}

bool step_broke(const StepAudit& a) {
    return a.right_nonfinite_residual || a.left_nonfinite_residual;
}

double certificate(const ValidationOutput& v, double reg) {
    return reg > 0.0 ? v.relative_energy_error_upper_bound : v.backward_error_upper_bound;
}

void check_common(const DeviceOperator& op, const double* d_b, const SolveOptions& o) {
    if (op.rows() <= 0 || op.cols() <= 0) throw std::invalid_argument("operator dimensions must be positive");
    if (d_b == nullptr) throw std::invalid_argument("right-hand side cannot be null");
    if (!std::isfinite(o.regularization) || o.regularization < 0.0)
        throw std::invalid_argument("regularization must be finite and nonnegative");
    if (!std::isfinite(o.tolerance) || o.tolerance <= 0.0 || o.tolerance >= 1.0)
        throw std::invalid_argument("tolerance must lie strictly between zero and one");
    if (!std::isfinite(o.failure_probability) || o.failure_probability <= 0.0 ||
        o.failure_probability >= 1.0)
        throw std::invalid_argument("failure_probability must lie strictly between zero and one");
}

// Candidate bookkeeping: three device solution buffers so that the latest
// and the best candidate survive without copies.
struct Candidate {
    ValidationOutput v{};
    int depth = 0, auxiliary_width = 0, basis_rank = 0;
    Statistics stats;
    int buffer = -1;
};

class Evaluator {
public:
    Evaluator(Workspace& ws, const DeviceOperator& op, const double* d_b, double reg,
              Statistics& stats, cudaStream_t stream)
        : ws_(ws), validator_(op, d_b, reg, stream), stats_(stats), stream_(stream), n_(op.cols()) {
        for (auto& p : buf_) stream_alloc(&p, sizeof(double) * std::max(1, n_), stream_);
    }
    ~Evaluator() {
        cudaStreamSynchronize(stream_);
        for (auto p : buf_) stream_free(p, stream_);
    }

    Candidate evaluate(double tol, int epoch, int aux, int keep_a, int keep_b, TraceRow* row) {
        int slot = 0;
        while (slot == keep_a || slot == keep_b) ++slot;
        const auto t0 = Clock::now();
        ws_.solve_projected(buf_[slot]);
        if (ws_.projected_flags() & 2) ++stats_.projected_rank_flags;
        stats_.projected_solve_seconds += seconds_since(t0);
        const ValidationOutput v = validator_.validate(buf_[slot], tol);
        Statistics& s = stats_;
        account_validation(s, v);
        Candidate c;
        c.v = v;
        c.depth = ws_.depth();
        c.auxiliary_width = aux;
        c.basis_rank = ws_.basis_rank();
        c.stats = s;
        c.buffer = slot;
        if (row) fill_trace_row(*row, c.v, c.stats, epoch, c.depth, c.auxiliary_width, c.basis_rank);
        return c;
    }

    double* buffer(int i) const { return buf_[i]; }

private:
    Workspace& ws_;
    Validator validator_;
    Statistics& stats_;
    cudaStream_t stream_;
    int n_;
    double* buf_[3] = {nullptr, nullptr, nullptr};
};

// Fold the device counters of executed search levels into the statistics.
void absorb_search_counters(const DevState& st, Statistics& s, long long& seen_a,
                            long long& seen_at, long long& seen_ac, long long& seen_atc) {
    const long long da = st.search_a_columns - seen_a, dat = st.search_at_columns - seen_at;
    const long long dac = st.search_a_calls - seen_ac, datc = st.search_at_calls - seen_atc;
    s.a_columns += da;
    s.search_a_columns += da;
    s.at_columns += dat;
    s.search_at_columns += dat;
    s.a_block_calls += dac;
    s.search_a_block_calls += dac;
    s.at_block_calls += datc;
    s.search_at_block_calls += datc;
    seen_a = st.search_a_columns;
    seen_at = st.search_at_columns;
    seen_ac = st.search_a_calls;
    seen_atc = st.search_at_calls;
}

}  // namespace

// Features of a width decision, all from the controller's own state and
// scaled to order one (their meaning is fixed: a trained policy depends on
// it):
//   0 log10(certificate / tol), clipped to [-2, 20]
//   1 recent certificate decrease per level, decades (0..5)
//   2 log10 operator seconds per level, clipped to [-7, 1]
//   3 log10 local (orthogonalisation) seconds per level, clipped to [-7, 1]
//   4 log10 of the relative block cost of the widened over the current width
//   5 log2(1 + current width), 6 log2(1 + increment)
//   7 free basis fraction, 8 free depth fraction
//   9 a matched-horizon plan is active (0/1), 10 the heuristic widens (0/1)
void width_features(double* f, double cert, double tol, const History& h, const Plan& plan,
                    double cost_now, double cost_wide, int frontier, int inc, int rank,
                    int limit, int depth, int max_depth, bool horizon, bool heuristic) {
    auto clip = [](double v, double lo, double hi) {
        return std::isfinite(v) ? std::min(hi, std::max(lo, v)) : (v > 0 ? hi : lo);
    };
    f[0] = clip(std::log10(cert / tol), -2.0, 20.0);
    double lvl = 0.0, op = kInf, loc = kInf;
    if (h.count > 0) {
        lvl = h.level_contr[h.count - 1] / std::log(10.0);
        op = h.op_s[h.count - 1];
        loc = h.local_s[h.count - 1];
    } else if (plan.count > 0) {
        op = plan.op_s[plan.count - 1];
        loc = plan.local_s[plan.count - 1];
    }
    f[1] = clip(lvl, 0.0, 5.0);
    f[2] = clip(std::log10(op), -7.0, 1.0);
    f[3] = clip(std::log10(loc), -7.0, 1.0);
    f[4] = clip(std::log10(cost_wide / cost_now), -3.0, 3.0);
    f[5] = std::log2(1.0 + frontier);
    f[6] = std::log2(1.0 + inc);
    f[7] = limit > 0 ? (double)(limit - rank) / limit : 0.0;
    f[8] = max_depth > 0 ? (double)(max_depth - depth) / max_depth : 0.0;
    f[9] = horizon ? 1.0 : 0.0;
    f[10] = heuristic ? 1.0 : 0.0;
}

SolveResult solve_amfls(const DeviceOperator& op, const double* d_b, const SolveOptions& o,
                        double* d_solution, cudaStream_t stream, const WidthControl* control) {
    check_common(op, d_b, o);
    if (o.maximum_epochs < 0 || o.maximum_depth < 0 || o.maximum_auxiliary_width < 0 ||
        o.maximum_basis_size < 0)
        throw std::invalid_argument("work limits must be nonnegative");
    const double reg = o.regularization, tol = o.tolerance;
    const auto t_start = Clock::now();
    const long long launches0 = launch_count();
    Statistics stats;
    Workspace ws(op, d_b, reg, o.maximum_basis_size, stream, o.time_operators,
                 o.use_graphs && op.graph_safe(), o.reduced_basis);
    Evaluator ev(ws, op, d_b, reg, stats, stream);
    long long seen[4] = {0, 0, 0, 0};
    auto absorb = [&] {
        absorb_search_counters(ws.state(), stats, seen[0], seen[1], seen[2], seen[3]);
        double a = 0.0, at = 0.0;
        ws.take_operator_seconds(a, at);
        stats.a_seconds += a;
        stats.at_seconds += at;
        return a + at;
    };

    const int dim = std::min(op.rows(), op.cols());
    const int max_depth = o.maximum_depth > 0 ? std::min(o.maximum_depth, dim) : dim;
    const int cap = std::max(0, ws.basis_limit() - 1);
    const int max_aux = std::min(o.maximum_auxiliary_width > 0 ? o.maximum_auxiliary_width : cap, cap);
    const int max_epochs = o.maximum_epochs > 0 ? o.maximum_epochs : default_epochs(dim);

    SolveResult out;
    out.rows = op.rows();
    out.cols = op.cols();
    CheckpointSchedule sched(reg, tol);
    int evaluations = 0, last_depth = -1, aux = 0;
    Candidate result, best;
    double best_cert = kInf;
    bool has = false;

    auto record = [&](const Candidate& c, bool train, const TraceRow& row) {
        if (c.depth == last_depth) throw std::logic_error("AMFLS evaluated one checkpoint more than once");
        last_depth = c.depth;
        if (train) sched.record(c.depth, c.v);
        out.trace.push_back(row);
        ++evaluations;
        const double cert = certificate(c.v, reg);
        const bool better = !has || (std::isfinite(cert) && !std::isfinite(best_cert)) ||
                            cert < best_cert;
        if (better) {
            best_cert = cert;
            best = c;
        }
        has = true;
        result = c;
    };
    auto evaluate = [&](bool train) {
        TraceRow row;
        const Candidate c = ev.evaluate(tol, evaluations, aux, result.buffer, best.buffer, &row);
        record(c, train, row);
    };
    // the open decision record, closed at the next decision or at the end
    int open_record = -1;
    double open_cert = kInf, open_time = 0.0;
    auto close_record = [&]() {
        if (!control || !control->log || open_record < 0) return;
        DecisionRecord& r = (*control->log)[open_record];
        const double now = seconds_since(t_start), cert = certificate(result.v, reg);
        const double dt = now - open_time;
        r.rate = (std::log10(open_cert) - std::log10(cert)) / dt;
        r.valid = std::isfinite(r.rate) && dt > 0.0 ? 1 : 0;
        open_record = -1;
    };
    auto finish = [&](const Candidate& c, int status, int reason) {
        close_record();
        out.iterations = ws.depth();
        out.depth = c.depth;
        out.auxiliary_width = c.auxiliary_width;
        out.basis_rank = c.basis_rank;
        out.v = c.v;
        out.status = status;
        out.stop_reason = reason;
        AMFLS_CUDA(cudaMemcpyAsync(d_solution, ev.buffer(c.buffer), sizeof(double) * op.cols(),
                                   cudaMemcpyDeviceToDevice, stream));
        stream_wait(stream);
        stats.total_seconds = seconds_since(t_start);
        stats.kernel_launches = launch_count() - launches0;
        stats.reduced_levels = ws.state().reduced_levels;
        stats.reduced_fallbacks = ws.state().reduced_fallbacks;
        out.statistics = stats;
        return out;
    };
    auto finish_self = [&](const Candidate& c) { return finish(c, c.v.status, c.v.stop_reason); };
    auto finish_at_limit = [&](int status, int reason) {
        return finish(reg > 0.0 || o.latest_at_limit ? result : best, status, reason);
    };

    ws.initialize(nullptr, 0);
    if (ws.can_advance() && max_depth > 0) {
        ws.advance_to(1);
        ws.sync();
    }
    absorb();
    evaluate(true);
    if (failed_numerically(result.v) || result.v.status == 0) return finish_self(result);
    bool truncated = step_truncated(ws.last_step_audit());
    bool broke = step_broke(ws.last_step_audit());

    History hist;
    Plan plan;
    int epoch = 0, replay_sites = 0;
    std::uint64_t generated = 0;
    bool feedback = false;
    int fb_target = 0, stage_rank = 0, stage_origin = 0, stage_target = 0;
    cudaEvent_t iv0, iv1;
    AMFLS_CUDA(cudaEventCreateWithFlags(&iv0, cudaEventBlockingSync));
    AMFLS_CUDA(cudaEventCreateWithFlags(&iv1, cudaEventBlockingSync));
    struct EventGuard {
        cudaEvent_t a, b;
        ~EventGuard() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } guard{iv0, iv1};

    while (true) {
        if (broke) return finish_at_limit(4, 7);
        if (ws.basis_rank() >= ws.basis_limit()) return finish_at_limit(2, 5);
        if (ws.depth() >= max_depth) return finish_at_limit(1, 3);
        if (truncated) return finish_at_limit(3, 6);
        const double interval_cert = certificate(result.v, reg);
        const int frontier = ws.active_left_width();
        const int avail_inc = std::max(0, std::max(0, ws.basis_limit() - ws.basis_rank()) - frontier);
        const int width_cap = std::min(avail_inc, std::max(0, max_aux - aux));
        const bool full_fb = max_depth - ws.depth() >= 2;
        const int fb_depth = full_fb ? ws.depth() + 2 : ws.depth();
        const int fb_inc = full_fb ? feedback_feasible_increment(ws.basis_rank(), ws.basis_limit(),
                                                                 frontier, fb_depth - ws.depth())
                                   : 0;
        const int feasible_cap = std::min(width_cap, fb_inc);
        if (plan.end >= 0 && remaining_horizon(plan, ws.basis_rank()) == 0) plan = Plan{};
        const int rem = remaining_horizon(plan, ws.basis_rank());
        const bool horizon_active = rem > 0;
        const bool collecting = horizon_active && !feedback && plan.count < 2;
        const bool ready = !feedback && !collecting;
        const bool stage_ok = ready && epoch < max_epochs;
        const int inc = stage_ok ? next_dyadic_increment(frontier, aux, max_aux, feasible_cap) : 0;
        int requested = 0, req_horizon = 0;
        if (stage_ok && inc > 0) {
            const int tw = frontier + inc;
            const Decision d =
                horizon_active
                    ? horizon_candidate(inc, rem, ws.depth(), max_depth, ws.basis_rank(),
                                        ws.basis_limit(), frontier, plan.op_s, plan.local_s,
                                        plan.count, op.relative_block_product_cost(frontier),
                                        op.relative_block_product_cost(tw), plan.origin > 1)
                    : initial_candidate(inc, interval_cert, tol, ws.depth(), max_depth,
                                        ws.basis_rank(), ws.basis_limit(), frontier, hist,
                                        op.relative_block_product_cost(frontier),
                                        op.relative_block_product_cost(tw));
            // the candidate bit, or the replayed one in schedule-replay mode
            bool candidate = d.candidate;
            if (control && control->replay_count >= 0) {
                if (replay_sites < control->replay_count)
                    candidate = control->replay[replay_sites] != 0;
                else if (control->overrun)
                    ++*control->overrun;
                ++replay_sites;
            }
            if (control && control->sites) control->sites->push_back(candidate ? 1 : 0);
            bool widen = candidate;
            if (control) {
                DecisionRecord rec{};
                width_features(rec.features, interval_cert, tol, hist, plan,
                               op.relative_block_product_cost(frontier),
                               op.relative_block_product_cost(tw), frontier, inc,
                               ws.basis_rank(), ws.basis_limit(), ws.depth(), max_depth,
                               horizon_active, d.candidate);
                if (control->policy) {
                    double stay = 0.0, wide = 0.0;
                    control->policy->score(rec.features, &stay, &wide, stream);
                    if (std::isfinite(stay) && std::isfinite(wide)) widen = wide > stay;
                }
                if (control->exploration > 0.0) {
                    std::uint64_t st = control->exploration_seed ^ (0x9e3779b97f4a7c15ULL *
                                                                    (std::uint64_t)(epoch + 1 + 1000 * ws.depth()));
                    st = (st ^ (st >> 30)) * 0xbf58476d1ce4e5b9ULL;
                    st = (st ^ (st >> 27)) * 0x94d049bb133111ebULL;
                    st ^= st >> 31;
                    const double u = (double)(st >> 11) * 0x1p-53;
                    if (u < control->exploration) widen = ((st >> 5) & 1u) != 0;
                }
                rec.action = widen ? 1 : 0;
                rec.heuristic = d.candidate ? 1 : 0;
                if (control->log) {
                    close_record();
                    control->log->push_back(rec);
                    open_record = (int)control->log->size() - 1;
                    open_cert = interval_cert;
                    open_time = seconds_since(t_start);
                }
            }
            if (widen) {
                requested = inc;
                if (!horizon_active && candidate) req_horizon = d.matched_horizon;
            }
        }
        if (horizon_active && ready && requested == 0) plan = Plan{};

        if (requested > 0) {
            fb_target = fb_depth;
            stage_rank = ws.basis_rank();
            stage_origin = horizon_active ? plan.origin : frontier;
            stage_target = frontier + requested;
            hist = History{};
            sched = CheckpointSchedule(reg, tol);
            // Gaussian block orthogonal to b/||b|| (amfls.cpp:191-231)
            double* rnd = nullptr;
            AMFLS_CUDA(cudaMallocAsync(&rnd, sizeof(double) * op.rows() * (size_t)requested, stream));
            gaussian_block(op.rows(), requested, o.seed, o.stream, generated, rnd, op.rows(), stream);
            project_out_direction(rnd, op.rows(), requested, d_b, ws.right_hand_side_norm(), stream);
            stats.gaussian_random_block_requests += 1;
            stats.gaussian_random_columns += requested;
            stats.gaussian_random_values += static_cast<long long>(op.rows()) * requested;
            generated += static_cast<std::uint64_t>(requested);
            aux += requested;
            ++epoch;
            ws.append_left_seed(rnd, requested);
            AMFLS_CUDA(cudaFreeAsync(rnd, stream));
            bool advanced = false;
            if (ws.can_advance()) advanced = ws.advance_level();
            absorb();
            if (advanced) {
                if (req_horizon > 0)
                    start_plan(plan, stage_rank, ws.basis_limit(), req_horizon, stage_origin,
                               stage_target, interval_cert);
                else
                    reset_plan_costs(plan, stage_target);
                truncated = step_truncated(ws.last_step_audit());
                broke = step_broke(ws.last_step_audit());
                const bool exhausted = remaining_horizon(plan, ws.basis_rank()) == 0;
                const bool terminal = ws.basis_rank() >= ws.basis_limit() ||
                                      ws.depth() >= max_depth || !ws.can_advance();
                if (terminal || exhausted) {
                    evaluate(false);
                    if (failed_numerically(result.v) || result.v.status == 0) return finish_self(result);
                }
                const bool reliable = !truncated && !broke && ws.basis_rank() > stage_rank &&
                                      ws.active_left_width() == stage_target;
                const bool extended = exhausted &&
                                      horizon_stalled(plan, certificate(result.v, reg)) &&
                                      extend_to_limit(plan, ws.basis_rank(), ws.basis_limit());
                if (!reliable || (exhausted && !extended)) {
                    plan = Plan{};
                    feedback = false;
                } else {
                    feedback = true;
                }
            } else {
                truncated = step_truncated(ws.last_step_audit());
                broke = step_broke(ws.last_step_audit());
                feedback = false;
                plan = Plan{};
            }
            continue;
        }

        if (ws.can_advance()) {
            const int d0 = ws.depth(), k0 = ws.basis_rank();
            const bool matched = !feedback && remaining_horizon(plan, k0) > 0 && plan.count < 2;
            int target;
            if (feedback) {
                target = fb_target;
            } else if (matched) {
                target = std::min(d0 + 1, max_depth);
            } else {
                target = d0 + 1;
                while (target < max_depth && !sched.should_evaluate(target)) ++target;
            }
            AMFLS_CUDA(cudaEventRecord(iv0, stream));
            ws.advance_to(target);
            AMFLS_CUDA(cudaEventRecord(iv1, stream));
            ws.sync();
            float ms = 0.0f;
            AMFLS_CUDA(cudaEventElapsedTime(&ms, iv0, iv1));
            const double span = ms * 1e-3;
            const double op_s = std::max(0.0, absorb());
            const double local_s = std::max(0.0, span - op_s);
            stats.orthogonalization_seconds += local_s;
            truncated = step_truncated(ws.last_step_audit());
            broke = step_broke(ws.last_step_audit());
            if (ws.depth() > d0) {
                const bool pair_done = matched && plan.count == 1;
                const bool exhausts = (feedback || matched) && remaining_horizon(plan, ws.basis_rank()) == 0;
                const bool terminal = ws.basis_rank() >= ws.basis_limit() ||
                                      ws.depth() >= max_depth || !ws.can_advance();
                if ((!feedback && !matched) || pair_done || exhausts || terminal) {
                    evaluate(!feedback && !matched);
                    if (failed_numerically(result.v) || result.v.status == 0) return finish_self(result);
                }
                if (feedback && ws.depth() >= fb_target) {
                    feedback = false;
                    const bool ok = !truncated && !broke && ws.basis_rank() > k0 &&
                                    ws.basis_rank() > stage_rank && frontier == stage_target &&
                                    ws.active_left_width() == stage_target;
                    const bool rec = ok && record_plan_cost(plan, frontier, ws.active_left_width(),
                                                            ws.depth() - d0, op_s, local_s);
                    const bool exh = remaining_horizon(plan, ws.basis_rank()) == 0;
                    const bool ext = exh && horizon_stalled(plan, certificate(result.v, reg)) &&
                                     extend_to_limit(plan, ws.basis_rank(), ws.basis_limit());
                    if (!rec || (exh && !ext)) plan = Plan{};
                } else if (matched) {
                    const bool ok = !truncated && !broke && ws.basis_rank() > k0 &&
                                    frontier == ws.active_left_width();
                    const bool rec = ok && record_plan_cost(plan, frontier, ws.active_left_width(),
                                                            ws.depth() - d0, op_s, local_s);
                    const bool exh = remaining_horizon(plan, ws.basis_rank()) == 0;
                    const bool ext = exh && horizon_stalled(plan, certificate(result.v, reg)) &&
                                     extend_to_limit(plan, ws.basis_rank(), ws.basis_limit());
                    if (!rec || (exh && !ext)) plan = Plan{};
                } else if (!feedback) {
                    record_progress(hist, interval_cert, certificate(result.v, reg), frontier,
                                    ws.active_left_width(), ws.depth() - d0, op_s, local_s);
                }
                continue;
            }
            if (feedback || matched) {
                feedback = false;
                plan = Plan{};
            }
            continue;
        }
        int reason = 2;
        if (!feedback && epoch >= max_epochs && aux < max_aux && avail_inc > 0) reason = 4;
        return finish_at_limit(1, reason);
    }
}

SolveResult solve_fixed_rbgk(const DeviceOperator& op, const double* d_b, const SolveOptions& o,
                             double* d_solution, cudaStream_t stream) {
    check_common(op, d_b, o);
    if (o.auxiliary_width < 0) throw std::invalid_argument("auxiliary_width must be nonnegative");
    if (o.maximum_depth <= 0) throw std::invalid_argument("maximum_depth must be positive");
    if (o.maximum_basis_size < 0) throw std::invalid_argument("maximum_basis_size must be nonnegative");
    if (o.auxiliary_width == std::numeric_limits<int>::max())
        throw std::length_error("fixed RBGK seed width exceeds LP64 limits");
    const double reg = o.regularization, tol = o.tolerance;
    const auto t_start = Clock::now();
    const long long launches0 = launch_count();
    Statistics stats;
    Workspace ws(op, d_b, reg, o.maximum_basis_size, stream, o.time_operators,
                 o.use_graphs && op.graph_safe(), o.reduced_basis);
    Evaluator ev(ws, op, d_b, reg, stats, stream);
    long long seen[4] = {0, 0, 0, 0};
    auto absorb = [&] {
        absorb_search_counters(ws.state(), stats, seen[0], seen[1], seen[2], seen[3]);
        double a = 0.0, at = 0.0;
        ws.take_operator_seconds(a, at);
        stats.a_seconds += a;
        stats.at_seconds += at;
    };
    SolveResult out;
    out.rows = op.rows();
    out.cols = op.cols();
    CheckpointSchedule sched(reg, tol);
    Candidate result;
    int depth = 0, evaluated = -1;
    // the zero-RHS test needs ||b|| before the seed is drawn
    ws.initialize(nullptr, 0);
    const bool zero_rhs = ws.right_hand_side_norm() == 0.0;
    const int aux = zero_rhs ? 0 : std::min(o.auxiliary_width, std::max(0, ws.basis_limit() - 1));
    auto evaluate = [&] {
        TraceRow row;
        result = ev.evaluate(tol, 0, aux, result.buffer, -1, &row);
        sched.record(depth, result.v);
        evaluated = depth;
        out.trace.push_back(row);
    };
    auto terminal_eval = [&] {
        if (evaluated != depth) evaluate();
        return failed_numerically(result.v);
    };
    if (aux > 0) {
        double* seed = nullptr;
        AMFLS_CUDA(cudaMallocAsync(&seed, sizeof(double) * op.rows() * (size_t)aux, stream));
        gaussian_block(op.rows(), aux, o.seed, o.stream, 0, seed, op.rows(), stream);
        stats.gaussian_random_block_requests += 1;
        stats.gaussian_random_columns += aux;
        stats.gaussian_random_values += static_cast<long long>(op.rows()) * aux;
        ws.append_left_seed(seed, aux);
        AMFLS_CUDA(cudaFreeAsync(seed, stream));
    }
    if (ws.can_advance()) ws.advance_level();
    absorb();
    depth = ws.depth();
    evaluate();
    bool truncated = step_truncated(ws.last_step_audit());
    bool broke = step_broke(ws.last_step_audit());
    int status = result.v.status, reason = result.v.stop_reason;
    auto set_status = [&](int s, int r) {
        if (result.v.status != 0) {
            status = s;
            reason = r;
        }
    };
    while (true) {
        status = result.v.status;
        reason = result.v.stop_reason;
        if (failed_numerically(result.v)) break;
        if (result.v.status == 0 && o.stop_early) break;
        if (broke) {
            if (terminal_eval()) {
                status = result.v.status;
                reason = result.v.stop_reason;
                break;
            }
            status = 4;
            reason = 7;
            break;
        }
        if (ws.basis_rank() >= ws.basis_limit()) {
            if (terminal_eval()) {
                status = result.v.status;
                reason = result.v.stop_reason;
                break;
            }
            status = result.v.status;
            reason = result.v.stop_reason;
            set_status(2, 5);
            break;
        }
        if (depth >= o.maximum_depth) {
            if (terminal_eval()) {
                status = result.v.status;
                reason = result.v.stop_reason;
                break;
            }
            status = result.v.status;
            reason = result.v.stop_reason;
            set_status(1, 3);
            break;
        }
        if (truncated) {
            if (terminal_eval()) {
                status = result.v.status;
                reason = result.v.stop_reason;
                break;
            }
            status = result.v.status;
            reason = result.v.stop_reason;
            set_status(3, 6);
            break;
        }
        if (!ws.can_advance()) {
            if (terminal_eval()) {
                status = result.v.status;
                reason = result.v.stop_reason;
                break;
            }
            status = result.v.status;
            reason = result.v.stop_reason;
            set_status(1, 2);
            break;
        }
        const bool ok = ws.advance_level();
        absorb();
        truncated = step_truncated(ws.last_step_audit());
        broke = step_broke(ws.last_step_audit());
        if (!ok) {
            if (!ws.last_step_audit().right_rank_loss && !broke)
                throw std::logic_error("failed fixed extension did not report rank loss");
            continue;
        }
        depth = ws.depth();
        const bool terminal = depth >= o.maximum_depth || ws.basis_rank() >= ws.basis_limit() ||
                              !ws.can_advance() || truncated || broke;
        if (sched.should_evaluate(depth) || terminal) evaluate();
    }
    out.iterations = depth;
    out.depth = depth;
    out.auxiliary_width = aux;
    out.basis_rank = result.basis_rank;
    out.v = result.v;
    out.status = status;
    out.stop_reason = reason;
    AMFLS_CUDA(cudaMemcpyAsync(d_solution, ev.buffer(result.buffer), sizeof(double) * op.cols(),
                               cudaMemcpyDeviceToDevice, stream));
    stream_wait(stream);
    stats.total_seconds = seconds_since(t_start);
    stats.kernel_launches = launch_count() - launches0;
    stats.reduced_levels = ws.state().reduced_levels;
    stats.reduced_fallbacks = ws.state().reduced_fallbacks;
    out.statistics = stats;
    return out;
}

void pack_metrics(const SolveResult& r, double m[21]) {
    const ValidationOutput& v = r.v;
    const double t[21] = {v.objective, v.residual_norm, v.augmented_residual_norm,
                          v.normal_residual_norm, v.solution_norm, v.solution_energy_norm,
                          v.operator_norm_lower_bound, v.augmented_operator_norm_lower_bound,
                          v.compatible_backward_error_upper_bound,
                          v.least_squares_backward_error_upper_bound, v.backward_error_upper_bound,
                          v.relative_normal_residual_upper_bound, v.energy_error_upper_bound,
                          v.relative_energy_error_upper_bound, v.objective_gap_upper_bound,
                          v.ridge_base_energy_error_upper_bound,
                          v.ridge_corrected_energy_error_upper_bound, v.ridge_correction_gamma,
                          v.ridge_correction_z_h_z, v.ridge_correction_two_abs_z_t_q,
                          v.ridge_correction_q_norm_squared};
    std::memcpy(m, t, sizeof(t));
}

void pack_counters(const SolveResult& r, long long c[36]) {
    const Statistics& s = r.statistics;
    const long long t[36] = {
        s.a_columns, s.at_columns, s.a_block_calls, s.at_block_calls, s.search_a_columns,
        s.search_at_columns, s.validation_a_columns, s.validation_at_columns, r.iterations,
        r.depth, r.auxiliary_width, r.basis_rank, s.sketch_a_columns, s.sketch_at_columns,
        s.sketch_a_block_calls, s.sketch_at_block_calls, s.iterative_a_columns,
        s.iterative_at_columns, s.iterative_a_block_calls, s.iterative_at_block_calls,
        s.gaussian_random_columns, s.gaussian_random_values, s.search_a_block_calls,
        s.search_at_block_calls, s.validation_a_block_calls, s.validation_at_block_calls,
        s.base_validation_a_columns, s.base_validation_at_columns,
        s.base_validation_a_block_calls, s.base_validation_at_block_calls,
        s.ridge_correction_a_columns, s.ridge_correction_at_columns,
        s.ridge_correction_a_block_calls, s.ridge_correction_at_block_calls,
        s.gaussian_random_block_requests, r.v.ridge_correction_disposition};
    std::memcpy(c, t, sizeof(t));
}

void pack_timings(const SolveResult& r, double t[9]) {
    const Statistics& s = r.statistics;
    const double other = std::max(0.0, s.total_seconds - s.a_seconds - s.at_seconds -
                                           s.orthogonalization_seconds - s.projected_solve_seconds);
    const double v[9] = {s.total_seconds, s.a_seconds, s.at_seconds, s.orthogonalization_seconds,
                         s.projected_solve_seconds, s.validation_seconds, other,
                         s.base_validation_seconds, s.ridge_correction_validation_seconds};
    std::memcpy(t, v, sizeof(v));
}

}  // namespace amfls_gpu
