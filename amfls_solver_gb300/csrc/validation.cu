// Device restatement of the reference's certified candidate validation
// (src/algorithms/mathematics/krylov/candidate_validation.cpp:67-1378).
// The scalar steps follow the reference function by function:
//   validation_model_is_available ........... :67-83
//   underflow / callback / one-op radii ..... :85-136
//   enlarge / augmented intervals ........... :138-166
//   certified_ratio / relative_energy_bound . :168-197
//   one_step_ridge_energy_bound ............. :395-566
//   evaluate_accuracy_contract .............. :594-692
//   evaluate_certified_accuracy_contract .... :694-814
//   build_base_validation_envelope .......... :822-926
//   refine_base_validation .................. :951-1149 (double-double here)
//   validate_original_candidate ............. :1176-1378
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "common.cuh"
#include "dd.cuh"
#include "fp_bounds.cuh"
#include "validation.hpp"
#include "vector_ops.hpp"

namespace amfls_gpu {
namespace {

using fpb::Interval;
using fpb::kInf;

struct Envelope {
    int certified;
    double op_upper, op_lower, res_lower, res_upper, grad_upper;
    double sol_lower, sol_upper, b_lower, energy_lower, grad_radius;
};

struct Model {
    double upper, lower;
    long long apply_steps, transpose_steps;
};

struct ValState {
    ValidationOutput out;
    Envelope env;
    NormResult nr;   // base vectors: b, x, Ax, r, A^T r, g
    NormResult nr2;  // refined or correction vectors
    double bnorm;
    int need_refine;
    int need_correction;
    int finite_flag;
    int pad;
    double dot;      // d . h for the correction
    double corr_gnorm;
    double corr_step;
    double corr_hn_upper, corr_dn_upper, corr_adn_upper, corr_ad_err, corr_herr;
};

enum { ST_SUCCESS = 0, ST_WORK = 1, ST_BREAKDOWN = 4 };
enum { SR_EXACT = 1, SR_DEPTH = 3, SR_BREAKDOWN = 7, SR_COMPAT = 8, SR_LS = 9, SR_ENERGY = 10 };
enum {
    RC_NA = 0, RC_SKIP_PASS = 1, RC_SKIP_ZERO = 2, RC_SKIP_NONFINITE = 3, RC_IMPROVED = 4,
    RC_NOT_IMPROVED = 5, RC_BAD_CURVATURE = 6, RC_PARTIAL = 7, RC_NONFINITE = 8
};

__device__ bool model_ok(const Model& m) {
    return isfinite(m.upper) && m.upper >= 0.0 && isfinite(m.lower) && m.lower >= 0.0 &&
           m.lower <= m.upper && m.apply_steps > 0 && m.transpose_steps > 0;
}

__device__ double underflow_radius(long long ops, long long size) {
    if (ops <= 0 || size <= 0) return 0.0;
    return fpb::widen_up(__dmul_ru(__dmul_ru((double)ops, __dsqrt_ru((double)size)),
                                   fpb::kDenormMin));
}

__device__ double callback_radius(const Model& m, bool transpose, double in_upper,
                                  long long out_size, double unit) {
    if (!model_ok(m) || !isfinite(in_upper) || in_upper < 0.0) return kInf;
    if (m.upper == 0.0 || in_upper == 0.0) return 0.0;
    const long long ops = transpose ? m.transpose_steps : m.apply_steps;
    return fpb::up_add(fpb::up_mul(fpb::gamma(ops, unit), fpb::up_mul(m.upper, in_upper)),
                       underflow_radius(ops, out_size));
}

// refinement accumulation: ops = 2 * dot length, double-double unit
__device__ double dd_callback_radius(const Model& m, long long dot_length, double in_upper,
                                     long long out_size) {
    if (!model_ok(m) || dot_length <= 0 || !isfinite(in_upper) || in_upper < 0.0) return kInf;
    if (m.upper == 0.0 || in_upper == 0.0) return 0.0;
    const long long ops = 2 * dot_length;
    return fpb::up_add(fpb::up_mul(fpb::gamma(ops, kDDUnit), fpb::up_mul(m.upper, in_upper)),
                       underflow_radius(ops, out_size));
}

__device__ double one_op_radius(double stored_upper, bool can_underflow, long long size,
                                double unit) {
    if (!isfinite(stored_upper) || stored_upper < 0.0) return kInf;
    double r = fpb::up_mul(fpb::gamma(2, unit), stored_upper);
    if (can_underflow) r = fpb::up_add(r, underflow_radius(1, size));
    return r;
}

__device__ Interval enlarge(Interval s, double radius) {
    if (!isfinite(radius) || radius < 0.0) return {0.0, kInf};
    return {fpb::down_diff(s.lower, radius), fpb::up_add(s.upper, radius)};
}

__device__ Interval augmented(Interval p, Interval s, double reg) {
    return {fpb::down_sqrt(fpb::down_add(fpb::down_mul(p.lower, p.lower),
                                         fpb::down_mul(reg, fpb::down_mul(s.lower, s.lower)))),
            fpb::up_sqrt(fpb::up_add(fpb::up_mul(p.upper, p.upper),
                                     fpb::up_mul(reg, fpb::up_mul(s.upper, s.upper))))};
}

__device__ double ratio_cert(double num, double den) {
    if (!isfinite(num)) return kInf;
    if (num == 0.0) return 0.0;
    if (!isfinite(den) || den <= 0.0) return kInf;
    return num / den;
}

__device__ double rel_energy(double abs_bound, double energy) {
    if (!isfinite(energy)) return kInf;
    if (abs_bound == 0.0) return 0.0;
    if (!isfinite(abs_bound) || energy <= 0.0) return kInf;
    const double s = abs_bound / energy;
    if (!isfinite(s) || s >= 1.0) return kInf;
    return s / (1.0 - s);
}

__device__ Interval nint(const NormResult& r, int i) {
    return fpb::norm_interval_from(r.max_abs[i], r.exponent[i], r.scaled_sumsq[i], r.count[i],
                                   r.nonfinite[i] == 0);
}

__device__ double euclid(const NormResult& r, int i) {
    if (r.nonfinite[i]) return __builtin_nan("");
    if (r.max_abs[i] == 0.0) return 0.0;
    return scalbn(sqrt(r.scaled_sumsq[i]), r.exponent[i]);
}

__device__ void nominal_contract(ValidationOutput& r, double bnorm, double reg, double tol,
                                 bool has_ridge, double ridge_bound) {
    const double rr = sqrt(reg);
    r.augmented_residual_norm = hypot(r.residual_norm, rr * r.solution_norm);
    r.augmented_operator_norm_lower_bound = hypot(r.operator_norm_lower_bound, rr);
    r.compatible_backward_error_upper_bound = ratio_cert(
        r.augmented_residual_norm, r.augmented_operator_norm_lower_bound * r.solution_norm + bnorm);
    r.least_squares_backward_error_upper_bound = ratio_cert(
        r.normal_residual_norm, r.augmented_operator_norm_lower_bound * r.augmented_residual_norm);
    r.backward_error_upper_bound = fmin(r.compatible_backward_error_upper_bound,
                                        r.least_squares_backward_error_upper_bound);
    const double opl = r.operator_norm_lower_bound;
    r.relative_normal_residual_upper_bound =
        ratio_cert(r.normal_residual_norm, (opl * opl + reg) * r.solution_norm + opl * bnorm);
    if (reg > 0.0) {
        const double req = has_ridge ? ridge_bound : r.normal_residual_norm / rr;
        r.energy_error_upper_bound = req >= 0.0 ? req : kInf;
        r.objective_gap_upper_bound = r.energy_error_upper_bound * r.energy_error_upper_bound;
        r.relative_energy_error_upper_bound =
            rel_energy(r.energy_error_upper_bound, r.solution_energy_norm);
    } else if (r.normal_residual_norm == 0.0) {
        r.energy_error_upper_bound = r.relative_energy_error_upper_bound = 0.0;
        r.objective_gap_upper_bound = 0.0;
    } else {
        r.energy_error_upper_bound = r.relative_energy_error_upper_bound = kInf;
        r.objective_gap_upper_bound = kInf;
    }
    auto fin = [](double v) { return isfinite(v) && v >= 0.0; };
    if (!(fin(bnorm) && fin(r.residual_norm) && fin(r.augmented_residual_norm) &&
          fin(r.normal_residual_norm) && fin(r.solution_norm) && fin(r.solution_energy_norm) &&
          fin(r.objective) && fin(r.operator_norm_lower_bound) &&
          fin(r.augmented_operator_norm_lower_bound))) {
        r.status = ST_BREAKDOWN;
        r.stop_reason = SR_BREAKDOWN;
        return;
    }
    const bool passed = reg > 0.0 ? r.relative_energy_error_upper_bound <= tol
                                  : r.backward_error_upper_bound <= tol;
    r.status = passed ? ST_SUCCESS : ST_WORK;
    if (r.normal_residual_norm == 0.0) r.stop_reason = SR_EXACT;
    else if (passed && reg > 0.0) r.stop_reason = SR_ENERGY;
    else if (passed && r.compatible_backward_error_upper_bound <=
                           r.least_squares_backward_error_upper_bound)
        r.stop_reason = SR_COMPAT;
    else if (passed) r.stop_reason = SR_LS;
    else r.stop_reason = SR_DEPTH;
}

__device__ void certified_contract(ValidationOutput& r, const Envelope& e, double reg, double tol,
                                   bool has_ridge, double ridge_bound) {
    if (!e.certified) {
        r.compatible_backward_error_upper_bound = kInf;
        r.least_squares_backward_error_upper_bound = kInf;
        r.backward_error_upper_bound = kInf;
        r.relative_normal_residual_upper_bound = kInf;
        r.energy_error_upper_bound = kInf;
        r.relative_energy_error_upper_bound = kInf;
        r.objective_gap_upper_bound = kInf;
        r.status = ST_WORK;
        r.stop_reason = SR_DEPTH;
        return;
    }
    const Interval sol{e.sol_lower, e.sol_upper};
    const Interval res{e.res_lower, e.res_upper};
    const Interval aug = augmented(res, sol, reg);
    const double opl = r.operator_norm_lower_bound;
    r.augmented_operator_norm_lower_bound =
        fpb::down_sqrt(fpb::down_add(fpb::down_mul(opl, opl), reg));
    const double aopl = r.augmented_operator_norm_lower_bound;
    r.compatible_backward_error_upper_bound =
        fpb::up_div(aug.upper, fpb::down_add(fpb::down_mul(aopl, e.sol_lower), e.b_lower));
    r.least_squares_backward_error_upper_bound =
        fpb::up_div(e.grad_upper, fpb::down_mul(aopl, aug.lower));
    r.backward_error_upper_bound = fmin(r.compatible_backward_error_upper_bound,
                                        r.least_squares_backward_error_upper_bound);
    r.relative_normal_residual_upper_bound = fpb::up_div(
        e.grad_upper,
        fpb::down_add(fpb::down_mul(fpb::down_add(fpb::down_mul(opl, opl), reg), e.sol_lower),
                      fpb::down_mul(opl, e.b_lower)));
    if (reg > 0.0) {
        const double base = fpb::up_div(e.grad_upper, fpb::down_sqrt(reg));
        r.energy_error_upper_bound = has_ridge ? ridge_bound : base;
        r.objective_gap_upper_bound =
            fpb::up_mul(r.energy_error_upper_bound, r.energy_error_upper_bound);
        r.relative_energy_error_upper_bound = fpb::up_div(
            r.energy_error_upper_bound, fpb::down_diff(e.energy_lower, r.energy_error_upper_bound));
    } else if (e.grad_upper == 0.0) {
        r.energy_error_upper_bound = r.relative_energy_error_upper_bound = 0.0;
        r.objective_gap_upper_bound = 0.0;
    } else {
        r.energy_error_upper_bound = r.relative_energy_error_upper_bound = kInf;
        r.objective_gap_upper_bound = kInf;
    }
    const bool passed = e.grad_upper == 0.0 ||
                        (reg > 0.0 ? r.relative_energy_error_upper_bound <= tol
                                   : r.backward_error_upper_bound <= tol);
    r.status = passed ? ST_SUCCESS : ST_WORK;
    if (e.grad_upper == 0.0) r.stop_reason = SR_EXACT;
    else if (passed && reg > 0.0) r.stop_reason = SR_ENERGY;
    else if (passed && r.compatible_backward_error_upper_bound <=
                           r.least_squares_backward_error_upper_bound)
        r.stop_reason = SR_COMPAT;
    else if (passed) r.stop_reason = SR_LS;
    else r.stop_reason = SR_DEPTH;
}

// nr slots: 0 b, 1 x, 2 Ax, 3 r, 4 A^T r, 5 g
__device__ void fill_norms(ValidationOutput& r, const NormResult& nr, double reg) {
    const double an = euclid(nr, 2);
    r.residual_norm = euclid(nr, 3);
    r.normal_residual_norm = euclid(nr, 5);
    r.solution_norm = euclid(nr, 1);
    r.solution_energy_norm = hypot(an, sqrt(reg) * r.solution_norm);
    r.objective = r.residual_norm * r.residual_norm + reg * r.solution_norm * r.solution_norm;
}

__global__ void base_contract_kernel(ValState* vs, Model mdl, long long m, long long n,
                                     double reg, double tol, int can_refine) {
    if (threadIdx.x != 0) return;
    ValidationOutput& r = vs->out;
    const NormResult& nr = vs->nr;
    r.ridge_base_energy_error_upper_bound = __builtin_nan("");
    r.ridge_corrected_energy_error_upper_bound = __builtin_nan("");
    r.ridge_correction_gamma = __builtin_nan("");
    r.ridge_correction_z_h_z = __builtin_nan("");
    r.ridge_correction_two_abs_z_t_q = __builtin_nan("");
    r.ridge_correction_q_norm_squared = __builtin_nan("");
    r.ridge_correction_disposition = RC_NA;
    r.operator_norm_lower_bound = 0.0;
    fill_norms(r, nr, reg);
    vs->bnorm = euclid(nr, 0);
    nominal_contract(r, vs->bnorm, reg, tol, false, 0.0);
    vs->need_refine = 0;
    const bool finite = !nr.nonfinite[1] && !nr.nonfinite[2] && !nr.nonfinite[3] &&
                        !nr.nonfinite[4] && !nr.nonfinite[5];
    Envelope& e = vs->env;
    memset(&e, 0, sizeof(e));
    e.op_upper = mdl.upper;
    e.res_upper = e.grad_upper = e.sol_upper = e.grad_radius = kInf;
    if (!finite || r.status == ST_BREAKDOWN || r.stop_reason == SR_BREAKDOWN) {
        r.status = ST_BREAKDOWN;
        r.stop_reason = SR_BREAKDOWN;
        return;
    }
    if (model_ok(mdl)) {
        const Interval bn = nint(nr, 0), xn = nint(nr, 1), an = nint(nr, 2), rn = nint(nr, 3);
        const Interval tn = nint(nr, 4), gn = nint(nr, 5);
        const double apply_err = callback_radius(mdl, false, xn.upper, m, fpb::kUnitRoundoff);
        const double sub_err = one_op_radius(rn.upper, an.upper > 0.0 || bn.upper > 0.0, m,
                                             fpb::kUnitRoundoff);
        const double res_err = fpb::up_add(apply_err, sub_err);
        const Interval true_res = enlarge(rn, res_err);
        const double t_err = callback_radius(mdl, true, rn.upper, n, fpb::kUnitRoundoff);
        const double ridge_err = one_op_radius(gn.upper, reg > 0.0 && xn.upper > 0.0, n,
                                               fpb::kUnitRoundoff);
        const double prop = fpb::up_mul(e.op_upper, res_err);
        const double g_err = fpb::up_add(fpb::up_add(t_err, prop), ridge_err);
        const Interval true_g = enlarge(gn, g_err);
        const Interval true_a = enlarge(an, apply_err);
        double opl = mdl.lower;
        if (xn.upper > 0.0)
            opl = fmax(opl, fpb::down_div(fpb::down_diff(an.lower, apply_err), xn.upper));
        if (rn.upper > 0.0)
            opl = fmax(opl, fpb::down_div(fpb::down_diff(tn.lower, t_err), rn.upper));
        const Interval energy = augmented(true_a, xn, reg);
        e.res_lower = true_res.lower;
        e.res_upper = true_res.upper;
        e.grad_upper = true_g.upper;
        e.sol_lower = xn.lower;
        e.sol_upper = xn.upper;
        e.b_lower = fmax(0.0, bn.lower);
        e.energy_lower = energy.lower;
        e.grad_radius = g_err;
        e.certified = isfinite(e.res_upper) && isfinite(e.grad_upper) && isfinite(e.sol_upper) &&
                      isfinite(e.op_upper);
        e.op_lower = opl;
    }
    r.operator_norm_lower_bound = e.op_lower;
    certified_contract(r, e, reg, tol, false, 0.0);
    vs->need_refine = can_refine && r.status != ST_SUCCESS && e.certified &&
                      e.grad_radius >= r.normal_residual_norm;
}

// refined vectors in nr2: 0 b, 1 x, 2 applied, 3 residual, 4 transposed, 5 gradient
__global__ void refined_contract_kernel(ValState* vs, Model mdl, long long m, long long n,
                                        double reg, double tol) {
    if (threadIdx.x != 0) return;
    ValidationOutput& r = vs->out;
    const NormResult& nr = vs->nr2;
    vs->need_refine = 0;  // reused as "refinement accepted"
    if (!vs->finite_flag || !model_ok(mdl)) return;
    for (int i = 2; i < 6; ++i)
        if (nr.nonfinite[i]) return;
    const Interval bn = nint(nr, 0), xn = nint(nr, 1);
    if (!isfinite(bn.upper) || !isfinite(xn.upper)) return;
    const Interval san = nint(nr, 2), srn = nint(nr, 3), stn = nint(nr, 4), sgn = nint(nr, 5);
    const double u = fpb::kUnitRoundoff;
    const double a_cast = one_op_radius(san.upper, true, m, u);
    const double a_acc = dd_callback_radius(mdl, n, xn.upper, m);
    const double a_err = fpb::up_add(a_acc, a_cast);
    const double r_cast = one_op_radius(srn.upper, true, m, u);
    const double lr_up = fpb::up_add(srn.upper, r_cast);
    const double r_sub = one_op_radius(lr_up, san.upper > 0.0 || bn.upper > 0.0, m, kDDUnit);
    const double lr_err = fpb::up_add(a_acc, r_sub);
    const double sr_err = fpb::up_add(lr_err, r_cast);
    const double t_cast = one_op_radius(stn.upper, true, n, u);
    const double t_acc = dd_callback_radius(mdl, m, lr_up, n);
    const double g_cast = one_op_radius(sgn.upper, true, n, u);
    const double lg_up = fpb::up_add(sgn.upper, g_cast);
    const double rs_err = one_op_radius(lg_up, reg > 0.0 && xn.upper > 0.0, n, kDDUnit);
    const double prop = fpb::up_mul(mdl.upper, lr_err);
    const double g_err = fpb::up_add(fpb::up_add(t_acc, prop), fpb::up_add(rs_err, g_cast));
    const Interval ta = enlarge(san, a_err), tr = enlarge(srn, sr_err), tg = enlarge(sgn, g_err);
    double opl = mdl.lower;
    if (xn.upper > 0.0) opl = fmax(opl, fpb::down_div(fpb::down_diff(san.lower, a_err), xn.upper));
    if (srn.upper > 0.0) {
        const double conv = fpb::up_mul(mdl.upper, r_cast);
        const double terr = fpb::up_add(fpb::up_add(t_acc, t_cast), conv);
        opl = fmax(opl, fpb::down_div(fpb::down_diff(stn.lower, terr), srn.upper));
    }
    const Interval energy = augmented(ta, xn, reg);
    Envelope e;
    memset(&e, 0, sizeof(e));
    e.op_upper = mdl.upper;
    e.op_lower = opl;
    e.res_lower = tr.lower;
    e.res_upper = tr.upper;
    e.grad_upper = tg.upper;
    e.sol_lower = xn.lower;
    e.sol_upper = xn.upper;
    e.b_lower = fmax(0.0, bn.lower);
    e.energy_lower = energy.lower;
    e.grad_radius = g_err;
    e.certified = isfinite(e.res_upper) && isfinite(e.grad_upper) && isfinite(e.sol_upper) &&
                  isfinite(e.op_upper);
    if (!e.certified) return;
    vs->env = e;
    vs->need_refine = 1;
    fill_norms(r, nr, reg);
    nominal_contract(r, vs->bnorm, reg, tol, false, 0.0);
    r.operator_norm_lower_bound = e.op_lower;
    certified_contract(r, e, reg, tol, false, 0.0);
}

__global__ void ridge_prelim_kernel(ValState* vs, double reg) {
    if (threadIdx.x != 0) return;
    ValidationOutput& r = vs->out;
    const Envelope& e = vs->env;
    vs->need_correction = 0;
    if (!(reg > 0.0) || r.status == ST_BREAKDOWN) return;
    r.ridge_base_energy_error_upper_bound = r.energy_error_upper_bound;
    if (r.status == ST_SUCCESS) r.ridge_correction_disposition = RC_SKIP_PASS;
    else if (!e.certified) r.ridge_correction_disposition = RC_SKIP_NONFINITE;
    else if (e.energy_lower == 0.0) r.ridge_correction_disposition = RC_SKIP_ZERO;
    else if (!(e.grad_upper > 0.0) || !isfinite(e.grad_upper))
        r.ridge_correction_disposition = RC_SKIP_NONFINITE;
    else {
        const double gn = r.normal_residual_norm;
        if (!(gn > 0.0) || !isfinite(gn) || vs->nr.nonfinite[5]) {
            r.ridge_correction_disposition = RC_SKIP_NONFINITE;
            return;
        }
        r.ridge_correction_disposition = RC_NONFINITE;
        vs->corr_gnorm = gn;
        vs->need_correction = 1;
    }
}

// correction stage scalars; nr2 slots: 0 d, 1 Ad, 2 h, 3 q
__global__ void correction_step_kernel(ValState* vs, Model mdl, long long m, long long n,
                                       double reg, int stage) {
    if (threadIdx.x != 0) return;
    ValidationOutput& r = vs->out;
    const NormResult& nr = vs->nr2;
    if (stage == 0) {  // after d and A d
        if (nr.nonfinite[0]) {
            r.ridge_correction_disposition = RC_SKIP_NONFINITE;
            vs->need_correction = 0;
            return;
        }
        if (nr.nonfinite[1]) {
            r.ridge_correction_disposition = RC_PARTIAL;
            vs->need_correction = 0;
            return;
        }
        const Interval dn = nint(nr, 0), adn = nint(nr, 1);
        vs->corr_dn_upper = dn.upper;
        vs->corr_adn_upper = adn.upper;
        vs->corr_ad_err = callback_radius(mdl, false, dn.upper, m, fpb::kUnitRoundoff);
        return;
    }
    if (stage == 1) {  // after h = A^T A d + lambda d and d.h
        if (nr.nonfinite[2]) {
            vs->need_correction = 0;  // RC_NONFINITE stays
            return;
        }
        const Interval hn = nint(nr, 2);
        const double t_err = callback_radius(mdl, true, vs->corr_adn_upper, n, fpb::kUnitRoundoff);
        const double prop = fpb::up_mul(vs->env.op_upper, vs->corr_ad_err);
        const double hsum = one_op_radius(hn.upper, reg > 0.0 && vs->corr_dn_upper > 0.0, n,
                                          fpb::kUnitRoundoff);
        vs->corr_hn_upper = hn.upper;
        vs->corr_herr = fpb::up_add(fpb::up_add(t_err, prop), hsum);
        const double curv = vs->dot;
        if (!isfinite(curv)) {
            vs->need_correction = 0;
            return;
        }
        if (!(curv > 0.0)) {
            r.ridge_correction_disposition = RC_BAD_CURVATURE;
            vs->need_correction = 0;
            return;
        }
        const double step = vs->corr_gnorm / curv;
        if (!(step > 0.0) || !isfinite(step)) {
            vs->need_correction = 0;
            return;
        }
        vs->corr_step = step;
        return;
    }
    // stage 2: after q = g - step h
    if (nr.nonfinite[3]) {
        vs->need_correction = 0;
        return;
    }
    const Interval qn = nint(nr, 3);
    const double step = vs->corr_step;
    const double curv = vs->dot;
    const double axpy_err = one_op_radius(qn.upper, vs->corr_gnorm > 0.0 && vs->corr_hn_upper > 0.0,
                                          n, fpb::kUnitRoundoff);
    const double q_err =
        fpb::up_add(fpb::up_add(vs->env.grad_radius, fpb::up_mul(step, vs->corr_herr)), axpy_err);
    const double q_up = fpb::up_add(qn.upper, q_err);
    const double ad_true = fpb::up_add(vs->corr_adn_upper, vs->corr_ad_err);
    const double step2 = fpb::up_mul(step, step);
    const double dn = vs->corr_dn_upper;
    const double de2 = fpb::up_add(fpb::up_mul(ad_true, ad_true), fpb::up_mul(reg, fpb::up_mul(dn, dn)));
    const double zhz = fpb::up_mul(step2, de2);
    const double two_cross = fpb::up_mul(2.0, fpb::up_mul(step, fpb::up_mul(dn, q_up)));
    const double qsq = fpb::up_mul(q_up, q_up);
    const double corrected =
        fpb::up_sqrt(fpb::up_add(zhz, fpb::up_add(two_cross, fpb::up_div(qsq, reg))));
    vs->need_correction = 0;
    if (isnan(corrected)) return;
    r.ridge_corrected_energy_error_upper_bound = corrected;
    r.ridge_correction_gamma = 1.0 / curv;
    r.ridge_correction_z_h_z = zhz;
    r.ridge_correction_two_abs_z_t_q = two_cross;
    r.ridge_correction_q_norm_squared = qsq;
    r.ridge_correction_disposition = RC_NOT_IMPROVED;
}

__global__ void finish_kernel(ValState* vs, double reg, double tol) {
    if (threadIdx.x != 0) return;
    ValidationOutput& r = vs->out;
    if (r.ridge_correction_disposition == RC_NOT_IMPROVED &&
        isfinite(r.ridge_corrected_energy_error_upper_bound) &&
        r.ridge_corrected_energy_error_upper_bound < r.energy_error_upper_bound) {
        r.ridge_correction_disposition = RC_IMPROVED;
        certified_contract(r, vs->env, reg, tol, true, r.ridge_corrected_energy_error_upper_bound);
    }
    if (reg > 0.0 && r.status == ST_BREAKDOWN) {
        r.ridge_base_energy_error_upper_bound =
            isnan(r.normal_residual_norm) ? __builtin_nan("") : kInf;
        r.energy_error_upper_bound = r.ridge_base_energy_error_upper_bound;
        r.relative_energy_error_upper_bound = kInf;
        r.objective_gap_upper_bound = kInf;
        r.ridge_correction_disposition = RC_SKIP_NONFINITE;
    }
}

// ------------------------------------------------------ vector kernels ----

__global__ void sub_kernel(const double* a, const double* b, double* out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = a[i] - b[i];
}

__global__ void fma_kernel(double lambda, const double* x, const double* t, double* out,
                           long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = fma(lambda, x[i], t[i]);
}

// refinement: residual r = (la - b) in double-double; outputs hi (stored
// double) and lo (carried into A^T)
__global__ void dd_residual_kernel(const double* la_hi, const double* la_lo, const double* b,
                                   double* r_hi, double* r_lo, long long m, int* finite) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x) {
        const dd v = dd_add(dd{la_hi[i], la_lo[i]}, dd{-b[i], 0.0});
        r_hi[i] = v.hi;
        r_lo[i] = v.lo;
        if (!isfinite(v.hi) || !isfinite(v.lo)) atomicAnd(finite, 0);
    }
}

__global__ void dd_gradient_kernel(double lambda, const double* x, const double* t_hi,
                                   const double* t_lo, double* g, long long n, int* finite) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double p = lambda * x[i];
        const double pe = fma(lambda, x[i], -p);
        const dd v = dd_add(dd{t_hi[i], t_lo[i]}, dd{p, pe});
        g[i] = v.hi;
        if (!isfinite(v.hi) || !isfinite(v.lo)) atomicAnd(finite, 0);
    }
}

__global__ void scale_kernel(const double* g, const ValState* vs, double* d, long long n) {
    const double s = vs->corr_gnorm;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        d[i] = g[i] / s;
}

__global__ void dot_kernel(const double* a, const double* b, long long n, double* partials,
                           unsigned* ticket, double* out) {
    __shared__ double red[32];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        s = fma(a[i], b[i], s);
    s = block_sum(s, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
    if (arrive_last(ticket, gridDim.x)) {
        double t = 0.0;
        for (unsigned b2 = threadIdx.x; b2 < gridDim.x; b2 += blockDim.x) t += partials[b2];
        t = block_sum(t, red);
        if (threadIdx.x == 0) *out = t;
    }
}

__global__ void correction_q_kernel(const double* h, const double* g, const ValState* vs,
                                    double* q, long long n) {
    const double step = vs->corr_step;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        q[i] = fma(-step, h[i], g[i]);
}

int vgrid(long long n) {
    return (int)std::max<long long>(1, std::min<long long>(grid_cap(), (n + 255) / 256));
}

}  // namespace

struct Validator::Impl {
    const DeviceOperator& op;
    const double* b;
    double reg;
    cudaStream_t stream;
    long long m, n;
    Model mdl{};
    ValState* vs = nullptr;
    double *ax = nullptr, *r = nullptr, *atr = nullptr, *g = nullptr;
    double *hi1 = nullptr, *lo1 = nullptr, *hi2 = nullptr, *lo2 = nullptr;  // refinement
    double *rn_hi = nullptr, *rn_lo = nullptr, *g2 = nullptr;
    double* partials = nullptr;
    unsigned* counters = nullptr;
    cudaEvent_t ev[2];

    Impl(const DeviceOperator& o, const double* bb, double rg, cudaStream_t s)
        : op(o), b(bb), reg(rg), stream(s), m(o.rows()), n(o.cols()) {
        const ValidationModel vm = op.validation_error_model();
        mdl = {vm.norm_upper, vm.norm_lower, vm.apply_steps, vm.transpose_steps};
        stream_alloc(&vs, sizeof(ValState), stream);
        auto alloc = [&](double*& p, long long cnt) {
            stream_alloc(&p, sizeof(double) * std::max<long long>(1, cnt), stream);
        };
        alloc(ax, m);
        alloc(r, m);
        alloc(atr, n);
        alloc(g, n);
        alloc(partials, 2 * kMaxVectors * kMaxGridCap + 8 * kMaxGridCap);
        stream_alloc(&counters, sizeof(unsigned) * 16, stream);
        AMFLS_CUDA(cudaMemsetAsync(counters, 0, sizeof(unsigned) * 16, stream));
        AMFLS_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventBlockingSync));
        AMFLS_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventBlockingSync));
    }
    ~Impl() {
        cudaStreamSynchronize(stream);
        for (double* p : {ax, r, atr, g, hi1, lo1, hi2, lo2, rn_hi, rn_lo, g2, partials}) stream_free(p, stream);
        stream_free(vs, stream);
        stream_free(counters, stream);
        cudaEventDestroy(ev[0]);
        cudaEventDestroy(ev[1]);
    }

    double timed_begin() {
        AMFLS_CUDA(cudaEventRecord(ev[0], stream));
        return 0.0;
    }
    double timed_end() {
        AMFLS_CUDA(cudaEventRecord(ev[1], stream));
        AMFLS_CUDA(cudaEventSynchronize(ev[1]));
        float ms = 0.0f;
        AMFLS_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        return ms * 1e-3;
    }

    void product(bool transpose, const double* x, double* t_out, double* out, const double* minus,
                 const double* fma_vec) {
        Epilogue ep;
        ep.t_out = t_out;
        ep.out = out;
        ep.minus_vec = minus;
        ep.fma_vec = fma_vec;
        ep.lambda = reg;
        ep.partials = partials;
        ep.counter = counters + 8;
        if (op.product1(transpose, x, ep, stream)) return;
        if (transpose) op.apply_transpose(x, 1, t_out, stream);
        else op.apply(x, 1, t_out, stream);
        if (minus) { sub_kernel<<<vgrid(m), 256, 0, stream>>>(t_out, minus, out, m);
            AMFLS_LAUNCHED();
        }
        if (fma_vec) {
            fma_kernel<<<vgrid(n), 256, 0, stream>>>(reg, fma_vec, t_out, out, n);
            AMFLS_LAUNCHED();
        }
    }

    void norms(NormResult* dst, std::initializer_list<std::pair<const double*, long long>> vecs) {
        VectorSet set{};
        for (auto& p : vecs) {
            set.v[set.count] = p.first;
            set.n[set.count] = p.second;
            ++set.count;
        }
        norm_passes(set, dst, partials, counters, stream);
    }

    ValState read() {
        ValState h;
        AMFLS_CUDA(cudaMemcpyAsync(&h, vs, sizeof(ValState), cudaMemcpyDeviceToHost, stream));
        stream_wait(stream);
        return h;
    }

    ValidationOutput run(const double* x, double tol) {
        AMFLS_CUDA(cudaMemsetAsync(vs, 0, sizeof(ValState), stream));
        double sec[6] = {0, 0, 0, 0, 0, 0};
        int calls[6] = {0, 0, 0, 0, 0, 0};
        timed_begin();
        product(false, x, ax, r, b, nullptr);
        sec[0] = timed_end();
        calls[0] = 1;
        timed_begin();
        product(true, r, atr, g, nullptr, x);
        sec[1] = timed_end();
        calls[1] = 1;
        norms(&vs->nr, {{b, m}, {x, n}, {ax, m}, {r, m}, {atr, n}, {g, n}});
        base_contract_kernel<<<1, 32, 0, stream>>>(vs, mdl, m, n, reg, tol,
                                                   op.supports_validation_refinement() ? 1 : 0);
        AMFLS_LAUNCHED();
        ValState h = read();
        const double* grad = g;
        if (h.need_refine) {
            auto alloc = [&](double*& p, long long cnt) {
                if (!p) stream_alloc(&p, sizeof(double) * std::max<long long>(1, cnt), stream);
            };
            alloc(hi1, m);
            alloc(lo1, m);
            alloc(rn_hi, m);
            alloc(rn_lo, m);
            alloc(hi2, n);
            alloc(lo2, n);
            alloc(g2, n);
            int one = 1;
            AMFLS_CUDA(cudaMemcpyAsync(&vs->finite_flag, &one, sizeof(int), cudaMemcpyHostToDevice,
                                       stream));
            timed_begin();
            op.apply_refined(x, nullptr, hi1, lo1, &vs->finite_flag, stream);
            sec[2] = timed_end();
            calls[2] = 1;
            dd_residual_kernel<<<vgrid(m), 256, 0, stream>>>(hi1, lo1, b, rn_hi, rn_lo, m,
                                                             &vs->finite_flag);
            AMFLS_LAUNCHED();
            timed_begin();
            op.apply_transpose_refined(rn_hi, rn_lo, hi2, lo2, &vs->finite_flag, stream);
            sec[3] = timed_end();
            calls[3] = 1;
            dd_gradient_kernel<<<vgrid(n), 256, 0, stream>>>(reg, x, hi2, lo2, g2, n,
                                                             &vs->finite_flag);
            AMFLS_LAUNCHED();
            norms(&vs->nr2, {{b, m}, {x, n}, {hi1, m}, {rn_hi, m}, {hi2, n}, {g2, n}});
            refined_contract_kernel<<<1, 32, 0, stream>>>(vs, mdl, m, n, reg, tol);
            AMFLS_LAUNCHED();
            h = read();
            if (h.need_refine) grad = g2;  // refined vectors replace the base ones
        }
        if (reg > 0.0) {
            ridge_prelim_kernel<<<1, 32, 0, stream>>>(vs, reg);
            AMFLS_LAUNCHED();
            h = read();
            if (h.need_correction) {
                // d = g / ||g||, A d, A^T A d + lambda d, d.h, q = g - step h
                double* d = atr;  // reuse: the base A^T r is no longer needed
                double* ad = ax;
                double* hv = nullptr;
                double* q = nullptr;
                AMFLS_CUDA(cudaMallocAsync(&hv, sizeof(double) * n, stream));
                AMFLS_CUDA(cudaMallocAsync(&q, sizeof(double) * n, stream));
                scale_kernel<<<vgrid(n), 256, 0, stream>>>(grad, vs, d, n);
                AMFLS_LAUNCHED();
                timed_begin();
                product(false, d, ad, ad, nullptr, nullptr);
                sec[4] = timed_end();
                calls[4] = 1;
                norms(&vs->nr2, {{d, n}, {ad, m}});
                correction_step_kernel<<<1, 32, 0, stream>>>(vs, mdl, m, n, reg, 0);
                AMFLS_LAUNCHED();
                h = read();
                if (h.need_correction) {
                    timed_begin();
                    product(true, ad, hv, hv, nullptr, d);  // h = A^T A d + lambda d
                    sec[5] = timed_end();
                    calls[5] = 1;
                    dot_kernel<<<vgrid(n), 256, 0, stream>>>(d, hv, n, partials, counters + 9,
                                                             &vs->dot);
                    AMFLS_LAUNCHED();
                    VectorSet set{};
                    set.v[0] = d; set.n[0] = n;
                    set.v[1] = ad; set.n[1] = m;
                    set.v[2] = hv; set.n[2] = n;
                    set.count = 3;
                    norm_passes(set, &vs->nr2, partials, counters, stream);
                    correction_step_kernel<<<1, 32, 0, stream>>>(vs, mdl, m, n, reg, 1);
                    AMFLS_LAUNCHED();
                    h = read();
                    if (h.need_correction) {
                        correction_q_kernel<<<vgrid(n), 256, 0, stream>>>(hv, grad, vs, q, n);
                        AMFLS_LAUNCHED();
                        VectorSet s2{};
                        s2.v[0] = d; s2.n[0] = n;
                        s2.v[1] = ad; s2.n[1] = m;
                        s2.v[2] = hv; s2.n[2] = n;
                        s2.v[3] = q; s2.n[3] = n;
                        s2.count = 4;
                        norm_passes(s2, &vs->nr2, partials, counters, stream);
                        correction_step_kernel<<<1, 32, 0, stream>>>(vs, mdl, m, n, reg, 2);
                        AMFLS_LAUNCHED();
                    }
                }
                AMFLS_CUDA(cudaFreeAsync(hv, stream));
                AMFLS_CUDA(cudaFreeAsync(q, stream));
            }
        }
        finish_kernel<<<1, 32, 0, stream>>>(vs, reg, tol);
        AMFLS_LAUNCHED();
        h = read();
        ValidationOutput out = h.out;
        for (int i = 0; i < 6; ++i) {
            out.calls[i] = calls[i];
            out.seconds[i] = sec[i];
        }
        return out;
    }
};

Validator::Validator(const DeviceOperator& op, const double* d_b, double regularization,
                     cudaStream_t stream)
    : impl_(new Impl(op, d_b, regularization, stream)) {}

Validator::~Validator() { delete impl_; }

ValidationOutput Validator::validate(const double* d_x, double tolerance) {
    return impl_->run(d_x, tolerance);
}

}  // namespace amfls_gpu
