// Test infrastructure: force-included (g++ -include) into every translation
// unit of the reference build by oracle/Makefile.  It wraps the reference
// controller's two width-decision calls (amfls.cpp:323-354 call
// make_horizon_width_candidate and make_initial_width_candidate,
// amfls_internal.hpp:332-552) so that the driver can record every decision
// the reference takes and, for schedule-replay fixtures, substitute a
// recorded list of decisions.  The wrapped functions themselves are compiled
// unchanged: the header includes them first (they are guarded by
// #pragma once) and only then defines the two function-like macros, so the
// macros rewrite the call sites in amfls.cpp alone.
//
// Only WidthDecision::candidate depends on wall-clock time (through the
// measured operator and local seconds of the cost gate); every other field,
// matched_horizon included, follows from certificates and basis ranks.  So
// replaying the candidate bits makes the whole solve independent of timing.
#pragma once
#ifdef __cplusplus
#include "algorithms/amfls/amfls_internal.hpp"

namespace amfls::detail {
WidthDecision ref_hook_width_decision(WidthDecision decision);
}  // namespace amfls::detail

#define make_horizon_width_candidate(...) \
    ref_hook_width_decision(::amfls::detail::make_horizon_width_candidate(__VA_ARGS__))
#define make_initial_width_candidate(...) \
    ref_hook_width_decision(::amfls::detail::make_initial_width_candidate(__VA_ARGS__))
#endif
