// Learned width controller (no counterpart in the reference).
//
// A small MLP scores the two choices the AMFLS width controller has at each
// widening decision (amfls.cpp:319-359 in the reference: inject the next
// dyadic block of Gaussian seeds, or keep the current width).  Its inputs are
// the controller's own features plus the action; its output is the predicted
// rate at which the certificate falls (decades per second) over the interval
// that follows, standardised.  The controller widens when the predicted rate
// for widening is higher; a non-finite score falls back to the heuristic.
// The FP64 certificate still decides termination, so the network can change
// how fast a solve converges but never what counts as converged.
//
// Network: inputs kPolicyInputs -> tanh(kPolicyHidden) -> tanh(kPolicyHidden)
// -> 1, FP64.  Training (full batch, mean squared error, Adam) and inference
// run as CUDA kernels; gradients are summed per parameter over the samples
// in a fixed order, so training is deterministic.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace amfls_gpu {

constexpr int kPolicyFeatures = 11;  // controller features (without the action)
constexpr int kPolicyInputs = kPolicyFeatures + 1;
constexpr int kPolicyHidden = 32;
// W1 [H][I], b1 [H], W2 [H][H], b2 [H], w3 [H], b3
constexpr int kPolicyParams = kPolicyHidden * kPolicyInputs + kPolicyHidden +
                              kPolicyHidden * kPolicyHidden + kPolicyHidden + kPolicyHidden + 1;

// Feature vector of one decision (see controller.cu for the definitions).
struct DecisionRecord {
    double features[kPolicyFeatures];
    int action;     // 1 = widen, 0 = stay
    int heuristic;  // the plain controller's choice
    double rate;    // decades of certificate per second until the next decision
    int valid;      // rate measured and finite
};

class WidthPolicy {
public:
    explicit WidthPolicy(const std::vector<double>& params);
    ~WidthPolicy();
    WidthPolicy(const WidthPolicy&) = delete;
    WidthPolicy& operator=(const WidthPolicy&) = delete;

    // Scores of (features, stay) and (features, widen); synchronous.
    void score(const double* features, double* stay, double* widen, cudaStream_t s) const;
    const double* device_params() const { return params_; }

private:
    double* params_ = nullptr;
    double* io_ = nullptr;  // 2 input rows + 2 outputs
};

// Deterministic initial parameters (uniform Glorot ranges from splitmix64).
std::vector<double> policy_initial_params(std::uint64_t seed);

// Batch forward pass: x (n x kPolicyInputs, host) -> out (n, host).
void policy_forward(const std::vector<double>& params, const double* x, int n, double* out,
                    cudaStream_t s);

// Loss (mean squared error) and its gradient for one full batch (host I/O).
double policy_gradient(const std::vector<double>& params, const double* x, const double* y,
                       int n, double* grad, cudaStream_t s);

// Adam on the full batch for `epochs` steps from `params` (updated in
// place); returns the losses before and after.
struct TrainSummary {
    double loss_first, loss_last;
    int epochs;
};
TrainSummary policy_train(std::vector<double>& params, const double* x, const double* y, int n,
                          int epochs, double lr, cudaStream_t s);

}  // namespace amfls_gpu
