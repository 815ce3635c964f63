// Kernels and host driver of the learned width controller (width_policy.hpp).
//
// Parameter layout: W1 [H][I] | b1 [H] | W2 [H][H] | b2 [H] | w3 [H] | b3.
// Forward, per sample n:
//   h1 = tanh(W1 x + b1),  h2 = tanh(W2 h1 + b2),  out = w3 . h2 + b3.
// Loss L = (1/N) sum_n (out_n - y_n)^2.  Backward, per sample:
//   d3 = 2 (out - y) / N,  d2 = d3 w3 (1 - h2^2),  d1 = (W2^T d2) (1 - h1^2),
// and the gradient of each parameter sums its per-sample terms over n in
// order (one thread per parameter), e.g. dW2[k][j] = sum_n d2[n][k] h1[n][j].
#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "common.cuh"
#include "width_policy.hpp"

namespace amfls_gpu {
namespace {

constexpr int I = kPolicyInputs;
constexpr int H = kPolicyHidden;
constexpr int kW1 = 0, kB1 = H * I, kW2 = kB1 + H, kB2 = kW2 + H * H, kW3 = kB2 + H,
              kB3 = kW3 + H;
static_assert(kB3 + 1 == kPolicyParams, "parameter layout");

__device__ void forward_one(const double* __restrict__ p, const double* __restrict__ x,
                            double* h1, double* h2, double* out) {
    for (int j = 0; j < H; ++j) {
        double s = p[kB1 + j];
        for (int i = 0; i < I; ++i) s = fma(p[kW1 + j * I + i], x[i], s);
        h1[j] = tanh(s);
    }
    for (int k = 0; k < H; ++k) {
        double s = p[kB2 + k];
        for (int j = 0; j < H; ++j) s = fma(p[kW2 + k * H + j], h1[j], s);
        h2[k] = tanh(s);
    }
    double s = p[kB3];
    for (int k = 0; k < H; ++k) s = fma(p[kW3 + k], h2[k], s);
    *out = s;
}

// Forward pass for n samples, one thread each; activations kept for the
// backward pass when h1 / h2 are given.
__global__ void forward_kernel(const double* p, const double* x, int n, double* h1, double* h2,
                               double* out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    double a1[H], a2[H];
    forward_one(p, x + (long long)s * I, a1, a2, out + s);
    if (h1)
        for (int j = 0; j < H; ++j) h1[(long long)s * H + j] = a1[j];
    if (h2)
        for (int k = 0; k < H; ++k) h2[(long long)s * H + k] = a2[k];
}

// Per-sample deltas and squared errors.
__global__ void delta_kernel(const double* p, const double* h1, const double* h2,
                             const double* out, const double* y, int n, double* d1, double* d2,
                             double* d3, double* sq) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const double e = out[s] - y[s];
    sq[s] = e * e;
    const double g3 = 2.0 * e / n;
    d3[s] = g3;
    double g2[H];
    for (int k = 0; k < H; ++k) {
        const double a = h2[(long long)s * H + k];
        g2[k] = g3 * p[kW3 + k] * (1.0 - a * a);
        d2[(long long)s * H + k] = g2[k];
    }
    for (int j = 0; j < H; ++j) {
        double t = 0.0;
        for (int k = 0; k < H; ++k) t = fma(p[kW2 + k * H + j], g2[k], t);
        const double a = h1[(long long)s * H + j];
        d1[(long long)s * H + j] = t * (1.0 - a * a);
    }
}

// One thread per parameter: its gradient summed over the samples in order.
__global__ void grad_kernel(const double* x, const double* h1, const double* h2,
                            const double* d1, const double* d2, const double* d3, int n,
                            double* grad) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= kPolicyParams) return;
    double g = 0.0;
    if (q < kB1) {
        const int j = q / I, i = q % I;
        for (int s = 0; s < n; ++s) g = fma(d1[(long long)s * H + j], x[(long long)s * I + i], g);
    } else if (q < kW2) {
        const int j = q - kB1;
        for (int s = 0; s < n; ++s) g += d1[(long long)s * H + j];
    } else if (q < kB2) {
        const int k = (q - kW2) / H, j = (q - kW2) % H;
        for (int s = 0; s < n; ++s) g = fma(d2[(long long)s * H + k], h1[(long long)s * H + j], g);
    } else if (q < kW3) {
        const int k = q - kB2;
        for (int s = 0; s < n; ++s) g += d2[(long long)s * H + k];
    } else if (q < kB3) {
        const int k = q - kW3;
        for (int s = 0; s < n; ++s) g = fma(d3[s], h2[(long long)s * H + k], g);
    } else {
        for (int s = 0; s < n; ++s) g += d3[s];
    }
    grad[q] = g;
}

// Adam (Kingma & Ba, ICLR 2015), bias-corrected, step t >= 1.
__global__ void adam_kernel(double* p, const double* g, double* m, double* v, int t, double lr) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= kPolicyParams) return;
    constexpr double b1 = 0.9, b2 = 0.999, eps = 1e-8;
    const double mq = b1 * m[q] + (1.0 - b1) * g[q];
    const double vq = b2 * v[q] + (1.0 - b2) * g[q] * g[q];
    m[q] = mq;
    v[q] = vq;
    const double mh = mq / (1.0 - pow(b1, (double)t));
    const double vh = vq / (1.0 - pow(b2, (double)t));
    p[q] -= lr * mh / (sqrt(vh) + eps);
}

// Sum of n values in one thread (fixed order).
__global__ void sum_kernel(const double* v, int n, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += v[i];
    *out = s;
}

int blocks(long long n) { return (int)std::max<long long>(1, (n + 127) / 128); }

struct Buffers {
    double *x = nullptr, *y = nullptr, *h1 = nullptr, *h2 = nullptr, *out = nullptr;
    double *d1 = nullptr, *d2 = nullptr, *d3 = nullptr, *sq = nullptr;
    double *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr, *loss = nullptr;
    Buffers(int n, const double* hx, const double* hy, const std::vector<double>& params,
            cudaStream_t s) {
        if (n <= 0) throw std::invalid_argument("training needs at least one sample");
        if ((int)params.size() != kPolicyParams)
            throw std::invalid_argument("policy parameter vector has the wrong length");
        const size_t nn = n;
        try {
            AMFLS_CUDA(cudaMalloc(&x, sizeof(double) * nn * I));
            AMFLS_CUDA(cudaMalloc(&y, sizeof(double) * nn));
            AMFLS_CUDA(cudaMalloc(&h1, sizeof(double) * nn * H));
            AMFLS_CUDA(cudaMalloc(&h2, sizeof(double) * nn * H));
            AMFLS_CUDA(cudaMalloc(&out, sizeof(double) * nn));
            AMFLS_CUDA(cudaMalloc(&d1, sizeof(double) * nn * H));
            AMFLS_CUDA(cudaMalloc(&d2, sizeof(double) * nn * H));
            AMFLS_CUDA(cudaMalloc(&d3, sizeof(double) * nn));
            AMFLS_CUDA(cudaMalloc(&sq, sizeof(double) * nn));
            AMFLS_CUDA(cudaMalloc(&p, sizeof(double) * kPolicyParams));
            AMFLS_CUDA(cudaMalloc(&g, sizeof(double) * kPolicyParams));
            AMFLS_CUDA(cudaMalloc(&m, sizeof(double) * kPolicyParams));
            AMFLS_CUDA(cudaMalloc(&v, sizeof(double) * kPolicyParams));
            AMFLS_CUDA(cudaMalloc(&loss, sizeof(double)));
            AMFLS_CUDA(cudaMemcpyAsync(x, hx, sizeof(double) * nn * I, cudaMemcpyHostToDevice, s));
            if (hy)
                AMFLS_CUDA(cudaMemcpyAsync(y, hy, sizeof(double) * nn, cudaMemcpyHostToDevice, s));
            AMFLS_CUDA(cudaMemcpyAsync(p, params.data(), sizeof(double) * kPolicyParams,
                                       cudaMemcpyHostToDevice, s));
            AMFLS_CUDA(cudaMemsetAsync(m, 0, sizeof(double) * kPolicyParams, s));
            AMFLS_CUDA(cudaMemsetAsync(v, 0, sizeof(double) * kPolicyParams, s));
        } catch (...) {  // free what was allocated before the failure
            free_all();
            throw;
        }
    }
    ~Buffers() { free_all(); }
    void free_all() noexcept {
        for (double* q : {x, y, h1, h2, out, d1, d2, d3, sq, p, g, m, v, loss}) cudaFree(q);
    }
    // forward + backward: gradient in g, loss in *loss
    void step(int n, cudaStream_t s) {
        forward_kernel<<<blocks(n), 128, 0, s>>>(p, x, n, h1, h2, out);
        AMFLS_LAUNCHED();
        delta_kernel<<<blocks(n), 128, 0, s>>>(p, h1, h2, out, y, n, d1, d2, d3, sq);
        AMFLS_LAUNCHED();
        grad_kernel<<<blocks(kPolicyParams), 128, 0, s>>>(x, h1, h2, d1, d2, d3, n, g);
        AMFLS_LAUNCHED();
    }
    double loss_value(int n, cudaStream_t s) {
        sum_kernel<<<1, 32, 0, s>>>(sq, n, loss);
        AMFLS_LAUNCHED();
        double h = 0.0;
        AMFLS_CUDA(cudaMemcpyAsync(&h, loss, sizeof(double), cudaMemcpyDeviceToHost, s));
        AMFLS_CUDA(cudaStreamSynchronize(s));
        return h / n;
    }
};

std::uint64_t splitmix64(std::uint64_t& state) {
    std::uint64_t z = (state += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

}  // namespace

std::vector<double> policy_initial_params(std::uint64_t seed) {
    std::vector<double> p(kPolicyParams, 0.0);
    std::uint64_t st = seed;
    auto uniform = [&](double a) {  // U(-a, a)
        const double u = (double)(splitmix64(st) >> 11) * 0x1p-53;
        return a * (2.0 * u - 1.0);
    };
    const double a1 = std::sqrt(6.0 / (I + H)), a2 = std::sqrt(6.0 / (H + H)),
                 a3 = std::sqrt(6.0 / (H + 1));
    for (int q = kW1; q < kB1; ++q) p[q] = uniform(a1);
    for (int q = kW2; q < kB2; ++q) p[q] = uniform(a2);
    for (int q = kW3; q < kB3; ++q) p[q] = uniform(a3);
    return p;
}

WidthPolicy::WidthPolicy(const std::vector<double>& params) {
    if ((int)params.size() != kPolicyParams)
        throw std::invalid_argument("policy parameter vector has the wrong length");
    for (double v : params)
        if (!std::isfinite(v)) throw std::invalid_argument("policy parameters must be finite");
    try {
        AMFLS_CUDA(cudaMalloc(&params_, sizeof(double) * kPolicyParams));
        AMFLS_CUDA(cudaMalloc(&io_, sizeof(double) * (2 * I + 2)));
        AMFLS_CUDA(cudaMemcpy(params_, params.data(), sizeof(double) * kPolicyParams,
                              cudaMemcpyHostToDevice));
    } catch (...) {  // free what was allocated before the failure
        cudaFree(params_);
        cudaFree(io_);
        throw;
    }
}

WidthPolicy::~WidthPolicy() {
    cudaFree(params_);
    cudaFree(io_);
}

void WidthPolicy::score(const double* features, double* stay, double* widen,
                        cudaStream_t s) const {
    double in[2 * I];
    for (int a = 0; a < 2; ++a) {
        for (int i = 0; i < kPolicyFeatures; ++i) in[a * I + i] = features[i];
        in[a * I + kPolicyFeatures] = a;
    }
    AMFLS_CUDA(cudaMemcpyAsync(io_, in, sizeof(in), cudaMemcpyHostToDevice, s));
    forward_kernel<<<1, 32, 0, s>>>(params_, io_, 2, nullptr, nullptr, io_ + 2 * I);
    AMFLS_LAUNCHED();
    double out[2];
    AMFLS_CUDA(cudaMemcpyAsync(out, io_ + 2 * I, sizeof(out), cudaMemcpyDeviceToHost, s));
    AMFLS_CUDA(cudaStreamSynchronize(s));
    *stay = out[0];
    *widen = out[1];
}

void policy_forward(const std::vector<double>& params, const double* x, int n, double* out,
                    cudaStream_t s) {
    Buffers b(n, x, nullptr, params, s);
    forward_kernel<<<blocks(n), 128, 0, s>>>(b.p, b.x, n, nullptr, nullptr, b.out);
    AMFLS_LAUNCHED();
    AMFLS_CUDA(cudaMemcpyAsync(out, b.out, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    AMFLS_CUDA(cudaStreamSynchronize(s));
}

double policy_gradient(const std::vector<double>& params, const double* x, const double* y,
                       int n, double* grad, cudaStream_t s) {
    Buffers b(n, x, y, params, s);
    b.step(n, s);
    AMFLS_CUDA(cudaMemcpyAsync(grad, b.g, sizeof(double) * kPolicyParams, cudaMemcpyDeviceToHost,
                               s));
    return b.loss_value(n, s);
}

TrainSummary policy_train(std::vector<double>& params, const double* x, const double* y, int n,
                          int epochs, double lr, cudaStream_t s) {
    if (epochs <= 0 || !(lr > 0.0) || !std::isfinite(lr))
        throw std::invalid_argument("training needs epochs > 0 and a positive learning rate");
    Buffers b(n, x, y, params, s);
    TrainSummary r{};
    for (int t = 1; t <= epochs; ++t) {
        b.step(n, s);
        if (t == 1) r.loss_first = b.loss_value(n, s);
        adam_kernel<<<blocks(kPolicyParams), 128, 0, s>>>(b.p, b.g, b.m, b.v, t, lr);
        AMFLS_LAUNCHED();
    }
    forward_kernel<<<blocks(n), 128, 0, s>>>(b.p, b.x, n, b.h1, b.h2, b.out);
    AMFLS_LAUNCHED();
    delta_kernel<<<blocks(n), 128, 0, s>>>(b.p, b.h1, b.h2, b.out, b.y, n, b.d1, b.d2, b.d3, b.sq);
    AMFLS_LAUNCHED();
    r.loss_last = b.loss_value(n, s);
    r.epochs = epochs;
    AMFLS_CUDA(cudaMemcpyAsync(params.data(), b.p, sizeof(double) * kPolicyParams,
                               cudaMemcpyDeviceToHost, s));
    AMFLS_CUDA(cudaStreamSynchronize(s));
    return r;
}

}  // namespace amfls_gpu
