"""CPU restatement of the learned width controller's network -- test
infrastructure only (the checker of the CUDA kernels; nothing in the
product imports it).

The learned controller has no counterpart in the reference (its width
controller is the heuristic of src/algorithms/amfls/amfls_internal.hpp);
this module restates, in float64 numpy, the network and loss the CUDA
kernels implement so that their forward pass and gradients can be checked:

    h1 = tanh(W1 x + b1),  h2 = tanh(W2 h1 + b2),  out = w3 . h2 + b3,
    L = mean_n (out_n - y_n)^2,

parameters laid out W1[32][12] | b1[32] | W2[32][32] | b2[32] | w3[32] | b3.
The gradient here is the textbook backward pass; tests/test_oracle_policy.py
pins it against central finite differences.
"""
import numpy as np

I, H = 12, 32
SIZES = [("W1", (H, I)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("w3", (H,)), ("b3", (1,))]
P = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, at = {}, 0
    for name, shape in SIZES:
        k = int(np.prod(shape))
        out[name] = np.asarray(p[at:at + k], dtype=np.float64).reshape(shape)
        at += k
    return out


def forward(p, x):
    w = unpack(p)
    h1 = np.tanh(x @ w["W1"].T + w["b1"])
    h2 = np.tanh(h1 @ w["W2"].T + w["b2"])
    return h2 @ w["w3"] + w["b3"][0], (h1, h2)


def loss_and_grad(p, x, y):
    w = unpack(p)
    out, (h1, h2) = forward(p, x)
    n = x.shape[0]
    e = out - y
    d3 = 2.0 * e / n
    d2 = d3[:, None] * w["w3"][None, :] * (1.0 - h2 ** 2)
    d1 = (d2 @ w["W2"]) * (1.0 - h1 ** 2)
    g = {"W1": d1.T @ x, "b1": d1.sum(0), "W2": d2.T @ h1, "b2": d2.sum(0),
         "w3": h2.T @ d3, "b3": np.array([d3.sum()])}
    return float(np.mean(e ** 2)), np.concatenate([g[name].ravel() for name, _ in SIZES])
