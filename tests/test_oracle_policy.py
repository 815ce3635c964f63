"""The numpy restatement of the learned controller's network (the checker of
its CUDA kernels) against central finite differences; CPU only."""
import numpy as np

from oracle import width_mlp


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.uniform(-0.4, 0.4, width_mlp.P)
    x = rng.standard_normal((17, width_mlp.I))
    y = rng.standard_normal(17)
    loss, g = width_mlp.loss_and_grad(p, x, y)
    assert g.shape == (width_mlp.P,)
    idx = rng.choice(width_mlp.P, 60, replace=False)
    for q in np.concatenate([idx, [width_mlp.P - 1]]):
        h = 1e-6
        e = np.zeros(width_mlp.P)
        e[q] = h
        fd = (width_mlp.loss_and_grad(p + e, x, y)[0] - width_mlp.loss_and_grad(p - e, x, y)[0]) / (2 * h)
        assert abs(fd - g[q]) <= 1e-7 * max(1.0, abs(fd)), q
    assert np.isclose(loss, np.mean((width_mlp.forward(p, x)[0] - y) ** 2))
