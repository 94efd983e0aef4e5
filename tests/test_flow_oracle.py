"""The CPU restatement of the flow loss: its analytic gradient agrees with
central finite differences (so it can check the CUDA training kernels)."""
import numpy as np

from oracle import flow_oracle as F


def test_flow_oracle_gradient_matches_finite_differences():
    d, L, W, H = 5, 4, 8, 2
    _, n = F.layout(d, L, W, H)
    rng = np.random.default_rng(0)
    p = rng.normal(size=n) * 0.3
    x = rng.normal(size=(16, d))
    _, g = F.loss_grad(p, x, d, L, W, H)
    eps = 1e-6
    idx = rng.choice(n, 40, replace=False)
    fd = []
    for i in idx:
        e = np.zeros(n)
        e[i] = eps
        fd.append((F.loss_grad(p + e, x, d, L, W, H)[0] - F.loss_grad(p - e, x, d, L, W, H)[0]) / (2 * eps))
    assert np.abs(np.array(fd) - g[idx]).max() <= 1e-7 * np.abs(g).max()


def test_flow_oracle_identity_at_zero_output_layer():
    d, L, W, H = 4, 2, 8, 2
    lay, n = F.layout(d, L, W, H)
    p = np.random.default_rng(1).normal(size=n)
    for (_, _, _, _, dense) in lay:  # zero the output layers: identity map
        w0, kin, kout, b = dense[-1]
        p[w0:b + kout] = 0
    x = np.random.default_rng(2).normal(size=(10, d))
    loss, _ = F.loss_grad(p, x, d, L, W, H)
    assert abs(loss - np.mean(0.5 * np.sum(x * x, 1))) < 1e-12
