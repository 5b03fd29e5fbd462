"""The numpy MLP reference's analytic gradient (used to check the tensor-core training kernel)
against central finite differences of its own float64 loss."""
import numpy as np

from mlp_ref import BLOCKS, NIN, K1, he_params, loss_grad


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(11)
    p = he_params(rng).astype(np.float64)
    x = rng.standard_normal((40, NIN))
    t = rng.standard_normal(40)
    _, g = loss_grad(p, x, t, rounded=False)
    eps = 1e-6
    for name, sl in BLOCKS.items():
        idx = np.arange(sl.start, sl.stop)
        if name == "W1":  # padded input columns carry no gradient
            idx = idx[(idx - sl.start) % K1 < NIN]
        for k in rng.choice(idx, size=min(6, len(idx)), replace=False):
            q = p.copy()
            q[k] += eps
            lp, _ = loss_grad(q, x, t, rounded=False)
            q[k] -= 2 * eps
            lm, _ = loss_grad(q, x, t, rounded=False)
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(g[k]), (name, k, fd, g[k])


def test_padded_input_columns_have_zero_gradient():
    rng = np.random.default_rng(3)
    p = he_params(rng)
    _, g = loss_grad(p, rng.standard_normal((16, NIN)), rng.standard_normal(16))
    w1 = g[BLOCKS["W1"]].reshape(-1, K1)
    assert np.all(w1[:, NIN:] == 0)
