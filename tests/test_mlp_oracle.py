"""The warm-start network's CPU restatement (oracle/mlp_oracle.py) pinned
by finite differences: its gradient is what the device backward kernels
are checked against."""
import numpy as np

from oracle import mlp_oracle as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    p = M.init(3)
    X = rng.standard_normal((7, M.N_IN))
    T = rng.standard_normal((7, M.N_OUT)) * 0.1
    L, g = M.loss_and_grad(p, X, T)
    idx = np.concatenate([rng.choice(p.size, 40, replace=False), np.arange(p.size - M.N_OUT, p.size)])
    h = 1e-6
    for i in idx:
        q = p.copy(); q[i] += h
        lp, _ = M.loss_and_grad(q, X, T)
        q[i] -= 2 * h
        lm, _ = M.loss_and_grad(q, X, T)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8, (i, fd, g[i])


def test_oracle_adam_first_step_moves_by_lr():
    p = M.init(1)
    g = np.linspace(-1, 1, p.size)
    q, m, v = M.adam_step(p, g, np.zeros_like(p), np.zeros_like(p), 1, 1e-3)
    # bias-corrected first step: |delta| = lr for every nonzero gradient component
    d = np.abs(q - p)[np.abs(g) > 1e-3]
    assert np.allclose(d, 1e-3, rtol=1e-4)


def test_oracle_layout_roundtrip():
    p = M.init(2)
    assert p.size == M.n_params() == 32 * 256 + 256 + 256 * 256 + 256 + 21 * 256 + 21
    assert np.array_equal(M.pack(M.unpack(p)), p)
