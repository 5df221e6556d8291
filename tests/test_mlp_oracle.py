"""The numpy checker of the learned preconditioner: its analytic gradient
against central finite differences (exact weights), BF16 rounding, and its
PCG against a direct solve."""
import numpy as np

from oracle import mlp


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e-3], dtype=np.float32)
    y = mlp.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == 1.0 + 2 ** -6 and y[3] == -2.5
    assert abs(y[4] - 3.0e-3) / 3.0e-3 < 2 ** -8


def test_gradient_matches_finite_differences():
    P, W, r, lam, us = 5, 7, 2, 1e-3, 0.1
    rng = np.random.default_rng(0)
    n = mlp.layout(P, W, r)[1][-1]
    w = rng.standard_normal(n) * 0.3
    th = rng.uniform(0, 2 * np.pi, (3, P))
    A = rng.standard_normal((3, P, P))
    metric = np.einsum("sij,skj->sik", A, A) / P
    _, g = mlp.loss_grad(w, th, metric, P, W, r, lam, us, round_weights=False)
    idx = rng.choice(n, 40, replace=False)
    for i in idx:
        e = np.zeros(n)
        e[i] = 1e-6
        lp, _ = mlp.loss_grad(w + e, th, metric, P, W, r, lam, us, round_weights=False)
        lm, _ = mlp.loss_grad(w - e, th, metric, P, W, r, lam, us, round_weights=False)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_pcg_matches_direct_solve():
    rng = np.random.default_rng(1)
    P = 30
    B = rng.standard_normal((P, 8))
    A = B @ B.T
    b = rng.standard_normal(P)
    x_cg, it_cg, _ = mlp.pcg(A, b, 1e-2)
    x_ref = np.linalg.solve(A + 1e-2 * np.eye(P), b)
    assert np.linalg.norm(x_cg - x_ref) / np.linalg.norm(x_ref) < 1e-8
    # exact preconditioner M = A + lam I as diag + U U^T: one iteration
    x_p, it_p, _ = mlp.pcg(A, b, 1e-2, d=np.full(P, 1e-2), U=B)
    assert it_p == 1 and np.linalg.norm(x_p - x_ref) / np.linalg.norm(x_ref) < 1e-8
    assert it_cg > it_p
