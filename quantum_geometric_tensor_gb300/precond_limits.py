"""How far a diagonal-plus-rank-r preconditioner can cut PCG iterations on the metric of a
circuit, and whether the map from circuit parameters to it can be learned from samples.

The learned preconditioner (qgt_precond_*) maps theta to M = diag(d) + U U^T.  This module
measures, on exact metrics A = Re Q + lam I of held-out parameter points, the iterations of
PCG (relative residual tol) with

  cg            no preconditioner;
  jacobi        M = diag(A);
  forward       M = diag(A - V L V^T) + V L V^T with the exact top-r eigenpairs (V, L) of A at
                the point itself: the best case of the form the network outputs;
  deflation     M^-1 = diag(A)^-1 + W W^T, W = the r smallest eigenvectors of A at the point
                itself scaled by eigenvalue^-1/2 (the inverse form that targets the small end
                of the spectrum);
  deflation_nn  the same W taken from the training point nearest in (wrapped) theta: what a
                learner that reproduced its training labels exactly would give at that point;
  deflation_at  the same W taken from A(theta + delta) with |delta| = rho, for a sweep of rho:
                the distance over which the smallest eigenspace stays useful;

and the overlap |V_h^T V_o|_F^2 / r of the r-dimensional smallest eigenspaces (1 = the same
subspace, r / P = unrelated subspaces).

`metric_fn(theta[S, P]) -> Re Q[S, P, P]` supplies the metrics (the GPU plan in the benchmark,
the FP64 oracle in the CPU tests).  The reference has no preconditioner: its natural-gradient
solve is unpreconditioned CG (src/quantum_geometric/hybrid/classical_optimization_engine.c:
543-611), the `cg` column here.
"""
from __future__ import annotations

import numpy as np


def pcg_iterations(A, b, minv=None, tol=1e-8, max_iter=5000):
    """PCG iterations for A x = b to |r| <= tol |b| (x0 = 0); minv(r) applies M^-1."""
    x = np.zeros_like(b)
    r = b.copy()
    z = r if minv is None else minv(r)
    p = z.copy()
    rz = r @ z
    bn = np.linalg.norm(b)
    for it in range(max_iter):
        Ap = A @ p
        a = rz / (p @ Ap)
        x += a * p
        r -= a * Ap
        if np.linalg.norm(r) <= tol * bn:
            return it + 1
        z = r if minv is None else minv(r)
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
    return max_iter


def wrapped_distance(a, b):
    """Euclidean distance between parameter vectors with every angle difference wrapped to (-pi, pi]."""
    d = np.angle(np.exp(1j * (np.asarray(a)[..., None, :] - np.asarray(b)[None, ...])))
    return np.sqrt((d * d).sum(-1))


def _small(A, r):
    w, V = np.linalg.eigh(A)
    return w[:r], V[:, :r], w, V


def _deflation_minv(A, w_r, V_r):
    d = np.diag(A).copy()
    W = V_r / np.sqrt(w_r)
    return lambda v: v / d + W @ (W.T @ v)


def _forward_minv(A, r):
    w, V = np.linalg.eigh(A)
    Vt, Lt = V[:, -r:], w[-r:]
    low = (Vt * Lt) @ Vt.T
    d = np.diag(A - low).copy()
    # Woodbury on M = diag(d) + Vt diag(Lt) Vt^T
    Di = 1.0 / d
    K = np.diag(1.0 / Lt) + (Vt.T * Di) @ Vt
    Kinv = np.linalg.inv(K)
    return lambda v: Di * v - Di * (Vt @ (Kinv @ (Vt.T @ (Di * v))))


def analyse(metric_fn, theta_train, theta_heldout, lam=1e-3, r=16, rhos=(0.1, 0.3, 1.0, 3.0),
            tol=1e-8, seed=11, learned=None):
    """Iterations and subspace overlaps on the held-out points (dict of means and per-point lists).

    learned = (d[H, P], U[H, P, r]) adds the network's own M = diag(d) + U U^T as column `learned`."""
    rng = np.random.default_rng(seed)
    th_h = np.atleast_2d(theta_heldout)
    H, P = th_h.shape
    eye = lam * np.eye(P)
    A_h = metric_fn(th_h) + eye
    dist = wrapped_distance(th_h, theta_train)           # H x S
    nn = dist.argmin(1)
    A_nn = metric_fn(np.asarray(theta_train)[nn]) + eye
    # random points of the same space: the typical distance between unrelated parameter points
    th_rand = rng.uniform(0, 2 * np.pi, (H, P))
    d_rand = np.sqrt((np.angle(np.exp(1j * (th_h - th_rand))) ** 2).sum(1))
    A_rand = metric_fn(th_rand) + eye
    pert = {}
    for rho in rhos:
        u = rng.standard_normal((H, P))
        u *= rho / np.linalg.norm(u, axis=1, keepdims=True)
        pert[rho] = metric_fn(th_h + u) + eye
    cols = {k: [] for k in ("cg", "jacobi", "forward", "deflation", "deflation_nn", "deflation_random")}
    cols.update({f"deflation_at_{rho:g}": [] for rho in rhos})
    if learned is not None:
        cols["learned"] = []
    ov = {"nn": [], "random": []}
    ov.update({f"at_{rho:g}": [] for rho in rhos})
    for k in range(H):
        A = A_h[k]
        b = rng.standard_normal(P)
        w_r, V_r, _, _ = _small(A, r)
        dg = np.diag(A).copy()
        cols["cg"].append(pcg_iterations(A, b, None, tol))
        cols["jacobi"].append(pcg_iterations(A, b, lambda v: v / dg, tol))
        cols["forward"].append(pcg_iterations(A, b, _forward_minv(A, r), tol))
        cols["deflation"].append(pcg_iterations(A, b, _deflation_minv(A, w_r, V_r), tol))
        for name, B in (("nn", A_nn[k]), ("random", A_rand[k])):
            wo, Vo, _, _ = _small(B, r)
            cols[f"deflation_{name}"].append(pcg_iterations(A, b, _deflation_minv(A, wo, Vo), tol))
            ov[name].append(float(np.linalg.norm(V_r.T @ Vo) ** 2 / r))
        for rho in rhos:
            wo, Vo, _, _ = _small(pert[rho][k], r)
            cols[f"deflation_at_{rho:g}"].append(pcg_iterations(A, b, _deflation_minv(A, wo, Vo), tol))
            ov[f"at_{rho:g}"].append(float(np.linalg.norm(V_r.T @ Vo) ** 2 / r))
        if learned is not None:
            d, U = learned[0][k], learned[1][k]
            Di = 1.0 / d
            K = np.eye(U.shape[1]) + (U.T * Di) @ U
            Kinv = np.linalg.inv(K)
            cols["learned"].append(pcg_iterations(
                A, b, lambda v, Di=Di, U=U, Kinv=Kinv: Di * v - Di * (U @ (Kinv @ (U.T @ (Di * v)))), tol))
    its = {k: float(np.mean(v)) for k, v in cols.items()}
    return {
        "params": P, "rank": r, "heldout": H, "train": int(np.asarray(theta_train).shape[0]), "tol": tol,
        "iterations": its,
        "reduction_vs_cg": {k: its["cg"] / v for k, v in its.items() if k != "cg"},
        "overlap": {k: float(np.mean(v)) for k, v in ov.items()},
        "overlap_unrelated": r / P,
        "distance": {"nearest_train": float(dist.min(1).mean()), "random_point": float(d_rand.mean())},
    }
