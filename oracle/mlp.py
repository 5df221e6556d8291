"""FP64 numpy restatement of the learned metric preconditioner (the checker of
the GPU training and inference kernels).

TEST INFRASTRUCTURE ONLY: used by tests/ to check the CUDA forward, backward
and PCG results; never by the product library.

The network has no reference counterpart (the reference's nearest piece is
the CPU float MLP of src/quantum_geometric/learning/quantum_pipeline_impl.c:
577-790).  Same definition as the product:
    x  = [cos theta, sin theta]
    h1 = silu(W1 x + b1), h2 = silu(W2 h1 + b2), o = W3 h2 + b3
    d  = softplus(o[:P]) + lambda, U = u_scale * o[P:].reshape(P, r)
    loss = mean_s ||diag(d) + U U^T - T_s||_F^2 / ||T_s||_F^2, T = metric + lambda I
Weights enter the products rounded to BF16 (round to nearest even), as on the GPU.
"""
from __future__ import annotations

import numpy as np


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16 << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def layout(P, W, r):
    O = P + P * r
    sizes = [W * 2 * P, W, W * W, W, O * W, O]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(int)
    return sizes, offs, O


def unpack(w, P, W, r):
    sizes, o, O = layout(P, W, r)
    W1 = w[o[0]:o[1]].reshape(W, 2 * P)
    b1 = w[o[1]:o[2]]
    W2 = w[o[2]:o[3]].reshape(W, W)
    b2 = w[o[3]:o[4]]
    W3 = w[o[4]:o[5]].reshape(O, W)
    b3 = w[o[5]:o[6]]
    return W1, b1, W2, b2, W3, b3


def silu(z):
    return z / (1.0 + np.exp(-z))


def forward(w, theta, P, W, r, lam, u_scale, round_weights=True):
    if round_weights:
        W1, b1, W2, b2, W3, b3 = unpack(np.asarray(w, dtype=np.float32), P, W, r)
        W1b, W2b, W3b = bf16(W1), bf16(W2), bf16(W3)
        b1, b2, b3 = (np.asarray(v, dtype=np.float64) for v in (b1, b2, b3))
    else:  # exact weights (for finite-difference checks of the algebra)
        W1b, b1, W2b, b2, W3b, b3 = unpack(np.asarray(w, dtype=np.float64), P, W, r)
    th = np.asarray(theta, dtype=np.float64).reshape(-1, P)
    x = np.concatenate([np.cos(th), np.sin(th)], axis=1)
    z1 = x @ W1b.T + b1
    h1 = silu(z1)
    z2 = h1 @ W2b.T + b2
    h2 = silu(z2)
    o = h2 @ W3b.T + b3
    d = np.logaddexp(0.0, o[:, :P]) + lam
    U = u_scale * o[:, P:].reshape(-1, P, r)
    return dict(x=x, z1=z1, h1=h1, z2=z2, h2=h2, o=o, d=d, U=U, W1b=W1b, W2b=W2b, W3b=W3b)


def loss_grad(w, theta, metric, P, W, r, lam, u_scale, round_weights=True):
    """Mean loss and its gradient with respect to the FP32 masters (flattened like the product)."""
    f = forward(w, theta, P, W, r, lam, u_scale, round_weights)
    S = f["o"].shape[0]
    T = np.asarray(metric, dtype=np.float64).reshape(S, P, P) + lam * np.eye(P)
    d, U, o = f["d"], f["U"], f["o"]
    M = np.einsum("sik,sjk->sij", U, U) + np.einsum("si,ij->sij", d, np.eye(P))
    E = M - T
    nrm = np.einsum("sij,sij->s", T, T)
    loss = float(np.mean(np.einsum("sij,sij->s", E, E) / nrm))
    dM = 2.0 * E / nrm[:, None, None] / S
    dd = np.einsum("sii->si", dM) / (1.0 + np.exp(-o[:, :P]))
    dU = 2.0 * np.einsum("sij,sjk->sik", dM, U)
    do = np.concatenate([dd, u_scale * dU.reshape(S, P * r)], axis=1)
    gW3 = do.T @ f["h2"]
    gb3 = do.sum(0)
    dh2 = do @ f["W3b"]
    sg2 = 1.0 / (1.0 + np.exp(-f["z2"]))
    dz2 = dh2 * sg2 * (1.0 + f["z2"] * (1.0 - sg2))
    gW2 = dz2.T @ f["h1"]
    gb2 = dz2.sum(0)
    dh1 = dz2 @ f["W2b"]
    sg1 = 1.0 / (1.0 + np.exp(-f["z1"]))
    dz1 = dh1 * sg1 * (1.0 + f["z1"] * (1.0 - sg1))
    gW1 = dz1.T @ f["x"]
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def pcg(A, b, lam, d=None, U=None, tol=1e-10, max_iter=1000):
    """PCG for (A + lam I) x = b with M = diag(d) + U U^T (the product's iteration, FP64)."""
    P = len(b)
    Am = A + lam * np.eye(P)
    dd = np.ones(P) if d is None else np.asarray(d, dtype=np.float64)
    if U is not None and U.size:
        M = np.diag(dd) + U @ U.T
        Minv = np.linalg.inv(M)
    else:
        Minv = np.diag(1.0 / dd)
    x = np.zeros(P)
    rv = b.copy()
    bn = np.linalg.norm(b)
    z = Minv @ rv
    p = z.copy()
    rz = rv @ z
    it, rn = 0, 1.0
    while it < max_iter:
        ap = Am @ p
        pap = p @ ap
        if not pap > 0:
            break
        a = rz / pap
        x += a * p
        rv -= a * ap
        it += 1
        rn = np.linalg.norm(rv) / bn
        if rn <= tol:
            break
        z = Minv @ rv
        rzn = rv @ z
        p = z + (rzn / rz) * p
        rz = rzn
    return x, it, rn
