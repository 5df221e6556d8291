"""The natural-gradient solve of complex64 plans: FP32 blocked Cholesky with
FP64 iterative refinement against the FP64 residual, and its fallback to the
FP64 solver.

The step must equal an FP64 solve of the plan's own outputs,
(Re Q + lambda I) x = grad, to 1e-10 on well-conditioned systems (the
refinement reaches FP64 accuracy), and to 1e-6 on a system with condition
number ~1e8 (duplicated parameter directions, lambda = 1e-8), where the FP32
factor cannot converge and the plan reruns the FP64 solver from lambda."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    Q.lib()
    return Q


def fp64_step(out, lam):
    A = out["Q"].real
    A = 0.5 * (A + A.T) + lam * np.eye(A.shape[0])
    return np.linalg.solve(A, out["grad"]), np.linalg.cond(A)


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("n,L,ent", [(14, 2, "cz"), (16, 3, "cnot"), (13, 3, "cz"), (14, 19, "cnot"),
                                     (10, 16, "cz"), (10, 15, "cnot")])
def test_refined_step_is_fp64_accurate(Q, n, L, ent):
    """P = 56, 96, 78 (a partial last block of the 32-wide blocked factor), 532 (17 blocks), 320
    (the headline's size) and 300 (10 blocks, the last partial)."""
    gates = Q.ansatz_gates(n, L, ent)
    P = 2 * n * L
    th = O.splitmix64_params(300 + n, P)
    with Q.Plan(n, gates, P, precision=Q.MIXED) as p:
        out = p.run(th)
        st, lam = p.status()
    x, cond = fp64_step(out, 1e-3)
    print(f"n={n}: cond {cond:.2e}, step rel err {rel(out['natgrad'], x):.2e}")
    assert st == 0 and lam == 1e-3
    assert rel(out["natgrad"], x) < 1e-10


def test_ill_conditioned_step_falls_back_to_fp64(Q):
    n = 13
    base = Q.ansatz_gates(n, 2, "cnot")
    # each RZ of the first layer is followed by a second RZ on the same qubit with its own
    # parameter: the two derivative states coincide, so Re Q has a null direction per pair
    gates, P = [], 0
    for g in base:
        if g[3] >= 0:
            gates.append((g[0], g[1], g[2], P, g[4]))
            P += 1
            if g[0] == Q.RZ and g[1] < 4:
                gates.append((Q.RZ, g[1], -1, P, 0.0))
                P += 1
        else:
            gates.append(g)
    th = O.splitmix64_params(77, P)
    lam = 1e-8
    with Q.Plan(n, gates, P, precision=Q.MIXED, lam=lam) as p:
        out = p.run(th)
        st, used = p.status()
    # the FP64 solver starts from lambda (a tiny negative eigenvalue of the mixed Re Q would
    # make it retry with 10 lambda: compare with the lambda it used)
    x, cond = fp64_step(out, used)
    print(f"cond {cond:.2e}, step rel err {rel(out['natgrad'], x):.2e}, status {st}, lambda {used}")
    assert st == 0 and lam <= used <= 1e3 * lam
    assert cond > 1e5
    assert rel(out["natgrad"], x) < 1e-6
