"""The preconditioner-limits measurement (quantum_geometric_tensor_gb300.precond_limits) on CPU
with FP64 oracle metrics of a 6-qubit circuit: PCG reaches the tolerance, the deflation form
built from the point's own eigenvectors beats plain CG, distances wrap angles."""
import numpy as np

from oracle import oracle as O
from quantum_geometric_tensor_gb300 import precond_limits as PL


def test_pcg_iterations_solve():
    rng = np.random.default_rng(0)
    X = rng.standard_normal((30, 30))
    A = X @ X.T + 1e-2 * np.eye(30)
    b = rng.standard_normal(30)
    it = PL.pcg_iterations(A, b, None, 1e-10, 1000)
    assert it < 1000
    d = np.diag(A).copy()
    assert PL.pcg_iterations(A, b, lambda v: v / d, 1e-10, 1000) < 1000
    # exact inverse as preconditioner: one iteration
    Ai = np.linalg.inv(A)
    assert PL.pcg_iterations(A, b, lambda v: Ai @ v, 1e-8, 10) == 1


def test_wrapped_distance():
    a = np.array([[0.0, 0.1]])
    b = np.array([[2 * np.pi - 0.1, 0.1], [np.pi, 0.1]])
    d = PL.wrapped_distance(a, b)
    assert np.allclose(d, [[0.1, np.pi]])


def test_analyse_on_oracle_metrics():
    orc = O.Oracle()
    n, L = 6, 3
    g = O.ansatz(n, L, "cnot")
    P = O.num_params(g)

    def mf(th):
        out = np.zeros((th.shape[0], P, P))
        for s in range(th.shape[0]):
            psi, D = orc.derivatives(n, g, th[s])
            out[s] = orc.qgt_from_states(psi, D).real
        return out

    rng = np.random.default_rng(3)
    res = PL.analyse(mf, rng.uniform(0, 2 * np.pi, (400, P)), rng.uniform(0, 2 * np.pi, (4, P)), r=4, rhos=(0.05,))
    it = res["iterations"]
    assert it["deflation"] < it["cg"]
    assert res["overlap"]["at_0.05"] > 0.9
    assert 0 < res["overlap_unrelated"] < 1
