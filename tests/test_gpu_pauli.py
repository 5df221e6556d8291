"""Pauli-sum Hamiltonians (the reference's compute_pauli_expectation
convention) through a plan: energy, gradient and natural-gradient step
against the FP64 oracle, whose Pauli apply is pinned to the reference's own
expectation code (tests/test_oracle_golden.py).  FP64 1e-10, mixed 2e-6."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    Q.lib()
    return Q


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def random_terms(n, T, seed):
    rng = np.random.default_rng(seed)
    return [(float(rng.standard_normal()), "".join(rng.choice(list("IXYZ"), n))) for _ in range(T)]


@pytest.mark.parametrize("prec,tol", [("FP64", 1e-10), ("MIXED", 2e-6)])
@pytest.mark.parametrize("n,L", [(6, 2), (14, 1)])
def test_pauli_energy_gradient_step(Q, orc, prec, tol, n, L):
    gates = Q.ansatz_gates(n, L, "cnot")
    P = 2 * n * L
    th = O.splitmix64_params(60 + n, P)
    terms = random_terms(n, 9, n)
    psi, D = orc.derivatives(n, O.gates_array(gates), th)
    hp = orc.pauli_apply(n, psi, terms)
    E = float(np.real(np.vdot(psi, hp)))
    g = orc.energy_grad(D, hp)
    Qm = orc.qgt_from_states(psi, D)
    x, _ = orc.cholesky_solve(Qm.real, g, 1e-3)
    with Q.Plan(n, gates, P, precision=getattr(Q, prec), pauli=terms) as p:
        out = p.run(th)
    assert abs(out["energy"] - E) < tol * max(1.0, abs(E)) * 10
    assert rel(out["grad"], g) < tol * 10
    assert rel(out["natgrad"], x) < (1e-8 if prec == "FP64" else 1e-4)


def test_tfim_as_pauli_strings_equals_tfim(Q):
    n, L = 8, 2
    gates = Q.ansatz_gates(n, L, "cz")
    P = 2 * n * L
    th = O.splitmix64_params(3, P)
    terms = list(O.tfim_pauli_strings(n))
    with Q.Plan(n, gates, P, precision=Q.FP64) as a, Q.Plan(n, gates, P, precision=Q.FP64, pauli=terms) as b:
        ra, rb = a.run(th), b.run(th)
    assert abs(ra["energy"] - rb["energy"]) < 1e-12
    assert rel(rb["grad"], ra["grad"]) < 1e-12
