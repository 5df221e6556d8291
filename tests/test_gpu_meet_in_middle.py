"""Meet-in-the-middle transport (first-half derivative states carried forward
to a cut, second-half ones backward to it through the inverse gates) against
the forward transport and the FP64 oracle.

FP64 plans forced to meet in the middle must agree with the oracle to 1e-10
(Q, gradient, energy, step, final state) on ansatz and random circuits of
every gate kind, single- and multi-pass, batched, with TFIM and Pauli
Hamiltonians; mixed plans (which take it by default) to 1e-6 on the metric."""
import numpy as np
import pytest

from oracle import oracle as O
from test_gpu_general_circuits import random_circuit

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    Q.lib()
    return Q


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def reference(orc, n, gates, theta, P, pauli=None):
    psi, D = orc.derivatives(n, O.gates_array(gates), theta, P)
    hp = orc.pauli_apply(n, psi, pauli) if pauli else orc.tfim_apply(n, psi)
    Qm = orc.qgt_from_states(psi, D)
    g = orc.energy_grad(D, hp)
    x, _ = orc.cholesky_solve(Qm.real, g, 1e-3)
    return psi, Qm, g, float(np.real(np.vdot(psi, hp))), x


@pytest.mark.parametrize("n,L,ent", [(8, 3, "cnot"), (13, 2, "cz"), (15, 2, "cnot"), (17, 2, "cz")])
def test_fp64_meet_matches_oracle_ansatz(Q, orc, n, L, ent):
    gates = Q.ansatz_gates(n, L, ent)
    P = 2 * n * L
    th = O.splitmix64_params(40 + n, P)
    psi, Qm, g, E, x = reference(orc, n, gates, th, P)
    with Q.Plan(n, gates, P, precision=Q.FP64, transport=Q.TRANSPORT_MEET) as p:
        info = p.info()
        out = p.run(th)
        st = p.state()
    assert info.meet_in_middle == 1 and 0 < info.cut_gate < len(gates)
    assert rel(out["Q"], Qm) < 1e-10
    assert rel(out["grad"], g) < 1e-10
    assert abs(out["energy"] - E) < 1e-10
    assert rel(out["natgrad"], x) < 1e-9
    assert rel(st, psi) < 1e-12


@pytest.mark.parametrize("n,seed", [(12, 11), (14, 12)])
def test_fp64_meet_random_circuits_pauli(Q, orc, n, seed):
    P = 14
    gates = random_circuit(n, 100, P, seed)
    th = O.splitmix64_params(seed, P)
    rng = np.random.default_rng(seed)
    pauli = [(float(rng.standard_normal()), "".join(rng.choice(list("IXYZ"), n))) for _ in range(7)]
    psi, Qm, g, E, x = reference(orc, n, gates, th, P, pauli)
    with Q.Plan(n, gates, P, precision=Q.FP64, transport=Q.TRANSPORT_MEET, pauli=pauli) as p:
        assert p.info().meet_in_middle == 1
        out = p.run(th)
    assert rel(out["Q"], Qm) < 1e-10
    assert rel(out["grad"], g) < 1e-10
    assert abs(out["energy"] - E) < 1e-10


def test_fp64_meet_batched(Q, orc):
    n, L = 14, 2
    gates = Q.ansatz_gates(n, L, "cz")
    P = 2 * n * L
    th = np.stack([O.splitmix64_params(70 + k, P) for k in range(3)])
    with Q.Plan(n, gates, P, precision=Q.FP64, transport=Q.TRANSPORT_MEET, batch=3) as p:
        out = p.run(th)
    for k in range(3):
        _, Qm, g, E, _ = reference(orc, n, gates, th[k], P)
        assert rel(out["Q"][k], Qm) < 1e-10 and rel(out["grad"][k], g) < 1e-10


@pytest.mark.parametrize("n,L,ent", [(14, 2, "cz"), (16, 3, "cnot")])
def test_mixed_meet_against_fp64(Q, n, L, ent):
    gates = Q.ansatz_gates(n, L, ent)
    P = 2 * n * L
    th = O.splitmix64_params(90 + n, P)
    with Q.Plan(n, gates, P, precision=Q.FP64) as p64:
        ref = p64.run(th)
    with Q.Plan(n, gates, P, precision=Q.MIXED) as pm:
        assert pm.info().meet_in_middle == 1
        out = pm.run(th)
    with Q.Plan(n, gates, P, precision=Q.MIXED, transport=Q.TRANSPORT_FORWARD) as pf:
        assert pf.info().meet_in_middle == 0
        fwd = pf.run(th)
    em, ef = rel(out["Q"].real, ref["Q"].real), rel(fwd["Q"].real, ref["Q"].real)
    print(f"n={n}: metric err meet {em:.2e} forward {ef:.2e}")
    assert em < 1e-6
    assert rel(out["Q"], ref["Q"]) < 2e-6
    assert rel(out["grad"], ref["grad"]) < 2e-6
    assert abs(out["energy"] - ref["energy"]) < 1e-6
