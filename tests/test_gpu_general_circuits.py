"""Random circuits over every gate kind of the boundary (RX, RY, RZ with shared
and fixed angles, H, X, Y, Z, S, T, CNOT, CZ, SWAP) at sizes that use the
register-resident full-tile passes (>= 12 qubits FP64, >= 13 complex64), against
the FP64 oracle.  Tolerances: FP64 1e-10 relative; mixed 2e-6 relative on Q."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def random_circuit(n, ngates, nparams, seed):
    rng = np.random.default_rng(seed)
    kinds = [O.RX, O.RY, O.RZ, O.H, O.X, O.Y, O.Z, O.S, O.T, O.CNOT, O.CZ, O.SWAP]
    g = []
    # make every parameter used at least once, some shared
    for k in range(nparams):
        g.append((int(rng.choice([O.RX, O.RY, O.RZ])), int(rng.integers(n)), -1, k, 0.0))
    for _ in range(ngates):
        t = int(rng.choice(kinds))
        if t in (O.CNOT, O.CZ, O.SWAP):
            a, b = rng.choice(n, 2, replace=False)
            g.append((t, int(a), int(b), -1, 0.0))
        elif t in (O.RX, O.RY, O.RZ):
            if rng.random() < 0.5:
                g.append((t, int(rng.integers(n)), -1, int(rng.integers(nparams)), 0.0))
            else:
                g.append((t, int(rng.integers(n)), -1, -1, float(rng.uniform(0, 6.28))))
        else:
            g.append((t, int(rng.integers(n)), -1, -1, 0.0))
    order = rng.permutation(len(g))
    return [g[i] for i in order]


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("n,seed", [(12, 1), (13, 2), (14, 3)])
def test_random_circuit_fp64_and_mixed(orc, n, seed):
    import quantum_geometric_tensor_gb300 as Q
    P = 12
    gates = random_circuit(n, 90, P, seed)
    theta = O.splitmix64_params(seed, P)
    psi, D = orc.derivatives(n, O.gates_array(gates), theta, P)
    Qref = orc.qgt_from_states(psi, D)
    gref = orc.energy_grad(D, orc.tfim_apply(n, psi))
    with Q.Plan(n, gates, P, precision=Q.FP64) as p:
        out = p.run(theta)
        assert rel(p.state(), psi) < 1e-12
    assert rel(out["Q"], Qref) < 1e-10
    assert rel(out["grad"], gref) < 1e-10
    with Q.Plan(n, gates, P, precision=Q.MIXED) as p:
        out = p.run(theta)
        st, _ = p.status()
    assert st == 0
    print(f"n={n}: mixed Q rel err {rel(out['Q'], Qref):.2e}")
    assert rel(out["Q"], Qref) < 2e-6
