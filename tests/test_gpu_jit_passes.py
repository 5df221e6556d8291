"""Pass programs compiled to straight-line kernels (qgt_jit.c / qgt_jit_rt.cu)
against the program interpreter (qgt_pass2.cu) and the FP64 plan.

QGT_PASS_JIT=1 compiles the passes of every complex64 plan on 13- or 14-qubit
register tiles, QGT_PASS_JIT=0 keeps them on the interpreter.  The compiled
kernels apply real gates as m0 x + m2 y (the interpreter uses the one-multiply
tangent forms), so the two agree to FP32 rounding, not bit for bit:
tolerance 1e-6 relative on Q and gradient, 1e-6 absolute on the energy, 5e-5 on
the natural-gradient step (the solve amplifies differences by the condition
number of Re Q + 1e-3 I); against FP64 the mixed-precision tolerances (metric
1e-6, Q and gradient 2e-6)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    Q.lib()
    return Q


def run(Q, monkeypatch, jit, n, gates, P, theta, batch=1, **kw):
    monkeypatch.setenv("QGT_PASS_JIT", "1" if jit else "0")
    with Q.Plan(n, gates, P, precision=Q.MIXED, batch=batch, **kw) as p:
        info = p.info()
        out = p.run(theta)
        st, _ = p.status()
    assert st == 0
    return info, out


@pytest.mark.parametrize("n,L,ent", [(13, 3, "cz"), (14, 2, "cnot"), (16, 3, "cz"), (19, 8, "cz")])
def test_compiled_passes_match_interpreter(Q, monkeypatch, n, L, ent):
    gates = Q.ansatz_gates(n, L, ent)
    P = 2 * n * L
    theta = O.splitmix64_params(400 + n, P)
    i0, ref = run(Q, monkeypatch, False, n, gates, P, theta)
    i1, out = run(Q, monkeypatch, True, n, gates, P, theta)
    assert i0.jit_passes == 0 and i1.jit_passes > 0
    for k in ("Q", "grad"):
        assert rel(out[k], ref[k]) < 1e-6, k
    assert rel(out["natgrad"], ref["natgrad"]) < 5e-5
    assert abs(out["energy"] - ref["energy"]) < 1e-6
    monkeypatch.setenv("QGT_PASS_JIT", "0")
    with Q.Plan(n, gates, P, precision=Q.FP64) as p64:
        r64 = p64.run(theta)
    assert rel(out["Q"].real, r64["Q"].real) < 1e-6
    assert rel(out["Q"], r64["Q"]) < 2e-6 and rel(out["grad"], r64["grad"]) < 2e-6


def test_compiled_passes_batched_and_forward_transport(Q, monkeypatch):
    n, L = 15, 3
    gates = Q.ansatz_gates(n, L, "cnot")
    P = 2 * n * L
    th = np.stack([O.splitmix64_params(500 + k, P) for k in range(3)])
    _, ref = run(Q, monkeypatch, False, n, gates, P, th, batch=3)
    i1, out = run(Q, monkeypatch, True, n, gates, P, th, batch=3)
    assert i1.jit_passes > 0
    assert rel(out["Q"], ref["Q"]) < 1e-6 and rel(out["grad"], ref["grad"]) < 1e-6
    # forward transport (every derivative carried to the end), deriv subset
    _, ref = run(Q, monkeypatch, False, n, gates, P, th[0], transport=Q.TRANSPORT_FORWARD, deriv_params=30)
    _, out = run(Q, monkeypatch, True, n, gates, P, th[0], transport=Q.TRANSPORT_FORWARD, deriv_params=30)
    assert rel(out["Q"], ref["Q"]) < 1e-6 and rel(out["grad"], ref["grad"]) < 1e-6


def test_general_gates_compiled(Q, monkeypatch):
    """Every gate kind (H, X, Y, Z, S, T, RX, RZ, CNOT, CZ, SWAP, shared parameters) through the compiled
    kernels: the same circuits as the interpreter, against the FP64 plan."""
    rng = np.random.default_rng(11)
    n = 14
    kinds = [Q.H, Q.X, Q.Y, Q.Z, Q.S, Q.T, Q.RX, Q.RY, Q.RZ, Q.CNOT, Q.CZ, Q.SWAP]
    gates, p = [], 0
    for _ in range(160):
        t = int(rng.choice(kinds))
        q0 = int(rng.integers(n))
        q1 = int((q0 + 1 + rng.integers(n - 1)) % n)
        if t in (Q.RX, Q.RY, Q.RZ):
            par = p if rng.random() < 0.8 or p == 0 else int(rng.integers(p))
            p = max(p, par + 1)
            gates.append((t, q0, -1, par, 0.0))
        elif t in (Q.CNOT, Q.CZ, Q.SWAP):
            gates.append((t, q0, q1, -1, 0.0))
        else:
            gates.append((t, q0, -1, -1, 0.0))
    theta = O.splitmix64_params(77, p)
    _, ref = run(Q, monkeypatch, False, n, gates, p, theta)
    i1, out = run(Q, monkeypatch, True, n, gates, p, theta)
    assert i1.jit_passes > 0
    assert rel(out["Q"], ref["Q"]) < 1e-6 and rel(out["grad"], ref["grad"]) < 1e-6
