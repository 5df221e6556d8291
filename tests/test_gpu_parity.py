"""GPU parity: the CUDA path through the C ABI against the FP64 oracle and the
golden fixtures made by the reference's own code.

Tolerances: FP64 path 1e-10 relative (Frobenius) on Q, gradient and natural
gradient; mixed path (complex64 evolution + split-FP16 tensor-core Gram)
1e-6 relative on the metric Re Q and 2e-6 on Q, gradient and step."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    Q.lib()
    return Q


def gates_of(z):
    return [tuple(g) for g in z["gates"].tolist()]


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_fp64_matches_golden(Q, orc, path):
    z = np.load(path)
    n, theta = int(z["n"]), z["theta"]
    gates = gates_of(z)
    with Q.Plan(n, gates, len(theta), precision=Q.FP64) as plan:
        out = plan.run(theta)
        st, lam = plan.status()
        psi = plan.state()
    assert st == 0 and lam == pytest.approx(float(z["lam"]))
    assert rel(psi, z["psi"]) < 1e-12
    assert rel(out["Q"], z["Q"]) < 1e-10
    assert abs(out["energy"] - float(z["energy"])) < 1e-10
    assert rel(out["grad"], z["grad"]) < 1e-10
    x, _ = orc.cholesky_solve(z["Q"].real, z["grad"], float(z["lam"]))
    assert rel(out["natgrad"], x) < 1e-10


@pytest.mark.parametrize("n,L,ent", [(12, 2, "cnot"), (14, 2, "cz"), (15, 1, "cnot"), (13, 3, "cz")])
def test_fp64_multipass_matches_oracle(Q, orc, n, L, ent):
    gates = Q.ansatz_gates(n, L, ent)
    P = 2 * n * L
    theta = O.splitmix64_params(100 + n, P)
    psi, D = orc.derivatives(n, O.gates_array(gates), theta)
    Qref = orc.qgt_from_states(psi, D)
    gref = orc.energy_grad(D, orc.tfim_apply(n, psi))
    with Q.Plan(n, gates, P, precision=Q.FP64) as plan:
        info = plan.info()
        out = plan.run(theta)
    if n > 12:
        assert info.num_passes >= 2
    assert rel(out["Q"], Qref) < 1e-10
    assert rel(out["grad"], gref) < 1e-10


@pytest.mark.parametrize("prec", ["MIXED", "MIXED_BF16X3"])
@pytest.mark.parametrize("n,L,ent", [(10, 4, "cnot"), (8, 3, "cz"), (14, 2, "cz")])
def test_mixed_against_fp64(Q, orc, prec, n, L, ent):
    gates = Q.ansatz_gates(n, L, ent)
    P = 2 * n * L
    theta = O.splitmix64_params(7 + n, P)
    with Q.Plan(n, gates, P, precision=Q.FP64) as p64:
        ref = p64.run(theta)
    with Q.Plan(n, gates, P, precision=getattr(Q, prec)) as pm:
        out = pm.run(theta)
        st, _ = pm.status()
    assert st == 0
    eg = rel(out["Q"].real, ref["Q"].real)
    eq = rel(out["Q"], ref["Q"])
    print(f"{prec} n={n} L={L}: metric {eg:.2e} Q {eq:.2e} grad {rel(out['grad'], ref['grad']):.2e} "
          f"step {rel(out['natgrad'], ref['natgrad']):.2e}")
    if prec == "MIXED":
        assert eg < 1e-6
        assert eq < 2e-6
        assert rel(out["grad"], ref["grad"]) < 2e-6
        assert abs(out["energy"] - ref["energy"]) < 1e-6
    else:
        assert eg < 1e-4


def test_cholesky_retry_and_solve(Q):
    rng = np.random.default_rng(3)
    A = rng.standard_normal((40, 40))
    A = A @ A.T
    b = rng.standard_normal(40)
    x, used = Q.cholesky_solve(A, b, 1e-3)
    assert used == 1e-3
    assert rel((A + 1e-3 * np.eye(40)) @ x, b) < 1e-10
    # indefinite matrix: lambda grows x10 until positive (-0.05 + 0.1 > 0)
    B = np.diag(np.r_[np.ones(39), -0.05])
    x, used = Q.cholesky_solve(B, np.ones(40), 1e-3)
    assert used == pytest.approx(0.1)
    assert rel((B + used * np.eye(40)) @ x, np.ones(40)) < 1e-12


def test_reused_output_buffers(Q):
    """run(theta, out=...) writes the same outputs into caller-owned arrays (one
    synchronisation per call; bad buffers are refused before any copy)."""
    n, L = 12, 2
    P = 2 * n * L
    g = Q.ansatz_gates(n, L, "cz")
    with Q.Plan(n, g, P, precision=Q.MIXED) as p:
        ref = p.run(O.splitmix64_params(61, P))
        bufs = p.output_buffers()
        for seed in (62, 61):
            out = p.run(O.splitmix64_params(seed, P), out=bufs)
        assert out["Q"] is not None and np.array_equal(out["Q"], ref["Q"])
        assert np.array_equal(out["natgrad"], ref["natgrad"]) and out["energy"] == ref["energy"]
        with pytest.raises(ValueError):
            p.run(ref["grad"], out={"Q": np.zeros((1, P, P))})


def test_wide_tiles_against_fp64(Q):
    """19 qubits, 8 layers on 14-qubit register tiles (512-thread CTAs; 6 passes instead of 9),
    with 32 tiles per vector and segment checkpoints, interpreted and compiled; single and
    batched complex64 plans against the FP64 plan (12-qubit tiles)."""
    n, L = 19, 8
    gates = Q.ansatz_gates(n, L, "cz")
    P = 2 * n * L
    th = np.stack([O.splitmix64_params(90, P), O.splitmix64_params(91, P)])
    with Q.Plan(n, gates, P, precision=Q.FP64) as p64:
        ref = p64.run(th[0])
    with Q.Plan(n, gates, P, precision=Q.MIXED, tile_bits=14) as pm:
        assert pm.info().tile_bits == 14
        out = pm.run(th[0])
    with Q.Plan(n, gates, P, precision=Q.MIXED, tile_bits=14, pass_kernels=Q.PASS_INTERPRET) as pi:
        assert pi.info().tile_bits == 14 and pi.info().jit_passes == 0
        outi = pi.run(th[0])
    with Q.Plan(n, gates, P, precision=Q.MIXED, batch=2, tile_bits=14) as pb:
        outb = pb.run(th)
    for o in (out, outi, {k: (v[0] if v is not None else None) for k, v in outb.items()}):
        assert rel(o["Q"].real, ref["Q"].real) < 1e-6
        assert rel(o["Q"], ref["Q"]) < 2e-6
        assert rel(o["grad"], ref["grad"]) < 2e-6
        assert abs(o["energy"] - ref["energy"]) < 1e-6
