"""Batched plans and ragged batches through the C ABI against the FP64 oracle.

- theta-batched plans (batch = B parameter points in one launch per kernel)
  equal B separate plans; FP64 1e-10 relative, mixed 1e-6 on the metric;
- derivative-parameter subsets give the leading block of the full QGT;
- ragged batches (mixed qubit counts and depths in one graph launch) match
  the oracle per circuit, and their Berry maps match the oracle's direct
  re-simulation of every lattice point (FP64 1e-10 absolute, mixed 1e-6)."""
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


@pytest.mark.parametrize("prec,tol", [("FP64", 1e-10), ("MIXED", 1e-6)])
@pytest.mark.parametrize("n,L,ent", [(10, 2, "cnot"), (14, 1, "cz")])
def test_theta_batch_equals_single_plans(Q, orc, prec, tol, n, L, ent):
    gates = Q.ansatz_gates(n, L, ent)
    P = 2 * n * L
    B = 5
    th = np.stack([O.splitmix64_params(300 + k, P) for k in range(B)])
    with Q.Plan(n, gates, P, precision=getattr(Q, prec), batch=B) as pb:
        out = pb.run(th)
        assert pb.info().batch == B
    for k in range(B):
        psi, D = orc.derivatives(n, O.gates_array(gates), th[k])
        Qref = orc.qgt_from_states(psi, D)
        gref = orc.energy_grad(D, orc.tfim_apply(n, psi))
        assert rel(out["Q"][k].real, Qref.real) < tol
        assert rel(out["grad"][k], gref) < 2 * tol
        x, _ = orc.cholesky_solve(Qref.real, gref, 1e-3)
        assert rel(out["natgrad"][k], x) < (1e-9 if prec == "FP64" else 1e-4)


@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
def test_deriv_param_subset_is_leading_block(Q, orc, prec):
    n, L = 9, 2
    gates = Q.ansatz_gates(n, L, "cnot")
    P = 2 * n * L
    th = O.splitmix64_params(41, P)
    psi, D = orc.derivatives(n, O.gates_array(gates), th)
    Qref = orc.qgt_from_states(psi, D)
    for Pd in (2, 5):
        with Q.Plan(n, gates, P, precision=getattr(Q, prec), deriv_params=Pd, hamiltonian=Q.HAM_NONE) as p:
            out = p.run(th, want=("Q",))
        tol = 1e-12 if prec == "FP64" else 1e-6
        assert np.abs(out["Q"] - Qref[:Pd, :Pd]).max() < tol


def ragged(seed, count, nmin, nmax, lmax):
    rng = np.random.default_rng(seed)
    circs, thetas, pairs = [], [], []
    for c in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        L = int(rng.integers(1, lmax + 1))
        circs.append((n, L))
        thetas.append(O.splitmix64_params(1000 + c, 2 * n * L))
        # first layer RY(q0), RZ(q0); every third circuit: last layer RY(q0), RZ(q1)
        pairs.append((0, n) if c % 3 else (2 * n * (L - 1), 2 * n * (L - 1) + n + 1))
    return circs, thetas, pairs


@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
def test_ragged_batch_qgt_and_berry_maps(Q, orc, prec):
    G = 8
    circs, thetas, pairs = ragged(7, 14, 4, 9, 3)
    spec = [(n, Q.ansatz_gates(n, L, "cnot"), 2 * n * L) for (n, L) in circs]
    with Q.Batch(spec, pairs, precision=getattr(Q, prec), grid=G) as b:
        info = b.info()
        Qs, maps = b.run(thetas)
    assert info.num_circuits == len(circs) and info.num_groups < len(circs)
    tq = 1e-10 if prec == "FP64" else 1e-6
    tm = 1e-10 if prec == "FP64" else 1e-6
    for c, ((n, L), th) in enumerate(zip(circs, thetas)):
        g = O.gates_array(Q.ansatz_gates(n, L, "cnot"))
        psi, D = orc.derivatives(n, g, th)
        Qref = orc.qgt_from_states(psi, D)
        assert rel(Qs[c].real, Qref.real) < tq, (c, n, L)
        ref = orc.berry_map(n, g, th, pairs[c][0], pairs[c][1], G)
        assert np.abs(maps[c] - ref.reshape(G, G)).max() < tm, (c, n, L, pairs[c])


def test_device_resident_batch_launch(Q):
    """qgt_batch_execute_device repeats the batch on the thetas of the last execute_host without the
    copies; the next execute_host returns the same results (same inputs, deterministic kernels)."""
    import torch
    circs, thetas, pairs = ragged(7, 14, 4, 9, 3)
    spec = [(n, Q.ansatz_gates(n, L, "cnot"), 2 * n * L) for (n, L) in circs]
    with Q.Batch(spec, pairs, precision=Q.MIXED, grid=8) as b:
        Q1, m1 = b.run(thetas)
        assert b.stream() != 0
        for _ in range(3):
            b.run_device()
        torch.cuda.synchronize()
        Q2, m2 = b.run(thetas, out=b.output_buffers())
    for a, c in zip(Q1, Q2):
        assert np.array_equal(a, c)
    assert np.array_equal(m1, m2)


def test_berry_map_shared_parameter_full_lattice(Q, orc):
    """A parameter driving two gates: every lattice point is evaluated."""
    n = 5
    gates = Q.ansatz_gates(n, 2, "cnot")
    P = 2 * n * 2
    # parameter 0 also drives the second layer's RY(q2)
    gates = [(t, q0, q1, 0 if (t == Q.RY and q0 == 2 and p == 2 * n + 2) else p, a) for (t, q0, q1, p, a) in gates]
    th = O.splitmix64_params(77, P)
    G = 6
    with Q.Batch([(n, gates, P)], [(0, n + 1)], precision=Q.FP64, grid=G) as b:
        _, maps = b.run([th])
    ref = orc.berry_map(n, O.gates_array(gates), th, 0, n + 1, G)
    assert np.abs(maps[0] - ref.reshape(G, G)).max() < 1e-10


@pytest.mark.parametrize("prec,tol", [("FP64", 1e-10), ("MIXED", 1e-6)])
def test_berry_plan_shared_by_deeper_circuits(Q, orc, prec, tol):
    """The same ansatz at 1, 2 and 3 layers with the Berry pair in the first
    layer: the truncated circuits coincide, so the three structural groups
    share one Berry plan (each circuit keeps its own theta); a pair in the
    last layer of the 3-layer circuit needs a plan of its own."""
    n, G = 7, 6
    circs = [(n, 1), (n, 2), (n, 3), (n, 3)]
    spec = [(n, Q.ansatz_gates(n, L, "cnot"), 2 * n * L) for (n, L) in circs]
    pairs = [(0, n), (0, n), (0, n), (4 * n + 1, 5 * n + 2)]
    thetas = [O.splitmix64_params(900 + c, s[2]) for c, s in enumerate(spec)]
    with Q.Batch(spec, pairs, precision=getattr(Q, prec), grid=G) as b:
        info = b.info()
        _, maps = b.run(thetas)
    assert info.num_groups == 3 and info.num_berry_plans == 2
    for c, ((n_, L), th) in enumerate(zip(circs, thetas)):
        ref = orc.berry_map(n_, O.gates_array(spec[c][1]), th, pairs[c][0], pairs[c][1], G)
        assert np.abs(maps[c] - ref.reshape(G, G)).max() < tol, (c, L, pairs[c])
