"""The benchmark configurations at their real sizes, through the C ABI.

* 20 qubits, 8 layers RY/RZ + CZ ring, P = 320 (the headline step): the mixed
  plan against the FP64 plan on the same point (metric 1e-6 relative, Q and
  gradient 2e-6, energy 1e-6 absolute, natural-gradient step 5e-5: the solve
  amplifies by the condition number of Re Q + 1e-3 I); and the FP64 plan with
  the first 16 parameters as derivative parameters against the FP64 oracle on
  the same 16 derivative states (1e-10 relative).
* Ragged batch from the real distribution (qubits U{12..18}, layers U{2..6},
  RY/RZ + CNOT ladder), 64 circuits with 32 x 32 Berry maps over (first RY,
  first RZ of qubit 0): QGTs of 4 circuits against the oracle (metric 1e-6,
  Q 2e-6) and 12 lattice points of each of their maps against the oracle's
  2 x 2 QGT at those points (1e-6 absolute).
* 26 qubits, 2 layers RY/RZ + CNOT ladder, P = 104: the FP64 plan with 4
  derivative parameters against the oracle (1e-10), the mixed plan with the same
  4 against the FP64 one, and the full mixed step (integer-digit tcgen05 Gram
  over 2^26 amplitudes) against the full FP64 step (metric 1e-6)."""
import math

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


def fixed_beyond(gates, theta, keep):
    """The gate list with parameters >= keep turned into fixed angles (the oracle's derivative rows are
    then the first `keep` parameters only)."""
    g = O.gates_array(gates).copy()
    for i in range(len(g)):
        if g[i]["param"] >= keep:
            g[i]["angle"] = theta[g[i]["param"]]
            g[i]["param"] = -1
    return g


def test_headline_mixed_against_fp64(Q):
    n, L = 20, 8
    gates = Q.ansatz_gates(n, L, "cz")
    P = 2 * n * L
    theta = O.splitmix64_params(2026, P)
    with Q.Plan(n, gates, P, precision=Q.FP64) as p64:
        ref = p64.run(theta)
        assert p64.status()[0] == 0
    with Q.Plan(n, gates, P, precision=Q.MIXED) as pm:
        info = pm.info()
        out = pm.run(theta)
        assert pm.status()[0] == 0
    assert info.tile_bits in (13, 14) and info.meet_in_middle == 1 and info.jit_passes > 0
    e = {"metric": rel(out["Q"].real, ref["Q"].real), "berry": rel(out["Q"].imag, ref["Q"].imag),
         "Q": rel(out["Q"], ref["Q"]), "grad": rel(out["grad"], ref["grad"]),
         "step": rel(out["natgrad"], ref["natgrad"]), "energy": abs(out["energy"] - ref["energy"])}
    print("20q/P=320 mixed vs FP64:", {k: f"{v:.2e}" for k, v in e.items()})
    assert e["metric"] < 1e-6 and e["Q"] < 2e-6 and e["grad"] < 2e-6
    assert e["energy"] < 1e-6 and e["step"] < 5e-5


def test_headline_fp64_subset_against_oracle(Q, orc):
    n, L, Pd = 20, 8, 16
    gates = Q.ansatz_gates(n, L, "cz")
    P = 2 * n * L
    theta = O.splitmix64_params(2026, P)
    with Q.Plan(n, gates, P, precision=Q.FP64, deriv_params=Pd) as p:
        out = p.run(theta)
        psi_gpu = p.state()
    g = fixed_beyond(gates, theta, Pd)
    psi, D = orc.derivatives(n, g, theta[:Pd], Pd)
    Qref = orc.qgt_from_states(psi, D)
    gref = orc.energy_grad(D, orc.tfim_apply(n, psi))
    assert rel(psi_gpu, psi) < 1e-12
    assert rel(out["Q"], Qref) < 1e-10
    assert rel(out["grad"], gref) < 1e-10


def berry_point(orc, n, gates, theta, a, b, ta, tb):
    """Im Q_ab of the oracle at theta_a = ta, theta_b = tb (the other parameters at theta)."""
    g = O.gates_array(gates).copy()
    for i in range(len(g)):
        p = g[i]["param"]
        if p == a:
            g[i]["param"] = 0
        elif p == b:
            g[i]["param"] = 1
        elif p >= 0:
            g[i]["angle"] = theta[p]
            g[i]["param"] = -1
    psi, D = orc.derivatives(n, g, np.array([ta, tb]), 2)
    return orc.qgt_from_states(psi, D)[0, 1].imag


def test_ragged_batch_real_distribution(Q, orc):
    G, count = 32, 64
    rng = np.random.default_rng(2026)
    ns, Ls = rng.integers(12, 19, count), rng.integers(2, 7, count)
    spec = [(int(n), Q.ansatz_gates(int(n), int(L), "cnot"), 2 * int(n) * int(L)) for n, L in zip(ns, Ls)]
    thetas = [O.splitmix64_params(5000 + c, s[2]) for c, s in enumerate(spec)]
    pairs = [(0, s[0]) for s in spec]   # first RY and first RZ of qubit 0
    with Q.Batch(spec, pairs, precision=Q.MIXED, grid=G) as b:
        info = b.info()
        Qs, maps = b.run(thetas)
    assert info.num_circuits == count
    assert np.all(np.isfinite(maps))
    # four circuits: the largest, the smallest and two from the middle of the batch
    order = np.argsort([s[0] * 10 + s[2] / 1000 for s in spec])
    pick = [int(order[-1]), int(order[0]), 21, 42]
    pts = [(int(i), int(j)) for i, j in np.random.default_rng(7).integers(0, G, (12, 2))]
    for c in pick:
        n, g, P = spec[c]
        psi, D = orc.derivatives(n, O.gates_array(g), thetas[c])
        Qref = orc.qgt_from_states(psi, D)
        assert rel(Qs[c].real, Qref.real) < 1e-6, (c, n, P)
        assert rel(Qs[c], Qref) < 2e-6, (c, n, P)
        a, bb = pairs[c]
        for i, j in pts:
            ref = berry_point(orc, n, g, thetas[c], a, bb, 2 * math.pi * i / G, 2 * math.pi * j / G)
            assert abs(maps[c][i, j] - ref) < 1e-6, (c, n, i, j)


def test_26_qubits(Q, orc):
    n, L, Pd = 26, 2, 4
    gates = Q.ansatz_gates(n, L, "cnot")
    P = 2 * n * L
    theta = O.splitmix64_params(26, P)
    with Q.Plan(n, gates, P, precision=Q.FP64, deriv_params=Pd) as p:
        sub64 = p.run(theta)
    g = fixed_beyond(gates, theta, Pd)
    psi, D = orc.derivatives(n, g, theta[:Pd], Pd)
    Qref = orc.qgt_from_states(psi, D)
    gref = orc.energy_grad(D, orc.tfim_apply(n, psi))
    del psi, D
    assert rel(sub64["Q"], Qref) < 1e-10
    assert rel(sub64["grad"], gref) < 1e-10
    with Q.Plan(n, gates, P, precision=Q.MIXED, deriv_params=Pd) as p:
        subm = p.run(theta)
    assert rel(subm["Q"].real, sub64["Q"].real) < 1e-6
    # the full step: every derivative state, digit Gram over 2^26 amplitudes
    with Q.Plan(n, gates, P, precision=Q.FP64) as p64:
        ref = p64.run(theta)
    with Q.Plan(n, gates, P, precision=Q.MIXED) as pm:
        out = pm.run(theta)
        assert pm.status()[0] == 0
    em, eb = rel(out["Q"].real, ref["Q"].real), rel(out["Q"].imag, ref["Q"].imag)
    print(f"26q/P=104 mixed vs FP64: metric {em:.2e} berry {eb:.2e}")
    assert em < 1e-6 and rel(out["Q"], ref["Q"]) < 2e-6
    assert rel(out["grad"], ref["grad"]) < 2e-6
    assert np.abs(out["Q"][:Pd, :Pd] - sub64["Q"]).max() < 1e-6
