"""CPU check of the pass scheduler: the host-side schedule of a plan (passes,
their gate ops, the vector entries that each pass carries, forward and
meet-in-the-middle transport) is dumped without a GPU and replayed in FP64
numpy with the same semantics as the pass kernels; the Q and the energy
gradient it yields must equal the FP64 oracle's to 1e-11."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

INV = 0x100
QENT_SRC_ZERO = 4


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    L = Q.lib()
    L.qgt_plan_schedule_dump.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p]
    return Q


def gate_matrix(t, a):
    c, s = np.cos(a / 2), np.sin(a / 2)
    r = 1 / np.sqrt(2)
    base = t & 0xFF
    inv = bool(t & INV)
    if base == O.RX:
        return np.array([[c, -1j * s], [-1j * s, c]])
    if base == O.RY:
        return np.array([[c, -s], [s, c]])
    if base == O.RZ:
        return np.diag([np.exp(-0.5j * a), np.exp(0.5j * a)])
    m = {O.X: np.array([[0, 1], [1, 0]]), O.Y: np.array([[0, -1j], [1j, 0]]), O.Z: np.diag([1, -1]),
         O.H: np.array([[r, r], [r, -r]]), O.S: np.diag([1, 1j]), O.T: np.diag([1, np.exp(0.25j * np.pi)])}[base]
    return m.conj().T if inv else m


def apply_1q(v, U, q):
    x = v.reshape(-1, 2, 1 << q)
    return np.einsum("ab,ibj->iaj", U, x).reshape(-1)


def apply_op(v, op, coefs, theta):
    t, q, q2, ci, slot, kind = op
    N = v.shape[0]
    idx = np.arange(N)
    if t == O.CNOT:      # q = target, q2 = control
        sel = ((idx >> q2) & 1) == 1
        w = v.copy()
        w[sel] = v[idx[sel] ^ (1 << q)]
        return w
    if t == O.CZ:
        w = v.copy()
        w[(((idx >> q) & 1) & ((idx >> q2) & 1)) == 1] *= -1
        return w
    if t == O.SWAP:
        j = idx ^ ((((idx >> q) ^ (idx >> q2)) & 1) * ((1 << q) | (1 << q2)))
        return v[j]
    ct, cp, ca = coefs[ci]
    a = theta[cp] if cp >= 0 else ca
    if ct & INV:
        a = -a
    return apply_1q(v, gate_matrix(ct, a), q)


def generator(v, op):
    t, q = op[0], op[1]
    G = {O.RX: np.array([[0, 1], [1, 0]]), O.RY: np.array([[0, -1j], [1j, 0]]), O.RZ: np.diag([1, -1])}[t]
    return apply_1q(v, -0.5j * G, q)


def replay(orc, plan, theta, n):
    N = 1 << n
    rows = {}
    zero = np.zeros(N, complex)
    zero[0] = 1
    coefs = plan["coefs"]
    h_done = False

    def ham():
        src = plan["row_T"] if plan["mitm"] else 0
        rows[1] = orc.tfim_apply(n, rows[src])

    for ps in plan["passes"]:
        if ps["part"] == 2 and not h_done:
            ham()
            h_done = True
        snap = dict(rows)
        out = {}
        for (src, dst, spawn, flags) in ps["entries"]:
            v = zero.copy() if flags & QENT_SRC_ZERO else snap[src].copy()
            for op in ps["ops"]:
                v = apply_op(v, op, coefs, theta)
                if spawn >= 0 and op[4] == dst - 2:
                    v = generator(v, op)
            out[dst] = v
        rows.update(out)
    if not h_done:
        ham()
    R = plan["rows"]
    V = np.stack([rows.get(r, np.zeros(N, complex)) for r in range(R)])
    HG = V.conj() @ V.T
    s = HG[0, 0].real
    sp = plan["slot_param"]
    P = max(sp) + 1
    M = np.zeros((P, R))
    for k, pr in enumerate(sp):
        M[pr, 2 + k] += 1
    B = M @ HG @ M.T
    v = M @ HG[:, 0]
    Qm = B / s - np.outer(v, v.conj()) / s ** 2
    E = HG[0, 1].real / s
    grad = 2 * (M @ HG[:, 1]).real / s - 2 * E * v.real / s
    return Qm, grad, E, rows


def dump(Q, n, gates, P, precision, transport, tmp_path):
    d = Q.circuit_desc(n, gates, P)
    o = Q.PlanOptions()
    Q.lib().qgt_plan_default_options(C.byref(o))
    o.precision, o.transport = precision, transport
    path = str(tmp_path / "sched.json")
    rc = Q.lib().qgt_plan_schedule_dump(C.cast(C.pointer(d), C.c_void_p), C.cast(C.pointer(o), C.c_void_p),
                                        path.encode())
    assert rc == 0, Q.lib().qgt_last_error()
    with open(path) as f:
        return json.load(f)


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


CASES = [(8, 3, "cnot"), (13, 2, "cz"), (15, 2, "cnot")]


@pytest.mark.parametrize("transport", [1, 2])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("n,L,ent", CASES)
def test_schedule_replay_matches_oracle(Q, orc, tmp_path, n, L, ent, precision, transport):
    gates = Q.ansatz_gates(n, L, ent)
    P = 2 * n * L
    th = O.splitmix64_params(500 + n, P)
    plan = dump(Q, n, gates, P, precision, transport, tmp_path)
    assert plan["mitm"] == (1 if transport == 2 else 0)
    Qm, grad, E, rows = replay(orc, plan, th, n)
    psi, D = orc.derivatives(n, O.gates_array(gates), th)
    Qref = orc.qgt_from_states(psi, D)
    gref = orc.energy_grad(D, orc.tfim_apply(n, psi))
    assert rel(Qm, Qref) < 1e-11
    assert rel(grad, gref) < 1e-11
    final = rows[plan["row_T"]] if plan["mitm"] else rows[0]
    assert rel(final, psi) < 1e-12


def test_schedule_replay_random_circuit_meet(Q, orc, tmp_path):
    from test_gpu_general_circuits import random_circuit
    n, P = 10, 12
    gates = random_circuit(n, 80, P, 5)
    th = O.splitmix64_params(5, P)
    plan = dump(Q, n, gates, P, 0, 2, tmp_path)
    assert plan["mitm"] == 1
    Qm, grad, _, _ = replay(orc, plan, th, n)
    psi, D = orc.derivatives(n, O.gates_array(gates), th, P)
    assert rel(Qm, orc.qgt_from_states(psi, D)) < 1e-11
    assert rel(grad, orc.energy_grad(D, orc.tfim_apply(n, psi))) < 1e-11
