"""CPU check of the register programs that the pass kernels execute.

The plan's schedule (test_schedule_replay.py) is lowered, for passes on full
register tiles, into programs of layout switches, single-qubit blocks,
diagonal runs in a fixed format and CZ / CNOT ops whose qubits are named by
their role in the current layout (lane bit, register bit, warp bit or a qubit
outside the tile).  This test replays those programs on full FP64 state vectors
with the kernels' semantics: every role is resolved through the segment layout
and the pass's local-to-physical map (and must name the qubit the op was built
for), every diagonal run is expanded from its fixed format (register-bit
factors with their CZ signs, thread factors, CZ parities, the static sign mask,
generator markers), and a derivative entry inserts its generator at its spawn
op.  The rows must give the FP64 oracle's QGT and energy gradient to 1e-11,
for complex64 (13-qubit tiles) and complex128 (12-qubit tiles) plans, forward
and meet-in-the-middle transport."""
import ctypes as C
import json

import numpy as np
import pytest

from oracle import oracle as O
from test_schedule_replay import INV, QENT_SRC_ZERO, apply_1q, apply_op, gate_matrix, generator

QENT_STORE_V = 1

RL_REG, RL_WARP, RL_OUT = 8, 16, 32
Q2_SEG, Q2_U, Q2_UR, Q2_PHASE, Q2_CZ, Q2_CNOT, Q2_DIAG, Q2_CZT, Q2_ZGEN, Q2_UM = 1, 2, 3, 4, 5, 6, 7, 9, 10, 11
GEN = {1: np.array([[0, 1], [1, 0]]), 2: np.array([[0, -1j], [1j, 0]]), 3: np.diag([1, -1])}


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    L = Q.lib()
    L.qgt_plan_schedule_dump.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p]
    return Q


def dump(Q, n, gates, P, precision, transport, tmp_path, ckpt=False, **opts):
    d = Q.circuit_desc(n, gates, P)
    o = Q.PlanOptions()
    Q.lib().qgt_plan_default_options(C.byref(o))
    o.precision, o.transport = precision, transport
    for k, v in opts.items():
        setattr(o, k, v)
    path = str(tmp_path / "sched.json")
    fn = Q.lib().qgt_plan_schedule_dump_ckpt if ckpt else Q.lib().qgt_plan_schedule_dump
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p]
    rc = fn(C.cast(C.pointer(d), C.c_void_p), C.cast(C.pointer(o), C.c_void_p), path.encode())
    assert rc == 0, Q.lib().qgt_last_error()
    with open(path) as f:
        return json.load(f)


class Program:
    """Replays one pass program on state vectors of n qubits."""

    def __init__(self, plan, ps, theta, n):
        self.plan, self.ps, self.theta, self.n = plan, ps, theta, n
        self.prog = ps["prog2"]
        self.l2p = ps["l2p"]
        self.RB = plan["reg_bits"]
        self.WB = ps["tile_bits"] - 5 - self.RB
        self.idx = np.arange(1 << n)
        self.coefs = plan["coefs"]

    def matrix(self, c):
        if c < 0:
            return np.eye(2)
        nc = self.plan["ncoef"]
        if c < nc:
            t, p, a = self.coefs[c]
            a = self.theta[p] if p >= 0 else a
            return gate_matrix(t, -a if t & INV else a)   # inverse rotations: the angle negated
        d = np.ones(2, complex)
        for k in self.plan["comb"][c - nc]:
            d *= np.diag(self.matrix(k))
        return np.diag(d)

    def layout(self, seg):
        L = self.plan["segs"][seg]
        regs, warps = L[:self.RB], L[8:8 + self.WB]
        # every local bit of the tile has exactly one role
        assert sorted(list(range(5)) + list(regs) + list(warps)) == list(range(self.ps["tile_bits"]))
        return regs, warps

    def phys(self, role, q, lay):
        regs, warps = lay
        if role < RL_REG:
            return self.l2p[role]
        if role < RL_WARP:
            return self.l2p[regs[role - RL_REG]]
        if role < RL_OUT:
            return self.l2p[warps[role - RL_WARP]]
        return q

    def bit(self, role, q, lay):
        return (self.idx >> self.phys(role, q, lay)) & 1

    def gate(self, v, op, role, lay, check=True):
        kind, _, _, _, _, coef, q, _, _ = op
        p = self.phys(role, q, lay)
        if check:
            assert p == q, (op, role, p)
        return apply_1q(v, self.matrix(coef), p) if coef >= 0 else v

    def gen(self, v, g, p):
        return apply_1q(v, -0.5j * GEN[g], p)

    def diag(self, v, pc, lay, spawn):
        kind, nt, nz, cnt, smask, _, _, _, _ = self.prog[pc]
        regs, _ = lay
        preg = [self.l2p[r] for r in regs]
        rmask = sum(1 << p for p in preg)
        pthr = self.idx & ~rmask
        j = sum(((self.idx >> p) & 1) << i for i, p in enumerate(preg))
        ph = np.ones(self.idx.shape, complex)
        r0 = pc + 1
        t0 = r0 + self.RB
        z0 = t0 + nt
        for i in range(self.RB):
            so = self.prog[r0 + i]
            assert so[0] == Q2_PHASE
            m = self.matrix(so[5])
            sg = 1 - 2 * (np.bitwise_count(pthr & so[4]).astype(np.int64) & 1) if so[4] else 1
            ph *= np.where((j >> i) & 1, sg * m[1, 1], m[0, 0])
        for u in range(t0, z0):
            so = self.prog[u]
            assert so[0] == Q2_PHASE and not (RL_REG <= so[1] < RL_WARP)
            if so[5] < 0:
                continue
            m = self.matrix(so[5])
            ph *= np.where(self.bit(so[1], so[6], lay), m[1, 1], m[0, 0])
        par = np.zeros(self.idx.shape, np.int64)
        for u in range(z0, z0 + nz):
            so = self.prog[u]
            assert so[0] == Q2_CZT
            par ^= ((pthr >> so[6]) & 1) & (np.bitwise_count(pthr & so[4]).astype(np.int64) & 1)
        ph *= 1 - 2 * (par & 1)
        ph *= 1 - 2 * ((smask >> j) & 1)
        v = v * ph
        for u in range(z0 + nz, pc + cnt + 1):
            so = self.prog[u]
            assert so[0] == Q2_ZGEN
            p = self.phys(so[1], so[6], lay)
            assert p == so[6]
            if spawn == u:
                v = self.gen(v, 3, p)
        return v, pc + cnt

    def block(self, v, pc, lay, spawn):
        _, nl, rmask, cnt, _, _, _, _, _ = self.prog[pc]
        spawned = []
        for u in range(pc + 1, pc + 1 + nl):
            op = self.prog[u]
            assert op[1] < RL_REG   # lane ops first
            v = self.gate(v, op, op[1], lay)
            if spawn == u and op[8]:
                spawned.append((op[8], op[6]))
        at = pc + 1 + nl
        for i in range(self.RB):
            if (rmask >> i) & 1:
                op = self.prog[at]
                v = self.gate(v, op, RL_REG + i, lay)   # the block's i-th register op acts on register bit i
                if spawn == at and op[8]:
                    spawned.append((op[8], op[6]))
                at += 1
        assert at == pc + cnt + 1
        for g, q in spawned:   # the ops of a block commute
            v = self.gen(v, g, q)
        return v, pc + cnt

    def run(self, v, start, spawn, ckpt=None):
        """The entry's vector from program op `start` (a layout switch) to the end; with `ckpt` (the
        checkpoint writer) the state before every layout switch that carries a checkpoint row."""
        assert self.prog[start][0] == Q2_SEG
        lay = self.layout(self.prog[start][3])
        pc = start + 1
        while pc < len(self.prog):
            op = self.prog[pc]
            kind = op[0]
            if kind == Q2_SEG:
                if ckpt is not None and op[4] >= 0:
                    ckpt[op[4]] = v.copy()
                lay = self.layout(op[3])
            elif kind == Q2_DIAG:
                v, pc = self.diag(v, pc, lay, spawn)
            elif kind == Q2_UM:
                v, pc = self.block(v, pc, lay, spawn)
            elif kind in (Q2_U, Q2_UR, Q2_PHASE):
                v = self.gate(v, op, op[1], lay)
                if spawn == pc and op[8]:
                    v = self.gen(v, op[8], op[6])
            elif kind == Q2_CZ:
                a, b = self.phys(op[1], op[6], lay), self.phys(op[2], op[7], lay)
                assert (a, b) == (op[6], op[7])
                v = v.copy()
                v[(((self.idx >> a) & 1) & ((self.idx >> b) & 1)) == 1] *= -1
            elif kind == Q2_CNOT:
                t, c = self.phys(op[1], op[6], lay), self.phys(op[2], op[7], lay)
                assert (t, c) == (op[6], op[7])
                sel = ((self.idx >> c) & 1) == 1
                w = v.copy()
                w[sel] = v[self.idx[sel] ^ (1 << t)]
                v = w
            else:
                raise AssertionError(f"op kind {kind} at {pc}")
            pc += 1
        return v


def replay_programs(orc, plan, theta, n):
    """The rows of the plan as the pass kernels would leave them (register programs where a pass has
    one, the gate list otherwise), and the QGT / gradient / energy assembled from them."""
    N = 1 << n
    rows = {}
    zero = np.zeros(N, complex)
    zero[0] = 1
    h_done = False
    nprog = 0
    stats = {"ckpt_starts": 0}

    def ham():
        src = plan["row_T"] if plan["mitm"] else 0
        rows[1] = orc.tfim_apply(n, rows[src])

    for ps in plan["passes"]:
        if ps["part"] == 2 and not h_done:
            ham()
            h_done = True
        snap = dict(rows)
        out = {}
        ck = {}   # checkpoint rows of this pass: written by its first entry, read by later ones
        prog = Program(plan, ps, theta, n) if ps["prog2"] else None
        nprog += prog is not None
        for k, (src, dst, spawn, flags) in enumerate(ps["entries"]):
            if flags & QENT_SRC_ZERO:
                v = zero.copy()
            else:
                v = (ck[src] if src in ck else snap[src]).copy()
            if prog is not None:
                writer = k == 0 and ps.get("ckpt_writer", 0)
                nck = len(ck)
                v = prog.run(v, ps["starts"][k], spawn, ck if writer else None)
                assert writer or len(ck) == nck
                stats["ckpt_starts"] += ps["starts"][k] > 0
            else:
                for op in ps["ops"]:
                    v = apply_op(v, op, plan["coefs"], theta)
                    if spawn >= 0 and op[4] == dst - 2:
                        v = generator(v, op)
            if flags & QENT_STORE_V:
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
    return Qm, grad, nprog, stats


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("transport", [1, 2])
@pytest.mark.parametrize("precision,n,L,ent", [(1, 13, 2, "cz"), (1, 14, 2, "cz"), (1, 15, 1, "cnot"),
                                               (0, 12, 2, "cz"), (0, 13, 1, "cnot")])
def test_register_programs_match_oracle(Q, orc, tmp_path, precision, n, L, ent, transport):
    gates = Q.ansatz_gates(n, L, ent)
    P = 2 * n * L
    th = O.splitmix64_params(700 + n, P)
    plan = dump(Q, n, gates, P, precision, transport, tmp_path)
    Qm, grad, nprog, _ = replay_programs(orc, plan, th, n)
    assert nprog > 0   # the register-tile passes really went through their programs
    psi, D = orc.derivatives(n, O.gates_array(gates), th)
    assert rel(Qm, orc.qgt_from_states(psi, D)) < 1e-11
    assert rel(grad, orc.energy_grad(D, orc.tfim_apply(n, psi))) < 1e-11


def test_register_programs_random_circuit(Q, orc, tmp_path):
    """Every gate kind (H, S, T, X, Y, Z, RX, RY, RZ, CNOT, CZ, SWAP) through the programs."""
    from test_gpu_general_circuits import random_circuit
    n, P = 13, 16
    gates = random_circuit(n, 90, P, 11)
    th = O.splitmix64_params(11, P)
    for transport in (1, 2):
        plan = dump(Q, n, gates, P, 1, transport, tmp_path)
        Qm, grad, nprog, _ = replay_programs(orc, plan, th, n)
        assert nprog > 0
        psi, D = orc.derivatives(n, O.gates_array(gates), th, P)
        assert rel(Qm, orc.qgt_from_states(psi, D)) < 1e-11
        assert rel(grad, orc.energy_grad(D, orc.tfim_apply(n, psi))) < 1e-11


@pytest.mark.parametrize("opts", [{"tile_bits": 14}, {"thread_amps": 16}, {"tile_bits": 14, "thread_amps": 16}])
def test_register_programs_other_tiles(Q, orc, tmp_path, opts):
    """14-qubit tiles (4 warp bits) and 16 amplitudes per thread (4 register bits) at 16 qubits."""
    n, L = 16, 2
    gates = Q.ansatz_gates(n, L, "cz")
    P = 2 * n * L
    th = O.splitmix64_params(716, P)
    plan = dump(Q, n, gates, P, 1, 2, tmp_path, **opts)
    assert plan["passes"] and all(ps["tile_bits"] == opts.get("tile_bits", 13) for ps in plan["passes"] if ps["prog2"])
    assert plan["reg_bits"] == (4 if opts.get("thread_amps") == 16 else 5)
    Qm, grad, nprog, _ = replay_programs(orc, plan, th, n)
    assert nprog > 0
    psi, D = orc.derivatives(n, O.gates_array(gates), th)
    assert rel(Qm, orc.qgt_from_states(psi, D)) < 1e-11
    assert rel(grad, orc.energy_grad(D, orc.tfim_apply(n, psi))) < 1e-11


@pytest.mark.parametrize("precision,n,L,ent,transport", [(1, 16, 4, "cz", 2), (1, 16, 4, "cnot", 1), (0, 13, 3, "cz", 2)])
def test_register_programs_with_checkpoints(Q, orc, tmp_path, precision, n, L, ent, transport):
    """Segment checkpoints: a pass's first entry stores its state before every segment that a
    group of spawns starts in, and those spawns run from their segment on the stored state."""
    gates = Q.ansatz_gates(n, L, ent)
    P = 2 * n * L
    th = O.splitmix64_params(900 + n, P)
    plan = dump(Q, n, gates, P, precision, transport, tmp_path, ckpt=True)
    assert any(ps.get("ckpt_writer") for ps in plan["passes"])
    Qm, grad, nprog, stats = replay_programs(orc, plan, th, n)
    assert nprog > 0 and stats["ckpt_starts"] > 0
    psi, D = orc.derivatives(n, O.gates_array(gates), th)
    assert rel(Qm, orc.qgt_from_states(psi, D)) < 1e-11
    assert rel(grad, orc.energy_grad(D, orc.tfim_apply(n, psi))) < 1e-11
