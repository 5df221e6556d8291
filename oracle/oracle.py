"""ctypes view of the FP64 CPU oracle and of the compiled reference code.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by
the CPU legs of ``bench.py`` as the checker.  The product library never imports it.

``Oracle``      wraps ``oracle/build/libqgt_oracle.so`` (``qgt_oracle.c``), the
                C11 + OpenMP restatement of the reference algorithms.
``Reference``   wraps ``oracle/_ref/libqgt_ref.so``: the reference library's own
                functions (state-vector simulator, Pauli expectation, diffgeo
                QGT contraction, CG natural gradient, float Cholesky inverse),
                compiled from the reference tree by ``oracle/Makefile``.  It only
                exists where that tree was present at build time.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "build", "libqgt_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libqgt_ref.so")

# gate codes = reference gate_type_t values (include/quantum_geometric/core/quantum_base_types.h:32-71)
I, X, Y, Z, H, S, T, RX, RY, RZ, CNOT, CZ, SWAP = 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 13
ROTATIONS = (RX, RY, RZ)

GATE_DTYPE = np.dtype([("type", "<i4"), ("q0", "<i4"), ("q1", "<i4"), ("param", "<i4"), ("angle", "<f8")])


def build(quiet: bool = True, ref_tree: str | None = None) -> None:
    """Compile the oracle, and oracle/_ref from the reference tree at ref_tree
    (or at $QGT_REFERENCE_TREE) when one is given and present."""
    tree = ref_tree or os.environ.get("QGT_REFERENCE_TREE")
    cmd = ["make", "-C", HERE, "-j4"]
    if tree and os.path.isdir(os.path.join(tree, "src", "quantum_geometric")):
        cmd.append(f"REF={tree}")
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def gates_array(gates) -> np.ndarray:
    """gates: iterable of (type, q0, q1, param, angle) -> structured array."""
    arr = np.zeros(len(gates), dtype=GATE_DTYPE)
    for i, g in enumerate(gates):
        arr[i] = tuple(g)
    return arr


def ansatz(n: int, layers: int, entangler: str = "cnot") -> np.ndarray:
    """RY layer, RZ layer, then CNOT ladder q->q+1 ("cnot") or CZ ring ("cz")
    (learning/quantum_pipeline_impl.c:2459-2529)."""
    g = []
    p = 0
    for _ in range(layers):
        for q in range(n):
            g.append((RY, q, -1, p, 0.0)); p += 1
        for q in range(n):
            g.append((RZ, q, -1, p, 0.0)); p += 1
        if entangler == "cnot":
            for q in range(n - 1):
                g.append((CNOT, q, q + 1, -1, 0.0))
        else:
            nb = n if n >= 3 else n - 1
            for q in range(nb):
                g.append((CZ, q, (q + 1) % n, -1, 0.0))
    return gates_array(g)


def num_params(gates: np.ndarray) -> int:
    ps = gates["param"]
    return int(ps.max()) + 1 if len(ps) and ps.max() >= 0 else 0


def splitmix64_params(seed: int, count: int) -> np.ndarray:
    """Uniform [0, 2pi) angles from a splitmix64 stream (same stream as or_seed_params)."""
    mask = (1 << 64) - 1
    s = seed & mask
    out = np.empty(count)
    for i in range(count):
        s = (s + 0x9E3779B97F4A7C15) & mask
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        z ^= z >> 31
        out[i] = 2.0 * math.pi * ((z >> 11) * (1.0 / 9007199254740992.0))
    return out


class Oracle:
    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build()
        self.lib = C.CDLL(path)
        L = self.lib
        vp, i32, f64, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
        L.or_simulate.argtypes = [i32, vp, i32, vp, vp]
        L.or_derivatives.argtypes = [i32, vp, i32, vp, i32, vp, vp]
        L.or_qgt.argtypes = [sz, i32, vp, vp, vp]
        L.or_tfim_apply.argtypes = [i32, f64, f64, vp, vp]
        L.or_pauli_apply.argtypes = [i32, i32, C.POINTER(C.c_char_p), vp, vp, vp]
        L.or_tfim_energy.argtypes = [i32, f64, f64, vp]
        L.or_tfim_energy.restype = f64
        L.or_energy_grad.argtypes = [sz, i32, vp, vp, vp]
        L.or_param_shift_grad.argtypes = [i32, vp, i32, vp, i32, f64, f64, vp]
        L.or_cholesky_solve.argtypes = [i32, vp, f64, vp, vp, vp]
        L.or_cg_solve.argtypes = [i32, vp, vp, vp, i32, f64]
        L.or_pcg_solve.argtypes = [i32, vp, vp, vp, i32, f64, vp, vp, i32]
        L.or_berry_map.argtypes = [i32, vp, i32, vp, i32, i32, i32, i32, vp]
        L.or_seed_params.argtypes = [C.c_uint64, i32, vp]
        L.or_berry_phase.argtypes = [vp, sz, sz, vp]
        L.or_berry_flux.argtypes = [i32, vp, i32, vp, i32, i32, i32, i32, i32, f64, f64, f64, f64, i32, vp]
        L.or_qgt_job_create.argtypes = [i32, vp, i32, vp, i32, i32, f64, f64, f64, vp, vp, vp, vp]
        L.or_qgt_job_create.restype = vp
        L.or_qgt_job_slices.argtypes = [vp]
        L.or_qgt_job_step.argtypes = [vp]
        L.or_qgt_job_destroy.argtypes = [vp]

    def qgt_job(self, n, gates, theta, nslices, J=1.0, h=1.0, lam=1e-3):
        """A full QGT step on the CPU cut into nslices calls (QGTJob)."""
        return QGTJob(self, n, gates, theta, nslices, J, h, lam)

    def seed_params(self, seed: int, count: int) -> np.ndarray:
        th = np.zeros(count)
        self.lib.or_seed_params(seed, count, _p(th))
        return th

    def simulate(self, n, gates, theta):
        psi = np.zeros(1 << n, dtype=np.complex128)
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        rc = self.lib.or_simulate(n, _p(gates), len(gates), _p(theta), _p(psi))
        assert rc == 0
        return psi

    def derivatives(self, n, gates, theta, P=None):
        P = num_params(gates) if P is None else P
        psi = np.zeros(1 << n, dtype=np.complex128)
        D = np.zeros((P, 1 << n), dtype=np.complex128)
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        rc = self.lib.or_derivatives(n, _p(gates), len(gates), _p(theta), P, _p(psi), _p(D))
        assert rc == 0
        return psi, D

    def qgt_from_states(self, psi, D):
        P = D.shape[0]
        Q = np.zeros((P, P), dtype=np.complex128)
        self.lib.or_qgt(psi.shape[0], P, _p(np.ascontiguousarray(psi)), _p(np.ascontiguousarray(D)), _p(Q))
        return Q

    def qgt(self, n, gates, theta):
        psi, D = self.derivatives(n, gates, theta)
        return self.qgt_from_states(psi, D)

    def tfim_apply(self, n, psi, J=1.0, h=1.0):
        out = np.zeros_like(psi)
        self.lib.or_tfim_apply(n, J, h, _p(np.ascontiguousarray(psi)), _p(out))
        return out

    def pauli_apply(self, n, psi, terms):
        """H psi for terms = [(coeff, "XZIY..."), ...] (character n-1-q acts on qubit q)."""
        strs = (C.c_char_p * len(terms))(*[s.encode() for _, s in terms])
        co = np.ascontiguousarray([c for c, _ in terms], dtype=np.float64)
        out = np.zeros_like(psi)
        self.lib.or_pauli_apply(n, len(terms), strs, _p(co), _p(np.ascontiguousarray(psi)), _p(out))
        return out

    def tfim_energy(self, n, psi, J=1.0, h=1.0):
        return self.lib.or_tfim_energy(n, J, h, _p(np.ascontiguousarray(psi)))

    def energy_grad(self, D, Hpsi):
        g = np.zeros(D.shape[0])
        self.lib.or_energy_grad(D.shape[1], D.shape[0], _p(np.ascontiguousarray(D)), _p(np.ascontiguousarray(Hpsi)), _p(g))
        return g

    def param_shift_grad(self, n, gates, theta, J=1.0, h=1.0):
        P = num_params(gates)
        g = np.zeros(P)
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        self.lib.or_param_shift_grad(n, _p(gates), len(gates), _p(theta), P, J, h, _p(g))
        return g

    def cholesky_solve(self, A, b, lam):
        A = np.ascontiguousarray(A, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        used = np.zeros(1)
        rc = self.lib.or_cholesky_solve(A.shape[0], _p(A), lam, _p(b), _p(x), _p(used))
        if rc != 0:
            raise RuntimeError("cholesky failed")
        return x, float(used[0])

    def cg_solve(self, A, b, max_iter=100, tol=1e-8):
        A = np.ascontiguousarray(A, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        it = self.lib.or_cg_solve(A.shape[0], _p(A), _p(b), _p(x), max_iter, tol)
        return x, it

    def pcg_solve(self, A, b, d, U, max_iter=1000, tol=1e-8):
        A = np.ascontiguousarray(A, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        d = np.ascontiguousarray(d, dtype=np.float64)
        U = np.ascontiguousarray(U, dtype=np.float64)
        x = np.zeros_like(b)
        it = self.lib.or_pcg_solve(A.shape[0], _p(A), _p(b), _p(x), max_iter, tol, _p(d), _p(U), U.shape[1])
        return x, it

    def berry_map(self, n, gates, theta, pa, pb, grid):
        out = np.zeros((grid, grid))
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        rc = self.lib.or_berry_map(n, _p(gates), len(gates), _p(theta), num_params(gates), pa, pb, grid, _p(out))
        assert rc == 0
        return out


    def berry_phase(self, states):
        """prod_i <psi_i|psi_{i+1 mod n}> / |.| as a complex number (0 when a link vanishes)."""
        states = [np.ascontiguousarray(x, dtype=np.complex128) for x in states]
        ptrs = (C.c_void_p * max(len(states), 1))(*[x.ctypes.data for x in states])
        out = np.zeros(2)
        self.lib.or_berry_phase(C.cast(ptrs, C.c_void_p), len(states), states[0].shape[0] if states else 0, _p(out))
        return complex(out[0], out[1])

    def berry_flux(self, n, gates, theta, pa, pb, rows, cols, a0, da, b0, db, periodic=True):
        out = np.zeros((rows, cols))
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        rc = self.lib.or_berry_flux(n, _p(gates), len(gates), _p(theta), len(theta), pa, pb, rows, cols,
                                    a0, da, b0, db, int(bool(periodic)), _p(out))
        assert rc == 0
        return out


class QGTJob:
    """or_qgt_job: one full QGT step (psi, all derivative states, Gram, projector, TFIM energy and
    gradient, Cholesky step) whose work is split over `slices` calls of step(); result() after the
    last one.  Every piece of the work happens exactly once over the slices."""

    def __init__(self, orc, n, gates, theta, nslices, J, h, lam):
        self.orc, self.n = orc, n
        self.gates = np.ascontiguousarray(gates)
        self.theta = np.ascontiguousarray(theta, dtype=np.float64)
        P = self.theta.shape[0]
        self.P = P
        self.Q = np.zeros((P, P), dtype=np.complex128)
        self.grad = np.zeros(P)
        self.energy = np.zeros(1)
        self.natgrad = np.zeros(P)
        self.h = orc.lib.or_qgt_job_create(n, _p(self.gates), len(self.gates), _p(self.theta), P, nslices, J, h, lam,
                                           _p(self.Q), _p(self.grad), _p(self.energy), _p(self.natgrad))
        if not self.h:
            raise MemoryError("or_qgt_job_create failed")
        self.slices = orc.lib.or_qgt_job_slices(self.h)

    def step(self) -> int:
        left = self.orc.lib.or_qgt_job_step(self.h)
        if left < 0:
            raise RuntimeError("or_qgt_job_step: no slice left")
        return left

    def result(self):
        return {"Q": self.Q, "grad": self.grad, "energy": float(self.energy[0]), "natgrad": self.natgrad}

    def close(self):
        if self.h:
            self.orc.lib.or_qgt_job_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Reference:
    """The reference library's own code (compiled from its sources by oracle/Makefile)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        L = self.lib
        vp, i32, f64, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
        L.ref_simulate.argtypes = [i32, vp, vp, vp, vp, i32, vp]
        L.ref_pauli_expectation.argtypes = [vp, i32, C.c_char_p]
        L.ref_pauli_expectation.restype = f64
        L.ref_fubini_study.argtypes = [vp, sz, vp, sz, vp]
        L.ref_berry_curvature.argtypes = [vp, sz, vp, sz, vp]
        L.ref_natural_gradient_cg.argtypes = [vp, vp, vp, sz]
        L.ref_invert_qfim_regularized.argtypes = [vp, vp, sz, C.c_float]
        L.ref_berry_phase.argtypes = [vp, sz, sz, vp]
        L.ref_matrix_inverse.argtypes = [vp, vp, sz]
        L.ref_matrix_inverse.restype = i32

    @staticmethod
    def available(path: str = REF_SO) -> bool:
        return os.path.exists(path)

    def matrix_inverse(self, M):
        """matrix_inverse (core/matrix_operations.c:176-217: LU with partial pivoting in ComplexFloat)
        -> (ok, inverse as complex64)."""
        a = np.ascontiguousarray(M, dtype=np.complex64)
        inv = np.zeros_like(a)
        ok = self.lib.ref_matrix_inverse(_p(a), _p(inv), a.shape[0])
        return bool(ok), inv

    def simulate(self, n, gates, theta):
        G = len(gates)
        types = np.ascontiguousarray(gates["type"], dtype=np.int32)
        q0 = np.ascontiguousarray(gates["q0"], dtype=np.int32)
        q1 = np.ascontiguousarray(gates["q1"], dtype=np.int32)
        ang = np.array([theta[g["param"]] if g["param"] >= 0 else g["angle"] for g in gates], dtype=np.float64)
        sv = np.zeros(1 << n, dtype=np.complex128)
        rc = self.lib.ref_simulate(n, _p(types), _p(q0), _p(q1), _p(ang), G, _p(sv))
        assert rc == 0
        return sv

    def derivatives_shift(self, n, gates, theta):
        """d psi/d theta_k = (psi(theta + pi/2 e_k) - psi(theta - pi/2 e_k)) / (2 sqrt 2),
        each psi from the reference simulator (exact for exp(-i theta G/2), G^2 = I)."""
        P = num_params(gates)
        D = np.zeros((P, 1 << n), dtype=np.complex128)
        th = np.array(theta, dtype=np.float64)
        for k in range(P):
            o = th[k]
            th[k] = o + math.pi / 2
            a = self.simulate(n, gates, th)
            th[k] = o - math.pi / 2
            b = self.simulate(n, gates, th)
            th[k] = o
            D[k] = (a - b) / (2.0 * math.sqrt(2.0))
        return D

    def fubini_study(self, psi, D):
        P = D.shape[0]
        out = np.zeros((P, P))
        rc = self.lib.ref_fubini_study(_p(psi), psi.shape[0], _p(np.ascontiguousarray(D)), P, _p(out))
        assert rc == 0
        return out

    def berry_curvature(self, psi, D):
        """Reference normalisation: F = -2 Im Q (differential_geometry.c:2899)."""
        P = D.shape[0]
        out = np.zeros((P, P))
        rc = self.lib.ref_berry_curvature(_p(psi), psi.shape[0], _p(np.ascontiguousarray(D)), P, _p(out))
        assert rc == 0
        return out

    def berry_phase(self, states):
        """diffgeo_compute_berry_phase (differential_geometry.c:2908-2945) as a complex number."""
        states = [np.ascontiguousarray(x, dtype=np.complex128) for x in states]
        ptrs = (C.c_void_p * max(len(states), 1))(*[x.ctypes.data for x in states])
        out = np.zeros(2)
        self.lib.ref_berry_phase(C.cast(ptrs, C.c_void_p), len(states), states[0].shape[0] if states else 0, _p(out))
        return complex(out[0], out[1])

    def pauli_expectation(self, psi, n, pauli: str) -> float:
        return self.lib.ref_pauli_expectation(_p(psi), n, pauli.encode())

    def tfim_energy(self, psi, n, J=1.0, h=1.0) -> float:
        e = 0.0
        for coeff, s in tfim_pauli_strings(n, J, h):
            e += coeff * self.pauli_expectation(psi, n, s)
        return e

    def param_shift_grad(self, n, gates, theta, J=1.0, h=1.0):
        P = num_params(gates)
        g = np.zeros(P)
        th = np.array(theta, dtype=np.float64)
        for k in range(P):
            o = th[k]
            th[k] = o + math.pi / 2
            ep = self.tfim_energy(self.simulate(n, gates, th), n, J, h)
            th[k] = o - math.pi / 2
            em = self.tfim_energy(self.simulate(n, gates, th), n, J, h)
            th[k] = o
            g[k] = (ep - em) / 2.0
        return g

    def natural_gradient_cg(self, F, g):
        F = np.ascontiguousarray(F, dtype=np.float64)
        g = np.ascontiguousarray(g, dtype=np.float64)
        x = np.zeros_like(g)
        self.lib.ref_natural_gradient_cg(_p(F), _p(g), _p(x), F.shape[0])
        return x

    def invert_qfim_regularized(self, F, lam):
        F = np.ascontiguousarray(F, dtype=np.float32)
        inv = np.zeros_like(F)
        rc = self.lib.ref_invert_qfim_regularized(_p(F), _p(inv), F.shape[0], lam)
        assert rc == 0
        return inv


def tfim_pauli_strings(n: int, J: float = 1.0, h: float = 1.0):
    """TFIM ring H = -J sum Z_i Z_{i+1 mod n} - h sum X_i as (coeff, string) terms;
    string character [n-1-q] acts on qubit q (hybrid/quantum_classical_algorithms.c:339)."""
    terms = []
    nb = n if n >= 3 else n - 1
    for b in range(nb):
        s = ["I"] * n
        s[n - 1 - b] = "Z"
        s[n - 1 - ((b + 1) % n)] = "Z"
        terms.append((-J, "".join(s)))
    for q in range(n):
        s = ["I"] * n
        s[n - 1 - q] = "X"
        terms.append((-h, "".join(s)))
    return terms


# ---------------------------------------------------------------------------
# natural-gradient configurations of the reference entry points (restated)
# ---------------------------------------------------------------------------

def condition_number_f32(G):
    """compute_complex_matrix_condition_number (core/quantum_geometric_gradient.c:2733-2781): the
    singular values of the ComplexFloat matrix (LAPACK, as the reference's lapack_svd), then
    sigma_max / sigma_min over the positive ones in float; inf when sigma_min <= 1e-15."""
    s = np.linalg.svd(np.asarray(G, dtype=np.complex64), compute_uv=False).astype(np.float32)
    mx = s.max()
    pos = s[s > 0]
    mn = pos.min() if pos.size else np.float32(0)
    return float(np.float32(mx / mn)) if mn > np.float32(1e-15) else math.inf


def pseudoinverse_natural_gradient(g, G, cutoff):
    """compute_pseudoinverse_natural_gradient (core/quantum_geometric_gradient.c:2800-2884):
    x = V S^+ U^H g with singular values <= cutoff dropped (FP64 here)."""
    U, s, Vh = np.linalg.svd(np.asarray(G, dtype=np.complex128))
    t = U.conj().T @ np.asarray(g, dtype=np.complex128)
    t = np.where(s > cutoff, t / np.where(s > 0, s, 1), 0)
    return Vh.conj().T @ t


def regularized_natural_gradient(ref, g, G, reg=1e-4, threshold=1e8, adaptive=True, pinv=True, cutoff=1e-10):
    """compute_regularized_natural_gradient (core/quantum_geometric_gradient.c:2887-2964): lambda from
    the config, raised to 1e-6 sqrt(kappa) when kappa exceeds the threshold; x = (G + lambda I)^-1 g
    with the reference's own matrix_inverse (ComplexFloat LU); when that reports a singular matrix,
    the pseudo-inverse of the unregularised G.  -> (x, lambda, kappa, path) with path "lu" / "pinv"."""
    lam = np.float32(reg)
    kappa = None
    if adaptive:
        kappa = condition_number_f32(G)
        if kappa > threshold:
            a = np.float32(1e-6) * np.float32(math.sqrt(np.float32(kappa)))
            if a > lam:
                lam = a
    M = np.array(G, dtype=np.complex64)
    M[np.diag_indices_from(M)] += lam
    ok, inv = ref.matrix_inverse(M)
    if ok:
        return (inv @ np.asarray(g, dtype=np.complex64)).astype(np.complex128), float(lam), kappa, "lu"
    if not pinv:
        return None, float(lam), kappa, "fail"
    return pseudoinverse_natural_gradient(g, G, cutoff), float(lam), kappa, "pinv"
