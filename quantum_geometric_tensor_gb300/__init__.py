"""GB300-native quantum geometric tensor engine (Python view of libqgt_gb300.so).

The product is the C ABI in ``include/``: ``libqgt_gb300.so`` (C11 host code +
sm_103a CUDA kernels).  This module only loads that library with ctypes and
wraps the plan entry points with numpy; it contains no numerics of its own and
has no fallback: if the library is missing it raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libqgt_gb300.so")

# gate codes (reference gate_type_t values)
I, X, Y, Z, H, S, T, RX, RY, RZ, CNOT, CZ, SWAP = 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 13
FP64, MIXED, MIXED_BF16X3 = 0, 1, 2
HAM_NONE, HAM_TFIM, HAM_PAULI = 0, 1, 2
TRANSPORT_AUTO, TRANSPORT_FORWARD, TRANSPORT_MEET = 0, 1, 2
PASS_AUTO, PASS_INTERPRET, PASS_COMPILED = 0, 1, 2


class GateDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("qubits", C.c_int32 * 2), ("param", C.c_int32), ("angle", C.c_double)]


class CircuitDesc(C.Structure):
    _fields_ = [("num_qubits", C.c_int32), ("num_gates", C.c_int32), ("gates", C.POINTER(GateDesc)),
                ("num_params", C.c_int32)]


class PlanOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("hamiltonian", C.c_int), ("tfim_J", C.c_double), ("tfim_h", C.c_double),
                ("lambda_", C.c_double), ("device", C.c_int32), ("use_graph", C.c_int32), ("batch", C.c_int32),
                ("num_deriv_params", C.c_int32), ("num_pauli_terms", C.c_int32), ("pauli_strings", C.c_char_p),
                ("pauli_coeffs", C.c_void_p), ("transport", C.c_int32), ("tile_bits", C.c_int32),
                ("pass_kernels", C.c_int32), ("thread_amps", C.c_int32)]


class PlanInfo(C.Structure):
    _fields_ = [("num_qubits", C.c_int32), ("num_params", C.c_int32), ("num_slots", C.c_int32),
                ("num_rows", C.c_int32), ("num_passes", C.c_int32), ("num_launches", C.c_int32),
                ("tile_bits", C.c_int32), ("vector_passes", C.c_int64), ("gate_bytes", C.c_int64),
                ("gram_flops", C.c_int64), ("device_bytes", C.c_int64), ("batch", C.c_int32),
                ("num_deriv_params", C.c_int32), ("meet_in_middle", C.c_int32), ("cut_gate", C.c_int32),
                ("jit_passes", C.c_int32), ("thread_amps", C.c_int32)]


class BatchOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("berry_grid", C.c_int32), ("device", C.c_int32), ("streams", C.c_int32),
                ("tune_cache", C.c_char_p)]


class BatchInfo(C.Structure):
    _fields_ = [("num_circuits", C.c_int32), ("num_groups", C.c_int32), ("num_berry_plans", C.c_int32),
                ("graph_kernels", C.c_int32), ("device_bytes", C.c_int64)]


class FluxOptions(C.Structure):
    _fields_ = [("param_a", C.c_int32), ("param_b", C.c_int32), ("rows", C.c_int32), ("cols", C.c_int32),
                ("a0", C.c_double), ("da", C.c_double), ("b0", C.c_double), ("db", C.c_double),
                ("periodic", C.c_int32), ("precision", C.c_int), ("device", C.c_int32)]


class PrecondConfig(C.Structure):
    _fields_ = [("num_params", C.c_int32), ("width", C.c_int32), ("rank", C.c_int32), ("lam", C.c_double),
                ("u_scale", C.c_double), ("seed", C.c_uint64), ("device", C.c_int32)]


class PrecondTrainOptions(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_double), ("weight_decay", C.c_double),
                ("seed", C.c_uint64)]


class VQEOptions(C.Structure):
    _fields_ = [("steps", C.c_int32), ("eta", C.c_double), ("pcg_tol", C.c_double), ("pcg_max_iter", C.c_int32),
                ("solver", C.c_int32)]


VQE_CHOLESKY, VQE_CG, VQE_PCG_LEARNED = 0, 1, 2


class StepProfile(C.Structure):
    _fields_ = [("total_ms", C.c_double), ("prepare_ms", C.c_double), ("passes_ms", C.c_double),
                ("hamiltonian_ms", C.c_double), ("gram_ms", C.c_double), ("post_ms", C.c_double),
                ("solve_ms", C.c_double)]


_lib = None


def lib() -> C.CDLL:
    """Load libqgt_gb300.so (built by __graft_entry__.build()); raise if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libqgt_gb300.so not built ({LIB_PATH}); run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.qgt_plan_default_options.argtypes = [C.POINTER(PlanOptions)]
        L.qgt_plan_create.argtypes = [C.POINTER(CircuitDesc), C.POINTER(PlanOptions), C.POINTER(vp)]
        L.qgt_plan_destroy.argtypes = [vp]
        L.qgt_plan_get_info.argtypes = [vp, C.POINTER(PlanInfo)]
        L.qgt_plan_execute_host.argtypes = [vp, vp, vp, vp, vp, vp]
        L.qgt_plan_execute_device.argtypes = [vp, vp, vp, vp, vp, vp]
        L.qgt_plan_synchronize.argtypes = [vp]
        L.qgt_plan_stream.argtypes = [vp]
        L.qgt_plan_stream.restype = vp
        L.qgt_plan_get_state.argtypes = [vp, vp]
        L.qgt_plan_get_row.argtypes = [vp, C.c_int, vp]
        L.qgt_plan_device_status.argtypes = [vp, vp]
        L.qgt_cholesky_solve_f64.argtypes = [vp, vp, C.c_double, C.c_int32, vp, vp]
        L.qgt_plan_profile_step.argtypes = [vp, C.POINTER(StepProfile)]
        L.qgt_plan_test_gram_stall.argtypes = [vp, C.c_int, C.c_int64]
        L.qgt_batch_default_options.argtypes = [C.POINTER(BatchOptions)]
        L.qgt_batch_create.argtypes = [vp, C.c_int32, vp, C.POINTER(BatchOptions), C.POINTER(vp)]
        L.qgt_batch_execute_host.argtypes = [vp, vp, vp, vp]
        L.qgt_batch_get_info.argtypes = [vp, C.POINTER(BatchInfo)]
        L.qgt_batch_execute_device.argtypes = [vp]
        L.qgt_batch_stream.argtypes = [vp]
        L.qgt_batch_stream.restype = vp
        L.qgt_batch_destroy.argtypes = [vp]
        L.qgt_flux_default_options.argtypes = [C.POINTER(FluxOptions)]
        L.qgt_berry_flux_grid.argtypes = [C.POINTER(CircuitDesc), vp, C.POINTER(FluxOptions), vp, vp]
        L.qgt_precond_default_config.argtypes = [C.POINTER(PrecondConfig)]
        L.qgt_precond_default_train_options.argtypes = [C.POINTER(PrecondTrainOptions)]
        L.qgt_precond_create.argtypes = [C.POINTER(PrecondConfig), C.POINTER(vp)]
        L.qgt_precond_destroy.argtypes = [vp]
        L.qgt_precond_num_weights.argtypes = [vp]
        L.qgt_precond_num_weights.restype = C.c_int64
        L.qgt_precond_get_weights.argtypes = [vp, vp]
        L.qgt_precond_set_weights.argtypes = [vp, vp]
        L.qgt_precond_loss_grad.argtypes = [vp, vp, vp, C.c_int32, vp, vp]
        L.qgt_precond_predict.argtypes = [vp, vp, C.c_int32, vp, vp]
        L.qgt_precond_train.argtypes = [vp, vp, vp, C.c_int32, C.POINTER(PrecondTrainOptions), vp]
        L.qgt_precond_train_circuit.argtypes = [vp, C.POINTER(CircuitDesc), vp, C.c_int32, C.c_int,
                                                C.POINTER(PrecondTrainOptions), vp]
        L.qgt_metric_dataset.argtypes = [C.POINTER(CircuitDesc), vp, C.c_int32, C.c_int, C.c_int32, vp]
        L.qgt_pcg_solve_f64.argtypes = [vp, vp, C.c_double, C.c_int32, vp, vp, C.c_int32, C.c_double, C.c_int32,
                                        vp, vp, vp]
        L.qgt_vqe_default_options.argtypes = [C.POINTER(VQEOptions)]
        L.qgt_vqe_run.argtypes = [C.POINTER(CircuitDesc), C.POINTER(PlanOptions), vp, C.POINTER(VQEOptions), vp,
                                  vp, vp, vp]
        L.qgt_last_error.restype = C.c_char_p
        L.qgt_version.restype = C.c_char_p
        _lib = L
    return _lib


class QGTError(RuntimeError):
    def __init__(self, code, where):
        super().__init__(f"{where}: error {code}: {lib().qgt_last_error().decode()}")
        self.code = code


def _check(rc, where):
    if rc != 0:
        raise QGTError(rc, where)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def circuit_desc(n: int, gates, num_params: int | None = None):
    """gates: iterable of (type, q0, q1, param, angle) or a structured array with those fields."""
    arr = (GateDesc * max(1, len(gates)))()
    maxp = -1
    for i, g in enumerate(gates):
        t, q0, q1, p, a = (int(g[0]), int(g[1]), int(g[2]), int(g[3]), float(g[4]))
        arr[i].type = t
        arr[i].qubits[0] = q0
        arr[i].qubits[1] = q1
        arr[i].param = p
        arr[i].angle = a
        maxp = max(maxp, p)
    P = maxp + 1 if num_params is None else num_params
    d = CircuitDesc(n, len(gates), C.cast(arr, C.POINTER(GateDesc)), P)
    d._keep = arr
    return d


def seeded_params(seed: int, count: int) -> np.ndarray:
    """`count` angles uniform in [0, 2 pi) from a splitmix64 stream started at `seed`: state
    s_i = seed + i * 0x9E3779B97F4A7C15 (mod 2^64), the splitmix64 finaliser of s_i, its top 53
    bits as a fraction of 2 pi.  The workloads' seeded parameter vectors."""
    with np.errstate(over="ignore"):
        s = np.uint64(seed & ((1 << 64) - 1)) + np.arange(1, count + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
        z = (s ^ (s >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z ^= z >> np.uint64(31)
    return 2.0 * np.pi * ((z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0))


def ansatz_gates(n: int, layers: int, entangler: str = "cnot"):
    """RY layer, RZ layer, then CNOT ladder q->q+1 ("cnot") or CZ ring ("cz")."""
    g, p = [], 0
    for _ in range(layers):
        for q in range(n):
            g.append((RY, q, -1, p, 0.0)); p += 1
        for q in range(n):
            g.append((RZ, q, -1, p, 0.0)); p += 1
        if entangler == "cnot":
            g += [(CNOT, q, q + 1, -1, 0.0) for q in range(n - 1)]
        else:
            nb = n if n >= 3 else n - 1
            g += [(CZ, q, (q + 1) % n, -1, 0.0) for q in range(nb)]
    return g


class Plan:
    """A compiled circuit plan (qgt_plan_t)."""

    def __init__(self, n, gates, num_params=None, precision=MIXED, hamiltonian=HAM_TFIM, J=1.0, h=1.0,
                 lam=1e-3, device=0, use_graph=True, batch=1, deriv_params=0, pauli=None, transport=0,
                 tile_bits=0, pass_kernels=0, thread_amps=0):
        """pauli: [(coeff, "XZIY..."), ...] selects the Pauli-sum Hamiltonian (character n-1-q acts on qubit q)."""
        L = lib()
        self.desc = circuit_desc(n, gates, num_params)
        o = PlanOptions()
        L.qgt_plan_default_options(C.byref(o))
        o.precision, o.hamiltonian, o.tfim_J, o.tfim_h = precision, hamiltonian, J, h
        if pauli is not None:
            strs = "".join(s_ for _, s_ in pauli)
            if any(len(s_) != n for _, s_ in pauli):
                raise ValueError("every Pauli string needs one character per qubit")
            self._pauli = (strs.encode(), np.ascontiguousarray([c for c, _ in pauli], dtype=np.float64))
            o.hamiltonian, o.num_pauli_terms = HAM_PAULI, len(pauli)
            o.pauli_strings = self._pauli[0]
            o.pauli_coeffs = self._pauli[1].ctypes.data
        o.lambda_, o.device, o.use_graph = lam, device, int(use_graph)
        o.batch, o.num_deriv_params, o.transport = int(batch), int(deriv_params), int(transport)
        o.tile_bits, o.pass_kernels, o.thread_amps = int(tile_bits), int(pass_kernels), int(thread_amps)
        self.opt = o
        h_ = C.c_void_p()
        _check(L.qgt_plan_create(C.byref(self.desc), C.byref(o), C.byref(h_)), "qgt_plan_create")
        self.h = h_
        self.n, self.P = n, self.desc.num_params
        self.B = int(batch)
        self.Pd = int(deriv_params) if deriv_params else self.P

    def info(self) -> PlanInfo:
        i = PlanInfo()
        _check(lib().qgt_plan_get_info(self.h, C.byref(i)), "qgt_plan_get_info")
        return i

    def output_buffers(self, want=("Q", "grad", "energy", "natgrad")):
        """Host arrays for run(..., out=): reusing them across steps saves the
        allocation and first-touch page faults of fresh outputs."""
        B, P = self.B, self.Pd
        return {"Q": np.zeros((B, P, P), dtype=np.complex128) if "Q" in want else None,
                "grad": np.zeros((B, P)) if "grad" in want else None,
                "energy": np.zeros(B) if "energy" in want else None,
                "natgrad": np.zeros((B, P)) if "natgrad" in want else None}

    def run(self, theta, want=("Q", "grad", "energy", "natgrad"), out=None):
        """One step.  theta: (P,) or, for a batched plan, (batch, P); outputs
        gain a leading batch axis when batch > 1.  out: arrays from
        output_buffers() to write into (their set replaces `want`)."""
        B, P = self.B, self.Pd
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        if theta.size != B * self.P:
            raise ValueError(f"theta has {theta.size} values, plan wants {B} x {self.P}")
        if out is None:
            out = self.output_buffers(want)
        for k, shape, dt in (("Q", (B, P, P), np.complex128), ("grad", (B, P), np.float64),
                             ("energy", (B,), np.float64), ("natgrad", (B, P), np.float64)):
            a = out.get(k)
            if a is not None and (a.shape != shape or a.dtype != dt or not a.flags.c_contiguous):
                raise ValueError(f"out[{k!r}] must be a C-contiguous {dt.__name__} array of shape {shape}")
        Q, g, e, x = out.get("Q"), out.get("grad"), out.get("energy"), out.get("natgrad")
        _check(lib().qgt_plan_execute_host(self.h, _ptr(theta), _ptr(Q), _ptr(g), _ptr(e), _ptr(x)),
               "qgt_plan_execute_host")
        if B == 1:
            return {"Q": None if Q is None else Q[0], "grad": None if g is None else g[0],
                    "energy": None if e is None else float(e[0]), "natgrad": None if x is None else x[0]}
        return {"Q": Q, "grad": g, "energy": e, "natgrad": x}

    def state(self):
        psi = np.zeros(1 << self.n, dtype=np.complex128)
        _check(lib().qgt_plan_get_state(self.h, _ptr(psi)), "qgt_plan_get_state")
        return psi

    def row(self, r):
        v = np.zeros(1 << self.n, dtype=np.complex128)
        _check(lib().qgt_plan_get_row(self.h, r, _ptr(v)), "qgt_plan_get_row")
        return v

    def status(self):
        lam = np.zeros(1)
        st = lib().qgt_plan_device_status(self.h, _ptr(lam))
        return st, float(lam[0])

    def stream(self) -> int:
        return lib().qgt_plan_stream(self.h) or 0

    def test_gram_stall(self, stall: bool, timeout_ns: int = 0):
        """Fault-injection hook (qgt_plan_test_gram_stall): with stall the digit Gram's
        bounded waits run out after timeout_ns and the step reports QGT_ERROR_TIMEOUT."""
        _check(lib().qgt_plan_test_gram_stall(self.h, int(bool(stall)), int(timeout_ns)), "qgt_plan_test_gram_stall")

    def close(self):
        if getattr(self, "h", None):
            lib().qgt_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Batch:
    """A ragged batch (qgt_batch_t): circuits = [(n, gates, num_params), ...];
    berry_params = [(a, b), ...] per circuit when grid > 0."""

    def __init__(self, circuits, berry_params=None, precision=MIXED, grid=32, device=0, streams=4, tune_cache=None):
        L = lib()
        self.descs = [circuit_desc(n, g, P) for (n, g, P) in circuits]
        arr = (CircuitDesc * len(self.descs))(*self.descs)
        self._arr = arr
        self.P = [d.num_params for d in self.descs]
        o = BatchOptions()
        L.qgt_batch_default_options(C.byref(o))
        o.precision, o.berry_grid, o.device, o.streams = precision, int(grid), device, int(streams)
        self._tune = None if tune_cache is None else str(tune_cache).encode()
        o.tune_cache = self._tune
        self.G = int(grid)
        bp = None
        if grid > 0:
            bp = np.ascontiguousarray(np.asarray(berry_params, dtype=np.int32).reshape(-1))
        h_ = C.c_void_p()
        _check(L.qgt_batch_create(C.cast(arr, C.c_void_p), len(self.descs), _ptr(bp), C.byref(o), C.byref(h_)),
               "qgt_batch_create")
        self.h = h_

    def info(self) -> BatchInfo:
        i = BatchInfo()
        _check(lib().qgt_batch_get_info(self.h, C.byref(i)), "qgt_batch_get_info")
        return i

    def output_buffers(self):
        """Host arrays for run(..., out=): the QGTs back to back (complex128) and the maps (or None)."""
        return (np.zeros(sum(P * P for P in self.P), dtype=np.complex128),
                np.zeros((len(self.P), self.G, self.G)) if self.G > 0 else None)

    def run(self, thetas, out=None):
        """thetas: one parameter vector per circuit -> (list of P x P complex Q, count x G x G maps or None).
        out: buffers from output_buffers(), reused (the returned matrices are views of them)."""
        th = np.ascontiguousarray(np.concatenate([np.asarray(t, dtype=np.float64).reshape(-1) for t in thetas]))
        Qflat, maps = out if out is not None else self.output_buffers()
        if Qflat.dtype != np.complex128 or Qflat.size != sum(P * P for P in self.P) or not Qflat.flags.c_contiguous:
            raise ValueError("out: QGT buffer of the wrong size or type")
        if self.G > 0 and (maps is None or maps.shape != (len(self.P), self.G, self.G) or maps.dtype != np.float64
                           or not maps.flags.c_contiguous):
            raise ValueError("out: map buffer of the wrong shape or type")
        _check(lib().qgt_batch_execute_host(self.h, _ptr(th), _ptr(Qflat), _ptr(maps)), "qgt_batch_execute_host")
        out, at = [], 0
        for P in self.P:
            out.append(Qflat[at:at + P * P].reshape(P, P))
            at += P * P
        return out, maps

    def run_device(self):
        """The batch on the thetas of the last run(), results left on the device: one asynchronous
        graph launch on stream() (qgt_batch_execute_device)."""
        _check(lib().qgt_batch_execute_device(self.h), "qgt_batch_execute_device")

    def stream(self) -> int:
        return lib().qgt_batch_stream(self.h) or 0

    def close(self):
        if getattr(self, "h", None):
            lib().qgt_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Precond:
    """Learned metric preconditioner (qgt_precond_t)."""

    def __init__(self, P, width=512, rank=16, lam=1e-3, seed=1, device=0):
        L = lib()
        c = PrecondConfig()
        L.qgt_precond_default_config(C.byref(c))
        c.num_params, c.width, c.rank, c.lam, c.seed, c.device = P, width, rank, lam, seed, device
        self.cfg = c
        h_ = C.c_void_p()
        _check(L.qgt_precond_create(C.byref(c), C.byref(h_)), "qgt_precond_create")
        self.h, self.P, self.r = h_, P, rank

    def _opts(self, epochs, batch, lr, seed):
        o = PrecondTrainOptions()
        lib().qgt_precond_default_train_options(C.byref(o))
        o.epochs, o.batch, o.lr, o.seed = epochs, batch, lr, seed
        return o

    def train(self, theta, metric, epochs=30, batch=256, lr=1e-3, seed=7):
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        metric = np.ascontiguousarray(metric, dtype=np.float64)
        o = self._opts(epochs, batch, lr, seed)
        hist = np.zeros(epochs)
        _check(lib().qgt_precond_train(self.h, _ptr(theta), _ptr(metric), theta.shape[0], C.byref(o), _ptr(hist)),
               "qgt_precond_train")
        return hist

    def train_circuit(self, n, gates, theta, precision=MIXED, epochs=30, batch=256, lr=1e-3, seed=7):
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        d = circuit_desc(n, gates, self.P)
        o = self._opts(epochs, batch, lr, seed)
        hist = np.zeros(epochs)
        _check(lib().qgt_precond_train_circuit(self.h, C.byref(d), _ptr(theta), theta.shape[0], precision,
                                               C.byref(o), _ptr(hist)), "qgt_precond_train_circuit")
        return hist

    def predict(self, theta):
        theta = np.ascontiguousarray(np.atleast_2d(theta), dtype=np.float64)
        S = theta.shape[0]
        d = np.zeros((S, self.P))
        U = np.zeros((S, self.P, self.r))
        _check(lib().qgt_precond_predict(self.h, _ptr(theta), S, _ptr(d), _ptr(U)), "qgt_precond_predict")
        return d, U

    def num_weights(self):
        return int(lib().qgt_precond_num_weights(self.h))

    def weights(self):
        w = np.zeros(self.num_weights(), dtype=np.float32)
        _check(lib().qgt_precond_get_weights(self.h, _ptr(w)), "qgt_precond_get_weights")
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        _check(lib().qgt_precond_set_weights(self.h, _ptr(w)), "qgt_precond_set_weights")

    def loss_grad(self, theta, metric):
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        metric = np.ascontiguousarray(metric, dtype=np.float64)
        loss = np.zeros(1)
        g = np.zeros(self.num_weights(), dtype=np.float32)
        _check(lib().qgt_precond_loss_grad(self.h, _ptr(theta), _ptr(metric), theta.shape[0], _ptr(loss), _ptr(g)),
               "qgt_precond_loss_grad")
        return float(loss[0]), g

    def close(self):
        if getattr(self, "h", None):
            lib().qgt_precond_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def metric_dataset(n, gates, theta, precision=FP64, device=0):
    """Re Q of S parameter points (theta S x P) on the GPU -> S x P x P."""
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    S, P = theta.shape
    d = circuit_desc(n, gates, P)
    out = np.zeros((S, P, P))
    _check(lib().qgt_metric_dataset(C.byref(d), _ptr(theta), S, precision, device, _ptr(out)), "qgt_metric_dataset")
    return out


def pcg_solve(A, b, lam, d=None, U=None, tol=1e-10, max_iter=1000):
    """GPU PCG of (A + lam I) x = b with M = diag(d) + U U^T -> (x, iterations, relative residual)."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    P = b.shape[0]
    dd = None if d is None else np.ascontiguousarray(d, dtype=np.float64)
    UU = None if U is None else np.ascontiguousarray(U, dtype=np.float64)
    r = 0 if UU is None else UU.shape[1]
    x = np.zeros(P)
    it = np.zeros(1, dtype=np.int32)
    res = np.zeros(1)
    _check(lib().qgt_pcg_solve_f64(_ptr(A), _ptr(b), lam, P, _ptr(dd), _ptr(UU), r, tol, max_iter, _ptr(x),
                                   _ptr(it), _ptr(res)), "qgt_pcg_solve_f64")
    return x, int(it[0]), float(res[0])


def vqe_run(n, gates, theta0, steps=500, eta=0.05, solver=VQE_CHOLESKY, precond=None, precision=MIXED,
            pcg_tol=1e-10, pcg_max_iter=1000, lam=1e-3):
    """Natural-gradient VQE on the TFIM ring, looped on the device -> (energies, pcg iterations, final theta)."""
    L = lib()
    th0 = np.ascontiguousarray(theta0, dtype=np.float64)
    P = th0.shape[0]
    d = circuit_desc(n, gates, P)
    po = PlanOptions()
    L.qgt_plan_default_options(C.byref(po))
    po.precision, po.lambda_ = precision, lam
    vo = VQEOptions()
    L.qgt_vqe_default_options(C.byref(vo))
    vo.steps, vo.eta, vo.solver, vo.pcg_tol, vo.pcg_max_iter = steps, eta, solver, pcg_tol, pcg_max_iter
    E = np.zeros(steps)
    its = np.zeros(steps, dtype=np.int32)
    th = np.zeros(P)
    _check(L.qgt_vqe_run(C.byref(d), C.byref(po), None if precond is None else precond.h, C.byref(vo), _ptr(th0),
                         _ptr(E), _ptr(its), _ptr(th)), "qgt_vqe_run")
    return E, its, th


def cholesky_solve(A, b, lam):
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    used = np.zeros(1)
    _check(lib().qgt_cholesky_solve_f64(_ptr(A), _ptr(b), lam, A.shape[0], _ptr(x), _ptr(used)),
           "qgt_cholesky_solve_f64")
    return x, float(used[0])


def qgt_from_states(psi, D, precision=FP64):
    """Q from given states on the GPU (qgt_qgt_from_states)."""
    L = lib()
    L.qgt_qgt_from_states.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int, C.c_void_p]
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    D = np.ascontiguousarray(D, dtype=np.complex128)
    P = D.shape[0]
    Q = np.zeros((P, P), dtype=np.complex128)
    _check(L.qgt_qgt_from_states(_ptr(psi), _ptr(D), psi.shape[0], P, precision, _ptr(Q)), "qgt_qgt_from_states")
    return Q


def berry_flux(n, gates, theta, pa, pb, rows, cols, a0, da, b0, db, periodic=True, precision=MIXED, device=0):
    """Plaquette (Wilson-loop) Berry flux over a rows x cols lattice of circuit
    states on the GPU (qgt_berry_flux_grid) -> (flux rows x cols, sum)."""
    L = lib()
    th = np.ascontiguousarray(theta, dtype=np.float64)
    d = circuit_desc(n, gates, th.shape[0])
    o = FluxOptions()
    L.qgt_flux_default_options(C.byref(o))
    o.param_a, o.param_b, o.rows, o.cols = pa, pb, rows, cols
    o.a0, o.da, o.b0, o.db = a0, da, b0, db
    o.periodic, o.precision, o.device = int(bool(periodic)), precision, device
    F = np.zeros((rows, cols))
    tot = np.zeros(1)
    _check(L.qgt_berry_flux_grid(C.byref(d), _ptr(th), C.byref(o), _ptr(F), _ptr(tot)), "qgt_berry_flux_grid")
    return F, float(tot[0])


class _ComplexDouble(C.Structure):
    _fields_ = [("real", C.c_double), ("imag", C.c_double)]


def berry_phase(states):
    """diffgeo_compute_berry_phase on the GPU: prod_i <psi_i|psi_{i+1 mod n}> / |.| as a complex number."""
    L = lib()
    L.diffgeo_engine_create.restype = C.c_void_p
    L.diffgeo_engine_destroy.argtypes = [C.c_void_p]
    L.diffgeo_compute_berry_phase.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t]
    L.diffgeo_compute_berry_phase.restype = _ComplexDouble
    st = [np.ascontiguousarray(x, dtype=np.complex128) for x in states]
    ptrs = (C.c_void_p * max(len(st), 1))(*[x.ctypes.data for x in st])
    e = L.diffgeo_engine_create()
    try:
        r = L.diffgeo_compute_berry_phase(e, C.cast(ptrs, C.c_void_p), len(st), st[0].shape[0] if st else 0)
    finally:
        L.diffgeo_engine_destroy(e)
    return complex(r.real, r.imag)


def autotune(n, gates, num_params=None, precision=MIXED, hamiltonian=HAM_TFIM, batch=1, deriv_params=0, lam=1e-3,
             device=0, cache=None, steps=5):
    """qgt_plan_autotune -> (tile_bits, pass_kernels, thread_amps, ms per step) of the fastest configuration."""
    L = lib()
    L.qgt_plan_autotune.argtypes = [C.POINTER(CircuitDesc), C.POINTER(PlanOptions), C.c_char_p, C.c_int32,
                                    C.POINTER(PlanOptions), C.POINTER(C.c_double)]
    d = circuit_desc(n, gates, num_params)
    o = PlanOptions()
    L.qgt_plan_default_options(C.byref(o))
    o.precision, o.hamiltonian, o.batch, o.num_deriv_params = precision, hamiltonian, int(batch), int(deriv_params)
    o.lambda_, o.device = lam, device
    t = PlanOptions()
    ms = C.c_double()
    _check(L.qgt_plan_autotune(C.byref(d), C.byref(o), None if cache is None else str(cache).encode(), int(steps),
                               C.byref(t), C.byref(ms)), "qgt_plan_autotune")
    return int(t.tile_bits), int(t.pass_kernels), int(t.thread_amps), float(ms.value)
