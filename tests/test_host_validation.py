"""Argument checks of the C ABI that run before any device call (CPU, no GPU):
plan options and circuits through the host-side schedule builder
(qgt_plan_schedule_dump shares qgt_plan_create's checks), and the Berry-flux
lattice options.  Every bad input returns -1 (E_INVAL) with a message naming
the argument, as the reference's entry points return an error code instead
of running on bad input."""
import ctypes as C
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    L = Q.lib()
    L.qgt_plan_schedule_dump.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p]
    L.qgt_last_error.restype = C.c_char_p
    return Q


def dump(Q, tmp_path, n, gates, P, **opts):
    L = Q.lib()
    d = Q.circuit_desc(n, gates, P)
    o = Q.PlanOptions()
    L.qgt_plan_default_options(C.byref(o))
    for k, v in opts.items():
        setattr(o, k, v)
    path = str(tmp_path / "schedule.json").encode()
    rc = L.qgt_plan_schedule_dump(C.cast(C.pointer(d), C.c_void_p), C.cast(C.pointer(o), C.c_void_p), path)
    return rc, L.qgt_last_error().decode()


def test_valid_circuit_builds_a_schedule(Q, tmp_path):
    rc, _ = dump(Q, tmp_path, 6, Q.ansatz_gates(6, 2, "cnot"), 24)
    assert rc == 0


@pytest.mark.parametrize("case,words", [
    ("qubits0", "num_qubits 0"),
    ("qubits31", "num_qubits 31"),
    ("qubit_range", "gate qubit 4"),
    ("same_qubits", "two distinct qubits"),
    ("param_range", "gate parameter 3"),
    ("nan_angle", "non-finite"),
    ("precision", "unknown precision"),
    ("hamiltonian", "unknown Hamiltonian"),
    ("batch", "batch 70000"),
    ("deriv", "num_deriv_params 9"),
    ("lambda", "lambda"),
    ("lambda_nan", "lambda"),
])
def test_bad_plan_arguments_are_rejected(Q, tmp_path, case, words):
    g = Q.ansatz_gates(4, 1, "cnot")
    args = {
        "qubits0": (0, [], 0, {}),
        "qubits31": (31, [], 0, {}),
        "qubit_range": (4, [(Q.RY, 4, -1, 0, 0.0)], 1, {}),
        "same_qubits": (4, [(Q.CNOT, 1, 1, -1, 0.0)], 0, {}),
        "param_range": (4, [(Q.RY, 0, -1, 3, 0.0)], 2, {}),
        "nan_angle": (4, [(Q.RY, 0, -1, -1, float("nan"))], 0, {}),
        "precision": (4, g, 8, {"precision": 7}),
        "hamiltonian": (4, g, 8, {"hamiltonian": 9}),
        "batch": (4, g, 8, {"batch": 70000}),
        "deriv": (4, g, 8, {"num_deriv_params": 9}),
        "lambda": (4, g, 8, {"lambda_": -1.0}),
        "lambda_nan": (4, g, 8, {"lambda_": float("nan")}),
    }[case]
    rc, msg = dump(Q, tmp_path, args[0], args[1], args[2], **args[3])
    assert rc == -1 and words in msg, msg


@pytest.mark.parametrize("kw", [dict(pa=1, pb=1), dict(pa=0, pb=12), dict(pa=-1, pb=0), dict(rows=1),
                                dict(cols=5000), dict(da=math.inf), dict(periodic=2), dict(precision=3)])
def test_bad_flux_lattices_are_rejected(Q, kw):
    """Rejected before any plan is made (no device needed)."""
    L = Q.lib()
    n = 6
    g = Q.ansatz_gates(n, 1, "cnot")
    th = np.zeros(2 * n)
    d = Q.circuit_desc(n, g, 2 * n)
    o = Q.FluxOptions()
    L.qgt_flux_default_options(C.byref(o))
    a = dict(pa=0, pb=1, rows=4, cols=4, da=0.1, periodic=1, precision=1)
    a.update(kw)
    o.param_a, o.param_b, o.rows, o.cols, o.da = a["pa"], a["pb"], a["rows"], a["cols"], a["da"]
    o.periodic, o.precision = a["periodic"], a["precision"]
    F = np.zeros((max(a["rows"], 1), max(a["cols"], 1)))
    rc = L.qgt_berry_flux_grid(C.byref(d), th.ctypes.data_as(C.c_void_p), C.byref(o),
                               F.ctypes.data_as(C.c_void_p), None)
    assert rc == -1, L.qgt_last_error()


def test_flux_rejects_non_finite_theta(Q):
    L = Q.lib()
    n = 6
    g = Q.ansatz_gates(n, 1, "cnot")
    th = np.zeros(2 * n)
    th[5] = np.nan
    d = Q.circuit_desc(n, g, 2 * n)
    F = np.zeros((32, 32))
    rc = L.qgt_berry_flux_grid(C.byref(d), th.ctypes.data_as(C.c_void_p), None, F.ctypes.data_as(C.c_void_p), None)
    assert rc == -1 and b"theta[5]" in L.qgt_last_error()
