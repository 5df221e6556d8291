"""The reference-compatible entry points (QGTN object, metric / curvature /
full-QGT objects, natural gradient) on the GPU against the golden fixtures.
Outputs are ComplexFloat (the reference ABI): tolerance 2e-7 absolute."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


class ComplexFloat(C.Structure):
    _fields_ = [("real", C.c_float), ("imag", C.c_float)]


class Metric(C.Structure):
    _fields_ = [("type", C.c_int), ("dimension", C.c_size_t), ("components", C.POINTER(ComplexFloat)),
                ("is_symmetric", C.c_bool), ("aux", C.c_void_p), ("hardware", C.c_int)]


class Curvature(C.Structure):
    _fields_ = [("type", C.c_int), ("dimension", C.c_size_t), ("components", C.POINTER(ComplexFloat)),
                ("aux", C.c_void_p), ("is_flat", C.c_bool), ("hardware", C.c_int)]


@pytest.fixture(scope="module")
def L():
    import quantum_geometric_tensor_gb300 as Q
    L = Q.lib()
    vp, sz = C.c_void_p, C.c_size_t
    L.create_quantum_geometric_tensor_network.argtypes = [sz, sz, C.c_bool, C.c_bool]
    L.create_quantum_geometric_tensor_network.restype = vp
    L.destroy_quantum_geometric_tensor_network.argtypes = [vp]
    for f in ("create_rx_gate", "create_ry_gate", "create_rz_gate"):
        getattr(L, f).argtypes = [sz, C.c_double]
        getattr(L, f).restype = vp
    for f in ("create_h_gate", "create_x_gate", "create_y_gate", "create_z_gate"):
        getattr(L, f).argtypes = [sz]
        getattr(L, f).restype = vp
    for f in ("create_cnot_gate", "create_cz_gate"):
        getattr(L, f).argtypes = [sz, sz]
        getattr(L, f).restype = vp
    L.create_quantum_gate.argtypes = [C.c_int, C.POINTER(sz), sz, C.POINTER(C.c_double), sz]
    L.create_quantum_gate.restype = vp
    L.destroy_quantum_gate.argtypes = [vp]
    L.apply_quantum_gate.argtypes = [vp, vp, C.POINTER(sz), sz]
    L.apply_quantum_gate.restype = C.c_bool
    L.count_trainable_parameters.argtypes = [vp]
    L.count_trainable_parameters.restype = sz
    L.geometric_compute_full_qgt.argtypes = [vp, vp, sz]
    L.geometric_create_metric.argtypes = [C.POINTER(C.POINTER(Metric)), C.c_int, sz]
    L.geometric_compute_fubini_study_metric.argtypes = [C.POINTER(Metric), vp, sz]
    L.geometric_destroy_metric.argtypes = [C.POINTER(Metric)]
    L.geometric_create_curvature.argtypes = [C.POINTER(C.POINTER(Curvature)), C.c_int, sz]
    L.geometric_compute_berry_curvature.argtypes = [C.POINTER(Curvature), vp, sz]
    L.geometric_destroy_curvature.argtypes = [C.POINTER(Curvature)]
    L.compute_quantum_geometric_tensor.argtypes = [vp, sz, sz, C.POINTER(ComplexFloat)]
    L.compute_quantum_geometric_tensor.restype = C.c_bool
    L.get_quantum_state.argtypes = [vp, C.POINTER(C.POINTER(ComplexFloat)), C.POINTER(sz)]
    L.get_quantum_state.restype = C.c_bool
    L.compute_quantum_gradient.argtypes = [vp, sz, C.POINTER(C.POINTER(ComplexFloat)), C.POINTER(sz)]
    L.compute_quantum_gradient.restype = C.c_bool
    L.compute_natural_gradient_gpu.argtypes = [vp, vp, vp, sz]
    L.compute_regularized_natural_gradient.argtypes = [vp, vp, vp, sz, vp]
    L.compute_regularized_natural_gradient.restype = C.c_bool
    L.qgtn_set_precision.argtypes = [vp, C.c_int]
    L.qgtn_set_precision.restype = C.c_bool
    L.get_quantum_geometric_tensor_network_error.restype = C.c_char_p
    return L


def build_qgtn(L, n, gates, theta):
    q = L.create_quantum_geometric_tensor_network(n, 1, False, True)
    assert q
    for g in gates:
        t, q0, q1, p, a = int(g[0]), int(g[1]), int(g[2]), int(g[3]), float(g[4])
        ang = theta[p] if p >= 0 else a
        if t in (O.RX, O.RY, O.RZ):
            gp = {O.RX: L.create_rx_gate, O.RY: L.create_ry_gate, O.RZ: L.create_rz_gate}[t](q0, ang)
            qs = (C.c_size_t * 1)(q0)
            nq = 1
            if p < 0:
                # fixed-angle rotations are not parameters of the reference QGTN; use a U1-free form
                pass
        elif t in (O.CNOT, O.CZ):
            gp = {O.CNOT: L.create_cnot_gate, O.CZ: L.create_cz_gate}[t](q0, q1)
            qs = (C.c_size_t * 2)(q0, q1)
            nq = 2
        else:
            gp = L.create_quantum_gate(t, (C.c_size_t * 1)(q0), 1, None, 0)
            qs = (C.c_size_t * 1)(q0)
            nq = 1
        assert gp
        assert L.apply_quantum_gate(q, gp, qs, nq), L.get_quantum_geometric_tensor_network_error()
        L.destroy_quantum_gate(gp)
    return q


HEA = [p for p in GOLDEN if "hea_" in p or "single" in p]


@pytest.mark.parametrize("path", HEA, ids=[os.path.basename(p)[:-4] for p in HEA])
def test_full_qgt_metric_curvature(L, path):
    z = np.load(path)
    n, theta = int(z["n"]), z["theta"]
    P = len(theta)
    q = build_qgtn(L, n, z["gates"].tolist(), theta)
    assert L.count_trainable_parameters(q) == P
    out = (ComplexFloat * (P * P))()
    assert L.geometric_compute_full_qgt(out, q, P) == 0
    Qg = np.array([[out[i * P + j].real + 1j * out[i * P + j].imag for j in range(P)] for i in range(P)])
    assert np.abs(Qg - z["Q"]).max() < 2e-7
    m = C.POINTER(Metric)()
    assert L.geometric_create_metric(C.byref(m), 2, P) == 0   # GEOMETRIC_METRIC_FUBINI_STUDY
    assert L.geometric_compute_fubini_study_metric(m, q, P) == 0
    g = np.array([[m.contents.components[i * P + j].real for j in range(P)] for i in range(P)])
    assert np.abs(g - z["metric"]).max() < 2e-7
    L.geometric_destroy_metric(m)
    c = C.POINTER(Curvature)()
    assert L.geometric_create_curvature(C.byref(c), 4, P) == 0   # GEOMETRIC_CURVATURE_BERRY
    assert L.geometric_compute_berry_curvature(c, q, P) == 0
    w = np.array([[c.contents.components[i * P + j].real for j in range(P)] for i in range(P)])
    assert np.abs(w - z["Q"].imag * (1 - np.eye(P))).max() < 2e-7
    L.geometric_destroy_curvature(c)
    e = ComplexFloat()
    assert L.compute_quantum_geometric_tensor(q, 0, P - 1, C.byref(e))
    assert abs(e.real - z["Q"][0, P - 1].real) < 2e-7
    sv = C.POINTER(ComplexFloat)()
    dim = C.c_size_t()
    assert L.get_quantum_state(q, C.byref(sv), C.byref(dim))
    psi = np.array([sv[i].real + 1j * sv[i].imag for i in range(dim.value)])
    assert np.abs(psi - z["psi"]).max() < 2e-7
    # mixed precision behind the same entry point
    assert L.qgtn_set_precision(q, 1)
    assert L.geometric_compute_full_qgt(out, q, P) == 0
    Qm = np.array([[out[i * P + j].real + 1j * out[i * P + j].imag for j in range(P)] for i in range(P)])
    assert np.abs(Qm - z["Q"]).max() < 1e-5
    L.destroy_quantum_geometric_tensor_network(q)


def test_quantum_gradient_states(L, orc):
    z = np.load([p for p in GOLDEN if "hea_cnot_n4" in p][0])
    n, theta = int(z["n"]), z["theta"]
    q = build_qgtn(L, n, z["gates"].tolist(), theta)
    psi, D = orc.derivatives(n, z["gates"], theta)
    for k in (0, 3, len(theta) - 1):
        gp = C.POINTER(ComplexFloat)()
        dim = C.c_size_t()
        assert L.compute_quantum_gradient(q, k, C.byref(gp), C.byref(dim))
        d = np.array([gp[i].real + 1j * gp[i].imag for i in range(dim.value)])
        assert np.abs(d - D[k]).max() < 2e-7
    L.destroy_quantum_geometric_tensor_network(q)


def test_natural_gradient_entry_points(L):
    z = np.load([p for p in GOLDEN if "hea_cz_n6" in p][0])
    g = z["metric"]
    P = g.shape[0]
    lam = float(z["lam"])
    A = g + lam * np.eye(P)
    x = np.zeros(P)
    L.compute_natural_gradient_gpu(A.ctypes.data, z["grad"].ctypes.data, x.ctypes.data, P)
    assert np.linalg.norm(x - z["natgrad_cg"]) / np.linalg.norm(z["natgrad_cg"]) < 1e-6
    Gc = (ComplexFloat * (P * P))(*[ComplexFloat(float(v), 0.0) for v in g.ravel()])
    gc = (ComplexFloat * P)(*[ComplexFloat(float(v), 0.0) for v in z["grad"]])
    xc = (ComplexFloat * P)()
    # regularisation lambda, no adaptive step
    cfg = (C.c_float * 5)()
    C.memmove(cfg, (C.c_float * 1)(lam), 4)
    raw = bytearray(C.string_at(C.addressof(cfg), 20))
    # natural_gradient_config_t {float lambda; float kappa; bool adaptive; bool pinv; float cutoff}
    import struct
    buf = C.create_string_buffer(struct.pack("ff??xxf", lam, 1e8, False, True, 1e-10), 16)
    assert L.compute_regularized_natural_gradient(gc, Gc, xc, P, buf)
    xr = np.array([xc[i].real for i in range(P)])
    ref = np.linalg.solve(A, z["grad"])
    assert np.linalg.norm(xr - ref) / np.linalg.norm(ref) < 1e-5
