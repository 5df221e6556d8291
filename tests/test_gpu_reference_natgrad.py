"""The reference's natural-gradient entry points and state metric on the GPU.

compute_complex_matrix_condition_number, compute_regularized_natural_gradient
(default configuration included: adaptive lambda, LU, pseudo-inverse fallback),
compute_pseudoinverse_natural_gradient, compute_natural_gradient_gpu and
geometric_compute_metric, through the C ABI, against
tests/golden/natgrad/natgrad_reg.npz (the reference's own LU inverse and CG,
restated flow of core/quantum_geometric_gradient.c:2887-2964) and against an
FP64 numpy solve of the same ComplexFloat input.

Tolerances: the library computes in FP64 and returns ComplexFloat, so against
the FP64 solve 1e-6 relative; the reference computes in FP32, so against its
fixture 1e-3 relative (its LU and inverse-times-gradient rounding).  The
reference's matrix_inverse solves each column in place over its right-hand
side, so any row swap of its pivoting corrupts the inverse
(core/matrix_operations.c:145-147, 204); the fixture records that residual and
the comparison with the reference's output is made where it is small.  The
condition number of a matrix whose smallest singular values sit below FP32
resolution depends on rounding (the circuit QGT with the default
configuration): there the check is against the FP64 singular values of the
same ComplexFloat input, with the lambda that condition number selects."""
import ctypes as C
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

Z = np.load(os.path.join(os.path.dirname(__file__), "golden", "natgrad", "natgrad_reg.npz"))
CASES = sorted({k.split("__")[0] for k in Z.files if k.endswith("__cfg")})


class NGConfig(C.Structure):
    _fields_ = [("regularization_param", C.c_float), ("condition_threshold", C.c_float),
                ("use_adaptive_regularization", C.c_bool), ("use_pseudoinverse_fallback", C.c_bool),
                ("singular_value_cutoff", C.c_float)]


class Metric(C.Structure):
    _fields_ = [("type", C.c_int), ("dimension", C.c_size_t), ("components", C.c_void_p),
                ("is_symmetric", C.c_bool), ("aux", C.c_void_p), ("hardware", C.c_int)]


class State(C.Structure):
    _fields_ = [("type", C.c_int), ("num_qubits", C.c_size_t), ("dimension", C.c_size_t),
                ("manifold_dim", C.c_size_t), ("coordinates", C.c_void_p), ("metric", C.c_void_p),
                ("connection", C.c_void_p), ("auxiliary_data", C.c_void_p), ("is_normalized", C.c_bool),
                ("hardware", C.c_int), ("lattice_width", C.c_size_t), ("lattice_height", C.c_size_t),
                ("num_stabilizers", C.c_size_t), ("num_plaquettes", C.c_size_t), ("num_vertices", C.c_size_t),
                ("stabilizers", C.c_void_p), ("num_anyons", C.c_size_t), ("max_anyons", C.c_size_t),
                ("anyons", C.c_void_p), ("syndrome_values", C.c_void_p), ("syndrome_size", C.c_size_t),
                ("measurement_confidence", C.c_void_p), ("confidence_size", C.c_size_t)]


@pytest.fixture(scope="module")
def L():
    import quantum_geometric_tensor_gb300 as Q
    L = Q.lib()
    vp, sz = C.c_void_p, C.c_size_t
    L.compute_complex_matrix_condition_number.argtypes = [vp, sz, C.POINTER(C.c_float)]
    L.compute_complex_matrix_condition_number.restype = C.c_bool
    L.compute_regularized_natural_gradient.argtypes = [vp, vp, vp, sz, C.POINTER(NGConfig)]
    L.compute_regularized_natural_gradient.restype = C.c_bool
    L.compute_pseudoinverse_natural_gradient.argtypes = [vp, vp, vp, sz, C.c_float]
    L.compute_pseudoinverse_natural_gradient.restype = C.c_bool
    L.get_default_natural_gradient_config.restype = NGConfig
    L.compute_natural_gradient_gpu.argtypes = [vp, vp, vp, sz]
    L.geometric_create_metric.argtypes = [C.POINTER(C.POINTER(Metric)), C.c_int, sz]
    L.geometric_destroy_metric.argtypes = [C.POINTER(Metric)]
    L.geometric_compute_metric.argtypes = [C.POINTER(Metric), C.POINTER(State)]
    return L


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def kappa_of(L, G):
    k = C.c_float()
    G = np.ascontiguousarray(G, dtype=np.complex64)
    assert L.compute_complex_matrix_condition_number(G.ctypes.data, G.shape[0], C.byref(k))
    return float(k.value)


def kappa64(G):
    s = np.linalg.svd(np.asarray(G, dtype=np.complex128), compute_uv=False)
    pos = s[s > 0]
    return s.max() / pos.min() if pos.size and pos.min() > 1e-15 else math.inf


def test_default_config_matches_reference(L):
    c = L.get_default_natural_gradient_config()
    assert c.regularization_param == np.float32(1e-4) and c.condition_threshold == np.float32(1e8)
    assert c.use_adaptive_regularization and c.use_pseudoinverse_fallback
    assert c.singular_value_cutoff == np.float32(1e-10)


@pytest.mark.parametrize("case", CASES)
def test_regularized_natural_gradient(L, case):
    G = Z[f"{case}__G"]
    g = Z[f"{case}__g"]
    reg, thr, adaptive, pinv, cutoff = Z[f"{case}__cfg"]
    P = G.shape[0]
    kap = kappa_of(L, G)
    k64 = kappa64(G)
    if math.isfinite(k64):
        assert abs(kap - k64) <= 1e-4 * k64, (kap, k64)
    else:
        assert math.isinf(kap)
    cfg = NGConfig(reg, thr, bool(adaptive), bool(pinv), cutoff)
    x = np.zeros(P, dtype=np.complex64)
    assert L.compute_regularized_natural_gradient(np.ascontiguousarray(g).ctypes.data,
                                                   np.ascontiguousarray(G).ctypes.data, x.ctypes.data, P,
                                                   C.byref(cfg))
    # the lambda this condition number selects (float arithmetic, as the reference)
    lam = np.float32(reg)
    if adaptive and kap > thr:
        lam = max(lam, np.float32(1e-6) * np.float32(math.sqrt(np.float32(kap))))
    path = str(Z[f"{case}__path"])
    if path == "lu":
        x64 = np.linalg.solve(G.astype(np.complex128) + float(lam) * np.eye(P), g.astype(np.complex128))
    else:
        U, s, Vh = np.linalg.svd(G.astype(np.complex128))
        t = U.conj().T @ g.astype(np.complex128)
        x64 = Vh.conj().T @ np.where(s > cutoff, t / np.where(s > 0, s, 1), 0)
    assert rel(x, x64) < 1e-6, rel(x, x64)
    if case != "circuit_qgt_default":   # kappa (and so lambda) of that case is set by FP32 rounding
        assert float(Z[f"{case}__lambda"]) == pytest.approx(float(lam), rel=1e-6)
        # the reference's own LU inverse is only right when no pivot swaps rows (its permutation
        # runs in place over the right-hand side it reads): compare where its residual is small
        if path == "pinv" or float(Z[f"{case}__ref_inverse_residual"]) < 1e-4:
            assert rel(x, Z[f"{case}__x"]) < 1e-3, rel(x, Z[f"{case}__x"])


def test_regularized_without_fallback_fails_on_singular(L):
    G = Z["singular_after_lambda__G"]
    g = Z["singular_after_lambda__g"]
    cfg = NGConfig(1e-4, 1e8, False, False, 1e-10)
    x = np.zeros(G.shape[0], dtype=np.complex64)
    assert not L.compute_regularized_natural_gradient(g.ctypes.data, G.ctypes.data, x.ctypes.data, G.shape[0],
                                                       C.byref(cfg))


def test_pseudoinverse_natural_gradient(L):
    G = Z["rank16_pinv_only__G"]
    g = Z["rank16_pinv_only__g"]
    x = np.zeros(G.shape[0], dtype=np.complex64)
    assert L.compute_pseudoinverse_natural_gradient(g.ctypes.data, G.ctypes.data, x.ctypes.data, G.shape[0], 1e-6)
    assert rel(x, Z["rank16_pinv_only__pinv_x"]) < 1e-5
    # every singular value of a non-square-free unitary is 1: kappa 1, pinv = inverse
    rng = np.random.default_rng(4)
    Uq, _ = np.linalg.qr(rng.standard_normal((33, 33)) + 1j * rng.standard_normal((33, 33)))
    Uq = Uq.astype(np.complex64)
    assert kappa_of(L, Uq) == pytest.approx(1.0, abs=1e-5)
    b = (rng.standard_normal(33) + 1j * rng.standard_normal(33)).astype(np.complex64)
    y = np.zeros(33, dtype=np.complex64)
    assert L.compute_pseudoinverse_natural_gradient(b.ctypes.data, Uq.ctypes.data, y.ctypes.data, 33, 1e-10)
    assert rel(y, np.linalg.solve(Uq.astype(np.complex128), b.astype(np.complex128))) < 1e-6


def test_condition_number_of_singular_matrix_is_infinite(L):
    G = np.zeros((6, 6), dtype=np.complex64)
    G[0, 0] = 1.0
    assert math.isinf(kappa_of(L, np.zeros((6, 6), dtype=np.complex64)))
    assert kappa_of(L, G) == pytest.approx(1.0)   # the reference takes the smallest POSITIVE singular value


def test_natural_gradient_gpu_is_the_reference_cg(L):
    for z_F, z_g, z_x in (("cg_rankdef__F", "cg_rankdef__g", "cg_rankdef__x"),):
        F, g = Z[z_F], Z[z_g]
        x = np.zeros_like(g)
        L.compute_natural_gradient_gpu(F.ctypes.data, g.ctypes.data, x.ctypes.data, g.shape[0])
        assert rel(x, Z[z_x]) < 1e-7
        assert rel(F @ x, g) < 1e-7


@pytest.mark.parametrize("n", [3, 7])
def test_geometric_compute_metric(L, n):
    dim = 1 << n
    rng = np.random.default_rng(n)
    psi = (rng.standard_normal(dim) + 1j * rng.standard_normal(dim)).astype(np.complex64)
    psi /= np.linalg.norm(psi)
    st = State()
    st.dimension, st.num_qubits, st.coordinates = dim, n, psi.ctypes.data
    EUCL, MINK, FS = 0, 1, 2
    m = C.POINTER(Metric)()
    assert L.geometric_create_metric(C.byref(m), FS, dim) == 0
    assert L.geometric_compute_metric(m, C.byref(st)) == 0
    M = np.ctypeslib.as_array(C.cast(m.contents.components, C.POINTER(C.c_float)), shape=(dim * dim * 2,))
    M = (M[0::2] + 1j * M[1::2]).reshape(dim, dim)
    ref = np.eye(dim) - np.outer(psi.conj(), psi)
    assert np.abs(M - ref).max() < 1e-6
    L.geometric_destroy_metric(m)
    # Euclidean leaves the components alone; Minkowski is not implemented (as in the reference);
    # mismatched dimensions are invalid
    m = C.POINTER(Metric)()
    assert L.geometric_create_metric(C.byref(m), EUCL, dim) == 0
    before = np.ctypeslib.as_array(C.cast(m.contents.components, C.POINTER(C.c_float)), shape=(dim * dim * 2,)).copy()
    assert L.geometric_compute_metric(m, C.byref(st)) == 0
    after = np.ctypeslib.as_array(C.cast(m.contents.components, C.POINTER(C.c_float)), shape=(dim * dim * 2,))
    assert np.array_equal(before, after)
    L.geometric_destroy_metric(m)
    m = C.POINTER(Metric)()
    assert L.geometric_create_metric(C.byref(m), MINK, dim) == 0
    assert L.geometric_compute_metric(m, C.byref(st)) == -7
    L.geometric_destroy_metric(m)
    m = C.POINTER(Metric)()
    assert L.geometric_create_metric(C.byref(m), FS, dim + 1) == 0
    assert L.geometric_compute_metric(m, C.byref(st)) == -1
    L.geometric_destroy_metric(m)
