"""Host-side parts of the reference tensor lifecycle (no GPU work):
geometric_tensor_initialize_random / _identity (reference
include/quantum_geometric/core/quantum_geometric_tensor.h:25-27; behaviour of
src/quantum_geometric/core/quantum_geometric_tensor.c:257-340 and
quantum_geometric_tensor_cpu.c:837-863), and the natural-gradient fixture
against the oracle's restatement (reference CG / LU when the compiled
reference is present)."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle as O

HERMITIAN, UNITARY = 6, 5


class Tensor(C.Structure):
    _fields_ = [("type", C.c_int), ("dimensions", C.POINTER(C.c_size_t)), ("rank", C.c_size_t),
                ("dimension", C.c_size_t), ("components", C.c_void_p), ("num_spins", C.c_size_t),
                ("aux", C.c_void_p), ("is_symmetric", C.c_bool), ("is_unitary", C.c_bool),
                ("is_hermitian", C.c_bool), ("hardware", C.c_int), ("mem_type", C.c_int),
                ("total_elements", C.c_size_t), ("aligned_elements", C.c_size_t)]


@pytest.fixture(scope="module")
def L():
    import quantum_geometric_tensor_gb300 as Q
    L = Q.lib()
    T = C.POINTER(Tensor)
    L.geometric_tensor_create.argtypes = [C.POINTER(T), C.c_int, C.POINTER(C.c_size_t), C.c_size_t]
    L.geometric_tensor_destroy.argtypes = [T]
    L.geometric_tensor_initialize_random.argtypes = [T, C.c_float, C.c_float]
    L.geometric_tensor_initialize_identity.argtypes = [T]
    return L


def make(L, ttype, dims):
    t = C.POINTER(Tensor)()
    d = (C.c_size_t * len(dims))(*dims)
    assert L.geometric_tensor_create(C.byref(t), ttype, d, len(dims)) == 0
    return t


def comps(t):
    n = t.contents.total_elements
    a = np.ctypeslib.as_array(C.cast(t.contents.components, C.POINTER(C.c_float)), shape=(2 * n,))
    return a[0::2] + 1j * a[1::2]


def test_initialize_identity(L):
    t = make(L, HERMITIAN, [5, 5])
    assert L.geometric_tensor_initialize_random(t, -1.0, 1.0) == 0
    assert L.geometric_tensor_initialize_identity(t) == 0
    assert np.array_equal(comps(t).reshape(5, 5), np.eye(5))
    L.geometric_tensor_destroy(t)
    t = make(L, UNITARY, [4, 3])
    assert L.geometric_tensor_initialize_identity(t) == -22     # square rank-2 only
    L.geometric_tensor_destroy(t)
    t = make(L, UNITARY, [4, 4, 4])
    assert L.geometric_tensor_initialize_identity(t) == -22
    L.geometric_tensor_destroy(t)
    assert L.geometric_tensor_initialize_identity(None) == -1


def test_initialize_random(L):
    t = make(L, UNITARY, [6, 7])
    assert L.geometric_tensor_initialize_random(t, 1.0, 1.0) == -1   # empty range
    assert L.geometric_tensor_initialize_random(t, -2.0, 3.0) == 0
    a = comps(t)
    assert np.allclose(np.abs(a), 1.0, atol=1e-6)                    # unit modulus
    first = a.copy()
    assert L.geometric_tensor_initialize_random(t, -2.0, 3.0) == 0
    assert not np.array_equal(first, comps(t))                         # a fresh stream per call
    L.geometric_tensor_destroy(t)
    t = make(L, HERMITIAN, [9, 9])
    assert L.geometric_tensor_initialize_random(t, 0.5, 2.0) == 0
    H = comps(t).reshape(9, 9)
    assert np.array_equal(H, H.conj().T)
    d = np.diag(H)
    assert np.all(d.imag == 0) and np.all((d.real >= 0.5) & (d.real <= 2.0))
    off = H[~np.eye(9, dtype=bool)]
    assert np.allclose(np.abs(off), 1.0, atol=1e-6)
    L.geometric_tensor_destroy(t)


Z = np.load(os.path.join(os.path.dirname(__file__), "golden", "natgrad", "natgrad_reg.npz"))


def test_natgrad_fixture_pseudoinverse_restatement():
    G, g = Z["rank16_pinv_only__G"], Z["rank16_pinv_only__g"]
    x = O.pseudoinverse_natural_gradient(g, G, 1e-6)
    assert np.linalg.norm(x - Z["rank16_pinv_only__pinv_x"]) <= 1e-12 * np.linalg.norm(x)


@pytest.mark.skipif(not O.Reference.available(), reason="compiled reference absent (oracle/_ref)")
def test_natgrad_fixture_matches_reference_code():
    ref = O.Reference()
    for case in sorted({k.split("__")[0] for k in Z.files if k.endswith("__cfg")}):
        reg, thr, adaptive, pinv, cutoff = Z[f"{case}__cfg"]
        x, lam, _, path = O.regularized_natural_gradient(ref, Z[f"{case}__g"], Z[f"{case}__G"], reg, thr,
                                                         bool(adaptive), bool(pinv), cutoff)
        assert path == str(Z[f"{case}__path"]) and lam == float(Z[f"{case}__lambda"])
        assert np.array_equal(x, Z[f"{case}__x"])
    F, g = Z["cg_rankdef__F"], Z["cg_rankdef__g"]
    assert np.linalg.norm(ref.natural_gradient_cg(F, g) - Z["cg_rankdef__x"]) < 1e-12 * np.linalg.norm(Z["cg_rankdef__x"])
