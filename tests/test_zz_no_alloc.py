"""qgt_cholesky_solve_f64_noalloc (static device scratch, no allocation)
against qgt_cholesky_solve_f64 through the C ABI.  Both run the same FP64
kernel, so results agree to 1e-13 relative; two calls in a row check that
the reused scratch carries nothing from one call into the next."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_P = 512


@pytest.fixture(scope="module")
def L():
    import quantum_geometric_tensor_gb300 as Q
    lib = Q.lib()
    vp = C.c_void_p
    lib.qgt_cholesky_solve_f64_noalloc.argtypes = [vp, vp, C.c_double, C.c_int32, vp, vp]
    lib.qgt_cholesky_solve_f64_noalloc.restype = C.c_int
    lib.qgt_cholesky_solve_f64.argtypes = [vp, vp, C.c_double, C.c_int32, vp, vp]
    lib.qgt_cholesky_solve_f64.restype = C.c_int
    lib.qgt_last_error.restype = C.c_char_p
    return lib


def solve(lib, fn, A, g, lam):
    A = np.ascontiguousarray(A, dtype=np.float64)
    g = np.ascontiguousarray(g, dtype=np.float64)
    x = np.zeros(len(g))
    used = C.c_double(0)
    rc = getattr(lib, fn)(A.ctypes.data, g.ctypes.data, lam, len(g), x.ctypes.data, C.byref(used))
    return rc, x, used.value


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def spd(P, seed):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((P, P))
    return M @ M.T / P, rng.standard_normal(P)


@pytest.mark.parametrize("P", [1, 40, 320, MAX_P])
def test_matches_allocating_solve_twice(L, P):
    A1, g1 = spd(P, 10 + P)
    A2, g2 = spd(P, 20 + P)
    for A, g in ((A1, g1), (A2, g2)):   # two calls in a row, different systems
        rc0, x0, u0 = solve(L, "qgt_cholesky_solve_f64", A, g, 1e-3)
        rc1, x1, u1 = solve(L, "qgt_cholesky_solve_f64_noalloc", A, g, 1e-3)
        assert rc0 == 0 and rc1 == 0, L.qgt_last_error()
        assert u1 == u0 == 1e-3
        assert rel(x1, x0) < 1e-13
        assert rel((A + 1e-3 * np.eye(P)) @ x1, g) < 1e-9


def test_lambda_retry_matches(L):
    B = np.diag(np.r_[np.ones(39), -0.05])
    b = np.ones(40)
    rc0, x0, u0 = solve(L, "qgt_cholesky_solve_f64", B, b, 1e-3)
    rc1, x1, u1 = solve(L, "qgt_cholesky_solve_f64_noalloc", B, b, 1e-3)
    assert rc0 == rc1 == 0
    assert u1 == pytest.approx(u0) and u1 == pytest.approx(0.1)
    assert rel(x1, x0) < 1e-13


def test_rejects_beyond_static_maximum(L):
    P = MAX_P + 1
    A, g = np.eye(P), np.ones(P)
    rc, _, _ = solve(L, "qgt_cholesky_solve_f64_noalloc", A, g, 1e-3)
    assert rc != 0
    assert b"exceeds the static scratch maximum 512" in L.qgt_last_error()
