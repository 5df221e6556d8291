"""GPU contraction from given states (qgt_qgt_from_states and the reference's
diffgeo entry points) against the oracle and the golden fixtures.
Tolerances: FP64 1e-12 relative; mixed (states rounded to complex64, split
FP16 x3 tensor-core Gram) 1e-6 relative on Q."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    Q.lib()
    return Q


@pytest.mark.parametrize("n,L,ent,seed", [(10, 4, "cnot", 1), (12, 3, "cz", 2), (16, 2, "cnot", 3)])
def test_states_contraction(Q, orc, n, L, ent, seed):
    g = O.ansatz(n, L, ent)
    th = O.splitmix64_params(seed, O.num_params(g))
    psi, D = orc.derivatives(n, g, th)
    Qref = orc.qgt_from_states(psi, D)
    Q64 = Q.qgt_from_states(psi, D, Q.FP64)
    assert rel(Q64, Qref) < 1e-12
    # Gram error alone: exact states rounded once to complex64, then split
    p32 = psi.astype(np.complex64).astype(np.complex128)
    D32 = D.astype(np.complex64).astype(np.complex128)
    Qr32 = orc.qgt_from_states(p32, D32)
    for prec in (Q.MIXED, Q.MIXED_BF16X3):
        Qm = Q.qgt_from_states(psi, D, prec)
        print(f"n={n} prec={prec}: vs exact {rel(Qm, Qref):.2e}  vs c64-rounded states {rel(Qm, Qr32):.2e} "
              f"(rounding alone {rel(Qr32, Qref):.2e})")
        if prec == Q.MIXED:
            assert rel(Qm, Qref) < 1e-6


def test_diffgeo_dropin_matches_golden(Q):
    L = Q.lib()
    L.diffgeo_engine_create.restype = C.c_void_p
    L.diffgeo_engine_destroy.argtypes = [C.c_void_p]
    L.diffgeo_compute_fubini_study.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p]
    L.diffgeo_compute_fubini_study.restype = C.c_bool
    L.diffgeo_compute_berry_curvature.argtypes = L.diffgeo_compute_fubini_study.argtypes
    L.diffgeo_compute_berry_curvature.restype = C.c_bool
    orc = O.Oracle()
    for path in GOLDEN:
        z = np.load(path)
        n = int(z["n"])
        psi, D = orc.derivatives(n, z["gates"], z["theta"])
        P = D.shape[0]
        e = L.diffgeo_engine_create()
        g = np.zeros((P, P))
        F = np.zeros((P, P))
        assert L.diffgeo_compute_fubini_study(e, psi.ctypes.data, psi.shape[0], D.ctypes.data, P, g.ctypes.data)
        assert L.diffgeo_compute_berry_curvature(e, psi.ctypes.data, psi.shape[0], D.ctypes.data, P, F.ctypes.data)
        L.diffgeo_engine_destroy(e)
        assert rel(g, z["metric"]) < 1e-12
        assert np.abs(F - z["berry_F"]).max() < 1e-12
