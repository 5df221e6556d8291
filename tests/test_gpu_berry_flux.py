"""Berry phases of loops on the GPU against the FP64 oracle and the fixtures
made by the reference's own diffgeo_compute_berry_phase.

- diffgeo_compute_berry_phase (reference prototype, GPU overlaps): equal to
  the oracle to 1e-12 on random loops of several sizes; its edge cases
  ({0, 0} for orthogonal neighbours, {1, 0} for fewer than two states).
- qgt_berry_flux_grid (plaquette Wilson loops over a lattice of circuit
  states): FP64 plans to 1e-11 against the fixtures and 1e-10 against the
  oracle, periodic and open lattices, lattices larger than one batched plan;
  mixed (complex64) plans to 2e-5 (absolute, radians); on every wrapped
  lattice the fluxes sum to 2 pi x an integer to 1e-8; for a small
  plaquette flux / (da db) equals 2 Im Q_ab of the plan's own QGT."""
import glob
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

BERRY = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "berry", "*.npz")))


@pytest.fixture(scope="module")
def Q():
    import quantum_geometric_tensor_gb300 as Q
    Q.lib()
    return Q


def chern_residual(F):
    c = F.sum() / (2 * math.pi)
    return abs(c - round(c))


@pytest.mark.parametrize("dim,count", [(16, 3), (4096, 7), (1 << 18, 4)])
def test_berry_phase_matches_oracle(Q, orc, dim, count):
    rng = np.random.default_rng(dim + count)
    st = [rng.standard_normal(dim) + 1j * rng.standard_normal(dim) for _ in range(count)]
    w = Q.berry_phase(st)
    assert abs(w - orc.berry_phase(st)) < 1e-12
    assert abs(abs(w) - 1) < 1e-12


def test_berry_phase_edge_cases(Q):
    a = np.zeros(8, complex)
    a[0] = 1
    b = np.zeros(8, complex)
    b[3] = 1j
    assert Q.berry_phase([a, b, a]) == 0
    assert Q.berry_phase([a]) == 1


def test_berry_phase_of_circuit_loop(Q, orc):
    n = 6
    g = O.ansatz(n, 2, "cnot")
    th = O.splitmix64_params(21, O.num_params(g))
    st = []
    for k in range(24):
        t = th.copy()
        t[2] = 2 * math.pi * k / 24
        st.append(orc.simulate(n, g, t))
    assert abs(Q.berry_phase(st) - orc.berry_phase(st)) < 1e-12


@pytest.mark.parametrize("path", BERRY, ids=[os.path.basename(p)[:-4] for p in BERRY])
def test_flux_fp64_matches_reference_fixture(Q, path):
    z = np.load(path)
    F, tot = Q.berry_flux(int(z["n"]), z["gates"], z["theta"], int(z["pa"]), int(z["pb"]), int(z["rows"]),
                          int(z["cols"]), float(z["a0"]), float(z["da"]), float(z["b0"]), float(z["db"]),
                          periodic=True, precision=Q.FP64)
    assert np.abs(F - z["flux"]).max() < 1e-11
    assert abs(tot - F.sum()) < 1e-12


@pytest.mark.parametrize("periodic", [True, False])
def test_flux_fp64_matches_oracle(Q, orc, periodic):
    n = 8
    g = O.ansatz(n, 2, "cz")
    th = O.splitmix64_params(31, O.num_params(g))
    args = (1, n + 2, 16, 12, 0.1, 2 * math.pi / 16, -0.3, 2 * math.pi / 12)
    ref = orc.berry_flux(n, g, th, *args, periodic=periodic)
    F, _ = Q.berry_flux(n, g, th, *args, periodic=periodic, precision=Q.FP64)
    assert np.abs(F - ref).max() < 1e-10
    if periodic:
        assert chern_residual(F) < 1e-8
    else:
        assert not F[-1].any() and not F[:, -1].any()


def test_flux_lattice_larger_than_one_plan(Q, orc):
    """300 x 300 sites: more than the 65535 points of one batched plan, so the
    lattice rows run in blocks whose edges must join."""
    n = 6
    g = O.ansatz(n, 2, "cnot")
    th = O.splitmix64_params(32, O.num_params(g))
    args = (0, n, 300, 300, 0.0, 2 * math.pi / 300, 0.0, 2 * math.pi / 300)
    ref = orc.berry_flux(n, g, th, *args, periodic=True)
    F, _ = Q.berry_flux(n, g, th, *args, periodic=True, precision=Q.FP64)
    assert np.abs(F - ref).max() < 1e-10
    assert chern_residual(F) < 1e-8


@pytest.mark.parametrize("n,L,ent", [(10, 3, "cz"), (13, 2, "cnot")])
def test_flux_mixed_matches_oracle(Q, orc, n, L, ent):
    g = O.ansatz(n, L, ent)
    th = O.splitmix64_params(40 + n, O.num_params(g))
    args = (0, n, 12, 12, 0.0, 2 * math.pi / 12, 0.0, 2 * math.pi / 12)
    ref = orc.berry_flux(n, g, th, *args, periodic=True)
    F, _ = Q.berry_flux(n, g, th, *args, periodic=True, precision=Q.MIXED)
    err = np.abs(F - ref).max()
    print(f"n={n}: max flux error {err:.2e} rad, max |flux| {np.abs(ref).max():.3f}")
    assert err < 2e-5
    assert chern_residual(F) < 1e-8


def test_flux_mixed_20_qubits_is_quantised(Q):
    """32 x 32 wrapped lattice of 20-qubit states (8 layers, CZ ring)."""
    n = 20
    g = Q.ansatz_gates(n, 8, "cz")
    P = 2 * n * 8
    th = O.splitmix64_params(7, P)
    F, tot = Q.berry_flux(n, g, th, 0, n, 32, 32, 0.0, 2 * math.pi / 32, 0.0, 2 * math.pi / 32)
    assert np.isfinite(F).all() and np.abs(F).max() <= math.pi
    assert chern_residual(F) < 1e-8


def test_flux_mixed_against_fp64_20_qubits(Q):
    n = 20
    g = Q.ansatz_gates(n, 8, "cz")
    th = O.splitmix64_params(9, 2 * n * 8)
    args = (3, 2 * n + 3, 6, 6, 0.2, 0.5, 1.0, 0.45)   # RY(q3) of layers 1 and 2
    F64, _ = Q.berry_flux(n, g, th, *args, periodic=False, precision=Q.FP64)
    F32, _ = Q.berry_flux(n, g, th, *args, periodic=False, precision=Q.MIXED)
    err = np.abs(F32 - F64).max()
    print(f"20 qubits: max flux error mixed vs FP64 {err:.2e} rad, max |flux| {np.abs(F64).max():.3f}")
    assert np.abs(F64).max() > 1e-4 and err < 2e-5


def test_small_plaquette_is_twice_curvature(Q):
    n = 9
    g = Q.ansatz_gates(n, 2, "cz")
    P = 4 * n
    th = O.splitmix64_params(50, P)
    pa, pb, h = 2, n + 4, 1e-3
    with Q.Plan(n, g, P, precision=Q.FP64) as p:
        Qm = p.run(th)["Q"]
    F, _ = Q.berry_flux(n, g, th, pa, pb, 2, 2, th[pa] - h / 2, h, th[pb] - h / 2, h, periodic=False,
                        precision=Q.FP64)
    assert abs(F[0, 0] / h ** 2 - 2 * Qm[pa, pb].imag) < 1e-5


def test_flux_rejects_bad_arguments(Q):
    n = 6
    g = Q.ansatz_gates(n, 1, "cnot")
    th = np.zeros(2 * n)
    for kw in [dict(pa=1, pb=1), dict(pa=0, pb=2 * n), dict(rows=1), dict(precision=Q.MIXED_BF16X3)]:
        a = dict(pa=0, pb=1, rows=4, cols=4, precision=Q.FP64)
        a.update(kw)
        with pytest.raises(Q.QGTError):
            Q.berry_flux(n, g, th, a["pa"], a["pb"], a["rows"], a["cols"], 0.0, 0.1, 0.0, 0.1,
                         precision=a["precision"])
    bad = th.copy()
    bad[3] = np.nan
    with pytest.raises(Q.QGTError):
        Q.berry_flux(n, g, bad, 0, 1, 4, 4, 0.0, 0.1, 0.0, 0.1, precision=Q.FP64)
