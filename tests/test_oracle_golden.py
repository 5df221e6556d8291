"""The FP64 oracle against the golden fixtures made by the reference's own code
(tests/golden/make_golden.py), plus analytic known answers.  CPU only."""
import glob
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
BERRY = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "berry", "*.npz")))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_golden_present():
    assert len(GOLDEN) >= 8


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference(orc, path):
    z = np.load(path)
    n, gates, theta = int(z["n"]), z["gates"], z["theta"]
    psi, D = orc.derivatives(n, gates, theta)
    assert rel(psi, z["psi"]) < 1e-13
    Q = orc.qgt_from_states(psi, D)
    assert rel(Q, z["Q"]) < 1e-12
    assert rel(Q.real, z["metric"]) < 1e-12
    assert rel(-2.0 * Q.imag, z["berry_F"]) < 1e-12 or np.linalg.norm(z["berry_F"]) < 1e-14
    assert abs(orc.tfim_energy(n, psi) - float(z["energy"])) < 1e-12
    g = orc.energy_grad(D, orc.tfim_apply(n, psi))
    assert rel(g, z["grad"]) < 1e-12
    # parameter-shift restatement agrees with the adjoint form and the reference
    if len(theta) <= 40:
        assert rel(orc.param_shift_grad(n, gates, theta), z["grad"]) < 1e-12
    lam = float(z["lam"])
    x, used = orc.cholesky_solve(Q.real, g, lam)
    assert used == lam
    A = Q.real + lam * np.eye(len(theta))
    # the reference CG stops at ||r|| < 1e-8: compare within that residual
    assert np.linalg.norm(A @ z["natgrad_cg"] - g) < 1e-7
    assert np.linalg.norm(A @ x - g) < 1e-10 * max(1.0, np.linalg.norm(g))
    # restated CG follows the reference CG
    xc, it = orc.cg_solve(A, g)
    assert rel(xc, z["natgrad_cg"]) < 1e-6
    # float Cholesky inverse of the reference (single precision)
    inv = z["qfim_inv"].astype(np.float64)
    assert np.linalg.norm(inv @ A - np.eye(len(theta))) < 5e-2 * max(1.0, np.linalg.cond(A) * 1e-4)


def test_single_qubit_known_answers(orc):
    th, ph = 0.9, 0.4
    g = O.gates_array([(O.RY, 0, -1, 0, 0.0), (O.RZ, 0, -1, 1, 0.0)])
    Q = orc.qgt(1, g, np.array([th, ph]))
    assert abs(Q[0, 0].real - 0.25) < 1e-15
    assert abs(Q[1, 1].real - math.sin(th) ** 2 / 4) < 1e-15
    assert abs(Q[0, 1].real) < 1e-15
    assert abs(Q[0, 1].imag - math.sin(th) / 4) < 1e-15


def test_qgt_invariants(orc):
    g = O.ansatz(6, 3, "cnot")
    th = O.splitmix64_params(7, O.num_params(g))
    psi, D = orc.derivatives(6, g, th)
    Q = orc.qgt_from_states(psi, D)
    assert np.abs(Q - Q.conj().T).max() < 1e-15
    assert np.linalg.eigvalsh(Q).min() > -1e-13
    # global phase invariance
    ph = np.exp(0.37j)
    Q2 = orc.qgt_from_states(psi * ph, D * ph)
    assert np.abs(Q2 - Q).max() < 1e-14
    # first-layer RY block on |0...0> is I/4
    assert np.abs(Q[:6, :6].real - 0.25 * np.eye(6)).max() < 1e-14


def test_seed_stream_matches_c(orc):
    a = orc.seed_params(12345, 17)
    b = O.splitmix64_params(12345, 17)
    assert np.array_equal(a, b)
    assert (a >= 0).all() and (a < 2 * math.pi).all()


def test_pcg_with_exact_preconditioner(orc):
    rng = np.random.default_rng(0)
    P, r = 40, 4
    U = rng.standard_normal((P, r))
    d = rng.uniform(0.5, 2.0, P)
    A = np.diag(d) + U @ U.T
    b = rng.standard_normal(P)
    x, it = orc.pcg_solve(A, b, d, U)
    assert it <= 2
    assert rel(x, np.linalg.solve(A, b)) < 1e-10
    x2, it2 = orc.cg_solve(A, b, max_iter=1000, tol=1e-10)
    assert it2 > it


def test_berry_map_matches_full_qgt(orc):
    g = O.ansatz(3, 2, "cnot")
    th = O.splitmix64_params(5, O.num_params(g))
    grid = 4
    m = orc.berry_map(3, g, th, 0, 3, grid)
    for i in range(grid):
        for j in range(grid):
            t = th.copy()
            t[0] = 2 * math.pi * i / grid
            t[3] = 2 * math.pi * j / grid
            Q = orc.qgt(3, g, t)
            assert abs(m[i, j] - Q[0, 3].imag) < 1e-14


def test_pauli_apply_matches_reference_expectation(orc):
    """or_pauli_apply (the oracle's H psi for Pauli sums) against the reference's own
    compute_pauli_expectation term by term (compiled from its sources when present)."""
    try:
        ref = O.Reference()
    except FileNotFoundError:
        pytest.skip("reference objects not built (no reference tree on this host)")
    rng = np.random.default_rng(4)
    n = 5
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    psi /= np.linalg.norm(psi)
    terms = [(float(rng.standard_normal()), "".join(rng.choice(list("IXYZxyz"), n))) for _ in range(12)]
    terms.append((0.7, "XZ"))   # wrong length: contributes nothing
    hp = orc.pauli_apply(n, psi, terms)
    e = float(np.real(np.vdot(psi, hp)))
    e_ref = sum(c * ref.pauli_expectation(psi, n, s) for c, s in terms if len(s) == n)
    assert abs(e - e_ref) < 1e-13
    # the TFIM ring as Pauli strings equals the dedicated TFIM apply
    tf = [(c, s) for c, s in O.tfim_pauli_strings(n)]
    assert np.abs(orc.pauli_apply(n, psi, tf) - orc.tfim_apply(n, psi)).max() < 1e-13


@pytest.mark.parametrize("path", BERRY, ids=[os.path.basename(p)[:-4] for p in BERRY])
def test_berry_flux_and_loop_phase_match_reference(orc, path):
    """Plaquette fluxes and the loop phase of the restated oracle against the
    reference's diffgeo_compute_berry_phase on the reference simulator's states."""
    z = np.load(path)
    n, gates, theta = int(z["n"]), z["gates"], z["theta"]
    rows, cols = int(z["rows"]), int(z["cols"])
    args = (int(z["pa"]), int(z["pb"]), rows, cols, float(z["a0"]), float(z["da"]), float(z["b0"]), float(z["db"]))
    F = orc.berry_flux(n, gates, theta, *args, periodic=True)
    assert np.abs(F - z["flux"]).max() < 1e-12
    # fluxes of a wrapped lattice sum to 2 pi x an integer (each link is met twice)
    c = F.sum() / (2 * math.pi)
    assert abs(c - round(c)) < 1e-10
    Fo = orc.berry_flux(n, gates, theta, *args, periodic=False)
    assert np.array_equal(Fo[:-1, :-1], F[:-1, :-1])
    assert not Fo[-1].any() and not Fo[:, -1].any()
    w = orc.berry_phase(list(z["row0_states"]))
    assert abs(w - complex(z["loop_phase"])) < 1e-12 and abs(abs(w) - 1) < 1e-12


def test_berry_phase_edge_cases(orc):
    a = np.zeros(4, complex)
    a[0] = 1
    b = np.zeros(4, complex)
    b[1] = 1
    assert orc.berry_phase([a, b]) == 0                 # orthogonal neighbours: undefined
    assert orc.berry_phase([a]) == 1                    # fewer than two states
    # invariant under a phase of any one state; conjugating the loop reverses the phase
    rng = np.random.default_rng(3)
    st = [rng.standard_normal(16) + 1j * rng.standard_normal(16) for _ in range(6)]
    w = orc.berry_phase(st)
    st2 = list(st)
    st2[2] = st2[2] * np.exp(0.7j)
    assert abs(orc.berry_phase(st2) - w) < 1e-13
    assert abs(orc.berry_phase(st[::-1]) - np.conj(w)) < 1e-13


def test_small_plaquette_flux_is_twice_curvature(orc):
    """flux / (da db) -> 2 Im Q_ab at the plaquette centre as the spacing shrinks."""
    n = 4
    g = O.ansatz(n, 2, "cz")
    th = O.splitmix64_params(8, O.num_params(g))
    pa, pb, h = 0, n, 1e-3
    F = orc.berry_flux(n, g, th, pa, pb, 2, 2, th[pa] - h / 2, h, th[pb] - h / 2, h, periodic=False)
    psi, D = orc.derivatives(n, g, th)
    Q = orc.qgt_from_states(psi, D)
    assert abs(F[0, 0] / h ** 2 - 2 * Q[pa, pb].imag) < 1e-5


@pytest.mark.parametrize("slices", [1, 3, 7, 1000])
def test_sliced_qgt_job_equals_one_shot(orc, slices):
    """The CPU baseline's sliced full step gives the one-shot oracle's Q, energy, gradient and step."""
    n, L = 8, 3
    g = O.ansatz(n, L, "cz")
    P = O.num_params(g)
    th = O.splitmix64_params(12, P)
    psi, D = orc.derivatives(n, g, th)
    Qref = orc.qgt_from_states(psi, D)
    hp = orc.tfim_apply(n, psi)
    gref = orc.energy_grad(D, hp)
    eref = float(np.vdot(psi, hp).real)
    xref, _ = orc.cholesky_solve(Qref.real, gref, 1e-3)
    job = orc.qgt_job(n, g, th, slices)
    k = 0
    while job.step() > 0:
        k += 1
    assert k + 1 == min(slices, P)
    r = job.result()
    assert np.linalg.norm(r["Q"] - Qref) < 1e-12 * np.linalg.norm(Qref)
    assert np.linalg.norm(r["grad"] - gref) < 1e-12 * np.linalg.norm(gref)
    assert abs(r["energy"] - eref) < 1e-12
    assert np.linalg.norm(r["natgrad"] - xref) < 1e-9 * np.linalg.norm(xref)
    job.close()
