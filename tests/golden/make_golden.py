"""Generate the golden fixtures under tests/golden from the REFERENCE's own code.

Every array in the fixtures comes from reference functions compiled from the
reference tree (oracle/_ref/libqgt_ref.so, built by oracle/Makefile):

  psi        execute_circuit_on_statevector   hybrid/quantum_classical_algorithms.c:278-318
  D          the same simulator at theta +- pi/2 e_k, divided by 2 sqrt 2
  metric     diffgeo_compute_fubini_study     distributed/differential_geometry.c:2819-2862
  berry_F    diffgeo_compute_berry_curvature  distributed/differential_geometry.c:2864-2906
             (F = -2 Im Q; the fixture also stores Q = metric - i F / 2)
  energy     compute_pauli_expectation over the TFIM Pauli strings  (:320-382)
  grad       parameter shift (E+ - E-)/2      hybrid/quantum_classical_algorithms.c:580-640
  natgrad_cg compute_natural_gradient_cpu on (metric + lambda I)
             hybrid/classical_optimization_engine.c:543-611
  qfim_inv   invert_qfim_regularized (float)  learning/quantum_pipeline_impl.c:1601-1682

The Berry-phase fixtures (berry/*.npz) hold states of the same simulator on a
two-parameter lattice and, from diffgeo_compute_berry_phase
(distributed/differential_geometry.c:2908-2945):
  flux       arg of the loop phase of each plaquette p00 -> p10 -> p11 -> p01
             (the Wilson loop of cuda/quantum_phase_cuda.cu:245-313 with
             full-state links), the lattice wrapping at its edges
  loop_phase the loop phase of the lattice's first row of sites

The natural-gradient fixture (natgrad/natgrad_reg.npz) holds, per case, a
metric G and gradient g and the outputs of compute_regularized_natural_gradient
(core/quantum_geometric_gradient.c:2887-2964) restated in oracle.py around the
reference's own LU inverse (core/matrix_operations.c:176-217) with LAPACK
singular values for kappa and the pseudo-inverse, as the reference's lapack_svd.

Only the circuits and seeded angles are chosen here.  Run from the repository
root in a container that has the reference tree (REF = its path):
    make -C oracle REF=... && python tests/golden/make_golden.py          (all fixtures)
    make -C oracle REF=... && python tests/golden/make_golden.py berry    (Berry-phase fixtures only)
    make -C oracle REF=... && python tests/golden/make_golden.py natgrad  (natural-gradient fixture only)
"""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

LAMBDA = 1e-3


def general_circuit():
    """A small circuit with every gate kind the boundary accepts, shared
    parameters and fixed-angle rotations."""
    g = [
        (O.H, 0, -1, -1, 0.0), (O.H, 1, -1, -1, 0.0), (O.X, 2, -1, -1, 0.0),
        (O.RX, 0, -1, 0, 0.0), (O.RY, 1, -1, 1, 0.0), (O.RZ, 2, -1, 2, 0.0),
        (O.CNOT, 0, 3, -1, 0.0), (O.CZ, 1, 4, -1, 0.0), (O.S, 3, -1, -1, 0.0),
        (O.T, 4, -1, -1, 0.0), (O.RY, 3, -1, 3, 0.0), (O.RX, 4, -1, 4, 0.0),
        (O.RZ, 0, -1, -1, 0.7), (O.Y, 1, -1, -1, 0.0), (O.CNOT, 4, 2, -1, 0.0),
        (O.RZ, 1, -1, 5, 0.0), (O.RY, 2, -1, 6, 0.0), (O.Z, 0, -1, -1, 0.0),
        (O.RX, 3, -1, 7, 0.0), (O.CZ, 2, 3, -1, 0.0), (O.RY, 0, -1, 8, 0.0),
        (O.H, 4, -1, -1, 0.0), (O.RZ, 4, -1, 9, 0.0), (O.CNOT, 1, 0, -1, 0.0),
    ]
    return 5, O.gates_array(g)


def cases():
    out = []
    for seed in (0, 1):
        g = O.ansatz(10, 4, "cnot")
        out.append((f"hea_cnot_n10_l4_s{seed}", 10, g, O.splitmix64_params(seed, O.num_params(g))))
    g = O.ansatz(6, 3, "cz")
    out.append(("hea_cz_n6_l3_s2", 6, g, O.splitmix64_params(2, O.num_params(g))))
    g = O.ansatz(8, 2, "cz")
    out.append(("hea_cz_n8_l2_s3", 8, g, O.splitmix64_params(3, O.num_params(g))))
    n, g = general_circuit()
    out.append(("general_n5_s4", n, g, O.splitmix64_params(4, O.num_params(g))))
    g = O.gates_array([(O.RY, 0, -1, 0, 0.0), (O.RZ, 0, -1, 1, 0.0)])
    out.append(("single_qubit_ry_rz", 1, g, np.array([0.9, 0.4])))
    for i, (n, L) in enumerate([(4, 2), (5, 3), (7, 2)]):
        g = O.ansatz(n, L, "cnot")
        out.append((f"hea_cnot_n{n}_l{L}_s{10 + i}", n, g, O.splitmix64_params(10 + i, O.num_params(g))))
    return out


def berry_cases():
    """(name, n, gates, theta, pa, pb, rows, cols, a0, da, b0, db)"""
    g4 = O.ansatz(4, 2, "cz")
    g5 = O.ansatz(5, 2, "cnot")
    return [
        ("berry_cz_n4_l2_s5", 4, g4, O.splitmix64_params(5, O.num_params(g4)), 0, 4, 8, 8,
         0.0, 2 * math.pi / 8, 0.0, 2 * math.pi / 8),
        ("berry_cnot_n5_l2_s6", 5, g5, O.splitmix64_params(6, O.num_params(g5)), 1, 7, 6, 5,
         0.3, 0.4, -0.2, 0.55),
    ]


def berry_main():
    ref = O.Reference()
    for name, n, gates, theta, pa, pb, rows, cols, a0, da, b0, db in berry_cases():
        S = {}
        for i in range(rows):
            for j in range(cols):
                t = np.array(theta, dtype=np.float64)
                t[pa], t[pb] = a0 + i * da, b0 + j * db
                S[i, j] = ref.simulate(n, gates, t)
        flux = np.zeros((rows, cols))
        for i in range(rows):
            for j in range(cols):
                i1, j1 = (i + 1) % rows, (j + 1) % cols
                flux[i, j] = np.angle(ref.berry_phase([S[i, j], S[i1, j], S[i1, j1], S[i, j1]]))
        loop = ref.berry_phase([S[0, j] for j in range(cols)])
        path = os.path.join(ROOT, "tests", "golden", "berry", f"{name}.npz")
        np.savez_compressed(path, n=n, gates=gates, theta=theta, pa=pa, pb=pb, rows=rows, cols=cols,
                            a0=a0, da=da, b0=b0, db=db, flux=flux, loop_phase=loop,
                            row0_states=np.stack([S[0, j] for j in range(cols)]))
        print(f"{name}: {rows}x{cols} sum flux / 2 pi = {flux.sum() / (2 * math.pi):.3e} -> {os.path.relpath(path, ROOT)}")


def natgrad_cases():
    """(name, G, g, config) with config = (reg, threshold, adaptive, pinv, cutoff)."""
    rng = np.random.default_rng(2029)
    out = []
    z = np.load(os.path.join(ROOT, "tests", "golden", "hea_cz_n6_l3_s2.npz"))
    P = z["Q"].shape[0]
    g = z["grad"].astype(np.complex128)
    # a circuit's QGT (Hermitian, positive semi-definite) with the default config
    out.append(("circuit_qgt_default", z["Q"], g, (1e-4, 1e8, True, True, 1e-10)))
    # the same with a larger lambda and no adaptive step
    out.append(("circuit_qgt_lambda", z["Q"], g, (1e-2, 1e8, False, True, 1e-10)))
    # condition number 1e10 held exactly by ComplexFloat entries (a permuted diagonal with phases: its
    # singular values are the moduli of the entries): the adaptive lambda 1e-6 sqrt(kappa) = 0.1 takes over
    P = 24
    perm = rng.permutation(P)
    Gd = np.zeros((P, P), dtype=np.complex128)
    Gd[perm, np.arange(P)] = np.logspace(0, -10, P) * np.exp(1j * rng.uniform(0, 2 * np.pi, P))
    gh = rng.standard_normal(P) + 1j * rng.standard_normal(P)
    out.append(("permuted_diagonal_kappa1e10", Gd, gh, (1e-4, 1e8, True, True, 1e-10)))
    # the same without the permutation: the reference's LU needs no row swap, so its output is right
    Gdd = np.diag(np.logspace(0, -10, P) * np.exp(1j * rng.uniform(0, 2 * np.pi, P)))
    out.append(("diagonal_kappa1e10", Gdd, gh, (1e-4, 1e8, True, True, 1e-10)))
    # general (non-Hermitian) complex matrix, well conditioned: LU on G as given
    Gn = np.eye(P) * 3 + (rng.standard_normal((P, P)) + 1j * rng.standard_normal((P, P))) / np.sqrt(P)
    out.append(("nonhermitian", Gn, gh, (1e-4, 1e8, True, True, 1e-10)))
    # G + lambda I singular (a row and column of G equal to -lambda e_k): LU fails, the pseudo-inverse
    # of the unregularised G answers
    Gs = np.array(Gn)
    Gs[5, :] = 0
    Gs[:, 5] = 0
    Gs[5, 5] = -np.float32(1e-4)
    out.append(("singular_after_lambda", Gs, gh, (1e-4, 1e8, False, True, 1e-10)))
    # rank-deficient PSD matrix through the pseudo-inverse path with a cutoff that drops the null space
    B = rng.standard_normal((P, 16)) + 1j * rng.standard_normal((P, 16))
    Gr = B @ B.conj().T / 16
    out.append(("rank16_pinv_only", Gr, gh, None))
    return out


def natgrad_main():
    ref = O.Reference()
    arrays = {}
    for name, G, g, cfg in natgrad_cases():
        G32 = np.asarray(G, dtype=np.complex64)
        g32 = np.asarray(g, dtype=np.complex64)
        arrays[f"{name}__G"] = G32
        arrays[f"{name}__g"] = g32
        arrays[f"{name}__kappa"] = np.float64(O.condition_number_f32(G32))
        if cfg is None:
            x = O.pseudoinverse_natural_gradient(g32, G32, 1e-6)
            arrays[f"{name}__pinv_x"] = x
            print(f"{name}: pinv |x| = {np.linalg.norm(x):.4e}")
            continue
        x, lam, kappa, path = O.regularized_natural_gradient(ref, g32, G32, *cfg)
        # the reference's LU inverse solves each column with b and x in one buffer, so its row
        # permutation overwrites entries it still reads (core/matrix_operations.c:145-147, 204):
        # its inverse is wrong whenever pivoting swaps rows; record how wrong
        Mr = G32.copy()
        Mr[np.diag_indices_from(Mr)] += np.float32(lam)
        okr, invr = ref.matrix_inverse(Mr)
        arrays[f"{name}__ref_inverse_residual"] = np.float64(np.abs(invr @ Mr - np.eye(len(Mr))).max()) if okr else np.inf
        arrays[f"{name}__cfg"] = np.array([cfg[0], cfg[1], float(cfg[2]), float(cfg[3]), cfg[4]])
        arrays[f"{name}__x"] = x
        arrays[f"{name}__lambda"] = np.float64(lam)
        arrays[f"{name}__path"] = np.array(path)
        print(f"{name}: kappa {arrays[f'{name}__kappa']:.3e} lambda {lam:.3e} path {path} |x| {np.linalg.norm(x):.4e}")
    # the reference CG (compute_natural_gradient_cpu) on a rank-deficient Fisher matrix (no lambda)
    rng = np.random.default_rng(2030)
    B = rng.standard_normal((40, 12))
    F = B @ B.T / 12
    gF = B @ rng.standard_normal(12)   # in the range of F: CG converges inside it
    arrays["cg_rankdef__F"] = F
    arrays["cg_rankdef__g"] = gF
    arrays["cg_rankdef__x"] = ref.natural_gradient_cg(F, gF)
    print(f"cg_rankdef: |x| = {np.linalg.norm(arrays['cg_rankdef__x']):.4e}")
    d = os.path.join(ROOT, "tests", "golden", "natgrad")
    os.makedirs(d, exist_ok=True)
    np.savez_compressed(os.path.join(d, "natgrad_reg.npz"), **arrays)


def main():
    if sys.argv[1:] == ["berry"]:
        berry_main()
        return
    if sys.argv[1:] == ["natgrad"]:
        natgrad_main()
        return
    berry_main()
    natgrad_main()
    ref = O.Reference()
    for name, n, gates, theta in cases():
        psi = ref.simulate(n, gates, theta)
        D = ref.derivatives_shift(n, gates, theta)
        metric = ref.fubini_study(psi, D)
        F = ref.berry_curvature(psi, D)
        Q = metric - 0.5j * F
        energy = ref.tfim_energy(psi, n)
        grad = ref.param_shift_grad(n, gates, theta)
        A = metric + LAMBDA * np.eye(len(theta))
        ng = ref.natural_gradient_cg(A, grad)
        qinv = ref.invert_qfim_regularized(metric, LAMBDA)
        path = os.path.join(ROOT, "tests", "golden", f"{name}.npz")
        np.savez_compressed(path, n=n, gates=gates, theta=theta, psi=psi, Q=Q, metric=metric,
                            berry_F=F, energy=energy, grad=grad, lam=LAMBDA, natgrad_cg=ng,
                            qfim_inv=qinv)
        print(f"{name}: P={len(theta)} |Q|={np.linalg.norm(Q):.4f} E={energy:.6f} -> {os.path.relpath(path, ROOT)}")


if __name__ == "__main__":
    main()
