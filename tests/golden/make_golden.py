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

Only the circuits and seeded angles are chosen here.  Run from the repository
root in a container that has the reference tree:
    make -C oracle && python tests/golden/make_golden.py          (all fixtures)
  make -C oracle && python tests/golden/make_golden.py berry    (Berry-phase fixtures only)
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


def main():
    if sys.argv[1:] == ["berry"]:
        berry_main()
        return
    berry_main()
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
