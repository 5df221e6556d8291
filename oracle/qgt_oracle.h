/*
 * qgt_oracle.h -- FP64 CPU oracle for the quantum-geometric-tensor hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA
 * product path is compared against.  Only tests/, __graft_entry__.smoke()
 * and the cpu_baseline / reference legs of bench.py may load it.  The
 * product library (libqgt_gb300.so) never links or calls it.
 *
 * Every routine restates an algorithm of the reference library
 * (tsotchke/quantum_geometric_tensor) in plain C11 + OpenMP, FP64, and cites
 * the reference file:line it follows.  Parity of this oracle is pinned by
 * the .npz fixtures under tests/golden, produced by the reference's own code
 * (the oracle/ref shims compiled against the reference sources; see
 * tests/golden/make_golden.py).
 *
 * Conventions (shared with the product ABI):
 *   - complex arrays are interleaved {re, im} doubles;
 *   - basis index bit q = qubit q (little endian), start state |0...0>
 *     (src/quantum_geometric/core/quantum_geometric_tensor_network.c:87-89);
 *   - parameter k <-> the k-th parameterised gate of the gate list, or an
 *     explicit index in og_gate_t.param (several gates may share one index);
 *   - R(theta) = exp(-i theta G / 2) with generator G in {X, Y, Z} for
 *     RX/RY/RZ (src/quantum_geometric/hybrid/quantum_classical_algorithms.c:254-264).
 */
#ifndef QGT_ORACLE_H
#define QGT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Gate type codes: the numeric values of the reference gate_type_t
 * (include/quantum_geometric/core/quantum_base_types.h:32-71). */
enum {
    OG_I = 0, OG_X = 1, OG_Y = 2, OG_Z = 3, OG_H = 4, OG_S = 5, OG_T = 6,
    OG_RX = 7, OG_RY = 8, OG_RZ = 9, OG_CNOT = 10, OG_CZ = 12, OG_SWAP = 13
};

typedef struct {
    int32_t type;    /* OG_* */
    int32_t q0;      /* 1q: target; CNOT: control; CZ/SWAP: first qubit */
    int32_t q1;      /* CNOT: target; CZ/SWAP: second qubit; else -1 */
    int32_t param;   /* parameter index for RX/RY/RZ, or -1 for a fixed angle */
    double angle;    /* fixed angle when param < 0 */
} og_gate_t;

/* Hardware-efficient ansatz: per layer RY(q0..n-1), RZ(q0..n-1), then the
 * entangler (0: CNOT ladder q->q+1, 1: CZ ring (q,q+1 mod n)).
 * Follows learning/quantum_pipeline_impl.c:2459-2529 (order RY, RZ, CNOT
 * ladder; parameters 2nl+q for RY, 2nl+n+q for RZ).  Returns #gates or -1. */
int or_build_ansatz(int n, int layers, int entangler, og_gate_t* gates, int max_gates);

/* splitmix64 stream -> uniform doubles in [0, 2*pi). */
void or_seed_params(uint64_t seed, int count, double* theta);
uint64_t or_splitmix64(uint64_t* state);

/* psi = U(theta)|0>.  psi: 2*2^n doubles. */
int or_simulate(int n, const og_gate_t* gates, int ngates, const double* theta, double* psi);

/* psi and exact derivative states D (row k = d psi / d theta_k, P x 2^n
 * complex) by generator insertion: d/dtheta R = (-i/2) G R. */
int or_derivatives(int n, const og_gate_t* gates, int ngates, const double* theta,
                   int nparams, double* psi, double* D);

/* Q_mn = <d_m psi|d_n psi> - <d_m psi|psi><psi|d_n psi>  (P x P complex).
 * Restates core/quantum_geometric_tensor_network.c:1120-1175 and
 * distributed/differential_geometry.c:2819-2906 (v = D^H psi computed once). */
int or_qgt(size_t dim, int nparams, const double* psi, const double* D, double* Q);

/* TFIM ring H = -J sum_i Z_i Z_{i+1 mod n} - h sum_i X_i (n bonds for n >= 3,
 * an open chain for n < 3).  out = H psi. */
void or_tfim_apply(int n, double J, double h, const double* psi, double* out);
double or_tfim_energy(int n, double J, double h, const double* psi);
/* H psi, H = sum_k coeffs[k] P(strings[k]) (reference Pauli-string convention) */
void or_pauli_apply(int n, int nterms, const char* const* strings, const double* coeffs, const double* psi,
                    double* out);

/* grad_k = 2 Re <d_k psi | H psi> */
void or_energy_grad(size_t dim, int nparams, const double* D, const double* Hpsi, double* grad);

/* grad_k = (E(theta + pi/2 e_k) - E(theta - pi/2 e_k)) / 2
 * (hybrid/quantum_classical_algorithms.c:580-640). */
int or_param_shift_grad(int n, const og_gate_t* gates, int ngates, const double* theta,
                        int nparams, double J, double h, double* grad);

/* x = (A + lambda I)^{-1} b by Cholesky, lambda x10 retries on failure
 * (learning/quantum_pipeline_impl.c:1601-1682, restated in double).
 * A is real symmetric P x P.  Returns 0 on success; *lambda_used = final lambda. */
int or_cholesky_solve(int P, const double* A, double lambda, const double* b, double* x,
                      double* lambda_used);

/* Unpreconditioned CG (hybrid/classical_optimization_engine.c:543-611):
 * x0 = 0, stop when ||r|| < tol or |p.Ap| < 1e-15.  Returns iterations. */
int or_cg_solve(int P, const double* A, const double* b, double* x, int max_iter, double tol);

/* PCG with M = diag(d) + U U^T (U: P x r, row-major), M^{-1} by Woodbury. */
int or_pcg_solve(int P, const double* A, const double* b, double* x, int max_iter, double tol,
                 const double* d, const double* U, int r);

/* Omega_ab(theta_a, theta_b) = Im Q_ab on a grid x grid lattice over
 * [0, 2pi)^2 (other parameters fixed), by direct re-simulation per point
 * (core/quantum_geometric_curvature.c:181-198 pointwise).  out: grid*grid,
 * row index = theta_a step. */
int or_berry_map(int n, const og_gate_t* gates, int ngates, const double* theta, int nparams,
                 int pa, int pb, int grid, double* out);

/* Berry phase of a closed loop of states, restating
 * diffgeo_compute_berry_phase (distributed/differential_geometry.c:2908-2945):
 * out = prod_i <psi_i|psi_{i+1 mod n}> / |.|, in loop order; {1, 0} for
 * n < 2 or dim 0; returns -1 (out = {0, 0}) when a link is <= 1e-14. */
int or_berry_phase(const double* const* states, size_t n, size_t dim, double* out);

/* Plaquette (Wilson-loop) flux over a rows x cols lattice of circuit states
 * at (theta_a, theta_b) = (a0 + i da, b0 + j db), restating the link
 * products of berry_curvature_kernel (src/cuda/quantum_phase_cuda.cu:245-313)
 * with full-state inner products as links: W = <p00|p10><p10|p11> x
 * <p11|p01><p01|p00>, flux = arg W (0 if |W| <= 1e-15); periodic lattices
 * wrap, otherwise the last row and column are 0. */
int or_berry_flux(int n, const og_gate_t* gates, int ngates, const double* theta, int nparams, int pa, int pb,
                  int rows, int cols, double a0, double da, double b0, double db, int periodic, double* flux);

/* One full QGT step (psi, derivative states, Gram, projector, TFIM energy
 * and gradient, FP64 Cholesky natural-gradient step) done in nslices calls of
 * or_qgt_job_step, each piece of work exactly once; the outputs (Q: P x P
 * complex, grad: P, energy: 1, natgrad: P, caller-owned) are written by the
 * last call.  The CPU baseline of the benchmark. */
typedef struct or_qgt_job or_qgt_job_t;
or_qgt_job_t* or_qgt_job_create(int n, const og_gate_t* gates, int ngates, const double* theta, int nparams,
                                int nslices, double J, double h, double lambda, double* Q, double* grad,
                                double* energy, double* natgrad);
int or_qgt_job_slices(const or_qgt_job_t* job);
int or_qgt_job_step(or_qgt_job_t* job);
void or_qgt_job_destroy(or_qgt_job_t* job);

#ifdef __cplusplus
}
#endif


#endif
