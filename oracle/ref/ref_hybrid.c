/*
 * ref_hybrid.c -- wrappers over the reference's FP64 state-vector simulator
 * and Pauli-string expectation (src/quantum_geometric/hybrid/
 * quantum_classical_algorithms.c:174-382).  TEST INFRASTRUCTURE ONLY.
 */
#include "ref_common.h"
#pragma GCC visibility push(hidden)
#include "src/quantum_geometric/hybrid/quantum_classical_algorithms.c"
#pragma GCC visibility pop

/* Build a reference quantum_circuit_t from a flat gate list and run
 * execute_circuit_on_statevector (quantum_classical_algorithms.c:278-318) on
 * |0...0>.  types use the reference gate_type_t values; for CNOT/CZ q0 is the
 * control and q1 the target; angles[g] is the gate angle.  sv: 2*2^n doubles. */
REF_EXPORT int ref_simulate(int n, const int* types, const int* q0, const int* q1,
                            const double* angles, int ngates, double* sv)
{
    size_t dim = (size_t)1 << n;
    quantum_gate_t* gs = calloc((size_t)ngates + 1, sizeof(quantum_gate_t));
    quantum_gate_t** gp = calloc((size_t)ngates + 1, sizeof(quantum_gate_t*));
    size_t* tq = calloc((size_t)ngates + 1, sizeof(size_t));
    size_t* cq = calloc((size_t)ngates + 1, sizeof(size_t));
    double* pa = calloc((size_t)ngates + 1, sizeof(double));
    if (!gs || !gp || !tq || !cq || !pa) return -1;
    for (int g = 0; g < ngates; g++) {
        quantum_gate_t* G = &gs[g];
        G->type = (gate_type_t)types[g];
        pa[g] = angles[g];
        G->parameters = &pa[g];
        G->num_parameters = 1;
        if (types[g] == GATE_TYPE_CNOT || types[g] == GATE_TYPE_CZ) {
            cq[g] = (size_t)q0[g];
            tq[g] = (size_t)q1[g];
            G->control_qubits = &cq[g];
            G->target_qubits = &tq[g];
            G->num_controls = 1;
            G->num_qubits = 2;
        } else {
            tq[g] = (size_t)q0[g];
            G->target_qubits = &tq[g];
            G->num_qubits = 1;
        }
        gp[g] = G;
    }
    quantum_circuit_t c;
    memset(&c, 0, sizeof c);
    c.num_qubits = (size_t)n;
    c.gates = gp;
    c.num_gates = (size_t)ngates;
    double complex* v = (double complex*)sv;
    memset(v, 0, dim * sizeof(double complex));
    v[0] = 1.0;
    bool ok = execute_circuit_on_statevector(&c, v);
    free(gs); free(gp); free(tq); free(cq); free(pa);
    return ok ? 0 : -1;
}

/* compute_pauli_expectation (quantum_classical_algorithms.c:320-382):
 * character [n-1-q] of the string acts on qubit q. */
REF_EXPORT double ref_pauli_expectation(const double* sv, int n, const char* pauli)
{
    return compute_pauli_expectation((const double complex*)sv, (size_t)n, pauli);
}
