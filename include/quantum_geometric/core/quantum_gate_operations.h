/*
 * quantum_gate_operations.h -- gate constructors of the reference ABI, same
 * prototypes (reference: include/quantum_geometric/core/quantum_gate_operations.h:22-138).
 * Matrices follow src/quantum_geometric/core/quantum_gate_operations.c:10-127.
 */
#ifndef QUANTUM_GATE_OPERATIONS_H
#define QUANTUM_GATE_OPERATIONS_H
#include <stdbool.h>
#include <stddef.h>
#include "quantum_geometric/core/quantum_types.h"
#ifdef __cplusplus
extern "C" {
#endif
quantum_gate_t* create_quantum_gate(gate_type_t type, const size_t* qubits, size_t num_qubits,
                                    const double* parameters, size_t num_parameters);
quantum_gate_t* copy_quantum_gate(const quantum_gate_t* gate);
void destroy_quantum_gate(quantum_gate_t* gate);
bool update_gate_parameters(quantum_gate_t* gate, const double* parameters, size_t num_parameters);
bool shift_gate_parameters(quantum_gate_t* gate, size_t param_idx, double shift_amount);
quantum_gate_t* create_rx_gate(size_t qubit, double angle);
quantum_gate_t* create_ry_gate(size_t qubit, double angle);
quantum_gate_t* create_rz_gate(size_t qubit, double angle);
quantum_gate_t* create_h_gate(size_t qubit);
quantum_gate_t* create_x_gate(size_t qubit);
quantum_gate_t* create_y_gate(size_t qubit);
quantum_gate_t* create_z_gate(size_t qubit);
quantum_gate_t* create_cnot_gate(size_t control, size_t target);
quantum_gate_t* create_cz_gate(size_t control, size_t target);
#ifdef __cplusplus
}
#endif
#endif
