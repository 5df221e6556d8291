/*
 * quantum_geometric_tensor_network.h -- the reference QGTN circuit object and
 * its QGT entry points, same prototypes (reference:
 * include/quantum_geometric/core/quantum_geometric_tensor_network.h:46-151).
 *
 * In this library the object records its gates layer by layer exactly as
 * the reference does (apply_quantum_gate appends to the last layer,
 * src/quantum_geometric/core/quantum_geometric_tensor_network.c:652), and
 * every QGT query is answered from one GPU step over the whole circuit
 * (cached per parameter values) instead of a per-element network
 * contraction.  `network` is always NULL; `backend_state` holds the plan.
 */
#ifndef QUANTUM_GEOMETRIC_TENSOR_NETWORK_H
#define QUANTUM_GEOMETRIC_TENSOR_NETWORK_H
#include <stdbool.h>
#include <stddef.h>
#include "quantum_geometric/core/quantum_geometric_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tensor_network_t tensor_network_t;

typedef enum {
    QGTN_BACKEND_SIMULATOR, QGTN_BACKEND_IBM, QGTN_BACKEND_RIGETTI, QGTN_BACKEND_DWAVE,
    QGTN_BACKEND_IONQ, QGTN_BACKEND_XANADU, QGTN_BACKEND_CUSTOM
} qgtn_backend_type_t;

typedef struct {
    qgtn_backend_type_t type;
    void* backend_specific;
    bool supports_gradients;
    bool supports_hybrid;
} qgtn_hardware_config_t;

typedef struct quantum_geometric_tensor_network {
    tensor_network_t* network;
    quantum_circuit_t* circuit;
    size_t num_qubits;
    size_t num_layers;
    bool is_distributed;
    bool use_hardware_acceleration;
    qgtn_hardware_config_t hardware_config;
    void* backend_state;
} quantum_geometric_tensor_network_t;

quantum_geometric_tensor_network_t* create_quantum_geometric_tensor_network(
    size_t num_qubits, size_t num_layers, bool is_distributed, bool use_hardware_acceleration);
void destroy_quantum_geometric_tensor_network(quantum_geometric_tensor_network_t* qgtn);
quantum_geometric_tensor_network_t* copy_quantum_geometric_tensor_network(
    const quantum_geometric_tensor_network_t* qgtn);
quantum_gate_t* copy_quantum_gate(const quantum_gate_t* gate);
bool apply_quantum_gate(quantum_geometric_tensor_network_t* qgtn, const quantum_gate_t* gate,
                        const size_t* qubits, size_t num_qubits);
bool apply_quantum_circuit(quantum_geometric_tensor_network_t* qgtn, const quantum_circuit_t* circuit);
bool qgtn_measure_qubit(const quantum_geometric_tensor_network_t* qgtn, size_t qubit,
                        double* probability_zero, double* probability_one);
bool get_quantum_state(const quantum_geometric_tensor_network_t* qgtn, ComplexFloat** state_vector,
                       size_t* dimension);
bool compute_quantum_geometric_tensor(const quantum_geometric_tensor_network_t* qgtn, size_t param_i,
                                      size_t param_j, ComplexFloat* result);
bool compute_quantum_metric(const quantum_geometric_tensor_network_t* qgtn, size_t param_i, size_t param_j,
                            double* result);
bool compute_berry_curvature(const quantum_geometric_tensor_network_t* qgtn, size_t param_i, size_t param_j,
                             double* result);
bool distribute_computation(quantum_geometric_tensor_network_t* qgtn, const size_t* device_ids,
                            size_t num_devices);
bool synchronize_distributed_state(quantum_geometric_tensor_network_t* qgtn);
bool enable_hardware_acceleration(quantum_geometric_tensor_network_t* qgtn, HardwareType type);
bool disable_hardware_acceleration(quantum_geometric_tensor_network_t* qgtn);
const char* get_quantum_geometric_tensor_network_error(void);

/* Extension (no reference counterpart): precision of the GPU step behind the
 * QGTN queries; 0 = FP64 (default), 1 = mixed (complex64 evolution, exact
 * integer-digit FP16 tensor-core Gram), 2 = mixed BF16x3. Networks of fewer
 * than 4 qubits run FP64 when 1 is selected. */
bool qgtn_set_precision(quantum_geometric_tensor_network_t* qgtn, int precision);

#ifdef __cplusplus
}
#endif
#endif
