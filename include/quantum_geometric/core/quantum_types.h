/*
 * quantum_types.h -- gate, circuit and state structs of the reference ABI,
 * same field order (reference: include/quantum_geometric/core/quantum_types.h:
 * 170-190 quantum_gate_t, 195-232 quantum_state_t, 238-274 circuit_layer_t /
 * quantum_circuit_t).  Types this path never dereferences are kept opaque.
 */
#ifndef QUANTUM_TYPES_H
#define QUANTUM_TYPES_H
#include <stdbool.h>
#include <stddef.h>
#include "quantum_geometric/core/quantum_base_types.h"

typedef struct computational_graph_t computational_graph_t;
typedef struct quantum_geometric_state_t quantum_geometric_state_t;
typedef struct quantum_compute_node_t quantum_compute_node_t;
typedef struct quantum_gate_t quantum_gate_t;
typedef struct quantum_circuit_t quantum_circuit_t;

struct quantum_gate_t {
    gate_type_t type;
    size_t num_qubits;
    bool is_controlled;
    bool is_parameterized;
    size_t* target_qubits;
    size_t* control_qubits;
    size_t num_controls;
    size_t* qubits;
    double* parameters;
    size_t num_parameters;
    ComplexFloat* matrix;
    void* custom_data;
};

typedef struct quantum_state_t quantum_state_t;
typedef struct StabilizerMeasurement StabilizerMeasurement;
typedef struct TopologicalAnyon TopologicalAnyon;

/* geometric_compute_metric reads dimension and coordinates; the other fields
 * keep the reference layout */
struct quantum_state_t {
    quantum_state_type_t type;
    size_t num_qubits;
    size_t dimension;
    size_t manifold_dim;
    ComplexFloat* coordinates;
    ComplexFloat* metric;
    ComplexFloat* connection;
    void* auxiliary_data;
    bool is_normalized;
    HardwareType hardware;
    size_t lattice_width;
    size_t lattice_height;
    size_t num_stabilizers;
    size_t num_plaquettes;
    size_t num_vertices;
    StabilizerMeasurement* stabilizers;
    size_t num_anyons;
    size_t max_anyons;
    TopologicalAnyon* anyons;
    double* syndrome_values;
    size_t syndrome_size;
    double* measurement_confidence;
    size_t confidence_size;
};

typedef struct circuit_layer_t {
    quantum_gate_t** gates;
    size_t num_gates;
    bool is_parameterized;
} circuit_layer_t;

struct quantum_circuit_t {
    size_t num_qubits;
    bool is_parameterized;
    circuit_layer_t** layers;
    size_t num_layers;
    size_t layers_capacity;
    quantum_gate_t** gates;
    size_t num_gates;
    size_t max_gates;
    int optimization_level;
    bool is_compiled;
    computational_graph_t* graph;
    quantum_geometric_state_t* state;
    quantum_compute_node_t** nodes;
    size_t num_nodes;
    size_t capacity;
};
#endif
