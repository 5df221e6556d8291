/*
 * quantum_geometric_types.h -- tensor / metric / curvature types of the
 * reference ABI on this path (reference: include/quantum_geometric/core/
 * quantum_geometric_types.h:239-250, 285-298, 331-353, 378-458; same field
 * order and enumerator values).
 */
#ifndef QUANTUM_GEOMETRIC_TYPES_H
#define QUANTUM_GEOMETRIC_TYPES_H
#include <stdbool.h>
#include <stddef.h>
#include "quantum_geometric/core/error_codes.h"
#include "quantum_geometric/core/quantum_types.h"

typedef enum {
    GEOMETRIC_TENSOR_SCALAR, GEOMETRIC_TENSOR_VECTOR, GEOMETRIC_TENSOR_COVECTOR,
    GEOMETRIC_TENSOR_BIVECTOR, GEOMETRIC_TENSOR_TRIVECTOR, GEOMETRIC_TENSOR_UNITARY,
    GEOMETRIC_TENSOR_HERMITIAN, GEOMETRIC_TENSOR_SYMMETRIC, GEOMETRIC_TENSOR_CUSTOM
} geometric_tensor_type_t;

typedef enum {
    QGT_MEM_STANDARD = 0, QGT_MEM_HUGE_PAGES, QGT_MEM_PINNED, QGT_MEM_UNIFIED
} qgt_memory_type_t;

typedef enum {
    GEOMETRIC_METRIC_EUCLIDEAN, GEOMETRIC_METRIC_MINKOWSKI, GEOMETRIC_METRIC_FUBINI_STUDY,
    GEOMETRIC_METRIC_KAHLER, GEOMETRIC_METRIC_CUSTOM
} geometric_metric_type_t;

typedef enum {
    GEOMETRIC_CURVATURE_RIEMANN, GEOMETRIC_CURVATURE_RICCI, GEOMETRIC_CURVATURE_SCALAR,
    GEOMETRIC_CURVATURE_WEYL, GEOMETRIC_CURVATURE_BERRY, GEOMETRIC_CURVATURE_CUSTOM
} geometric_curvature_type_t;

typedef struct quantum_geometric_tensor_t quantum_geometric_tensor_t;
typedef struct quantum_geometric_metric_t quantum_geometric_metric_t;
typedef struct quantum_geometric_curvature_t quantum_geometric_curvature_t;

struct quantum_geometric_tensor_t {
    geometric_tensor_type_t type;
    size_t* dimensions;
    size_t rank;
    size_t dimension;
    ComplexFloat* components;
    size_t num_spins;
    void* auxiliary_data;
    bool is_symmetric;
    bool is_unitary;
    bool is_hermitian;
    HardwareType hardware;
    qgt_memory_type_t mem_type;
    size_t total_elements;
    size_t aligned_elements;
};

struct quantum_geometric_metric_t {
    geometric_metric_type_t type;
    size_t dimension;
    ComplexFloat* components;
    bool is_symmetric;
    void* auxiliary_data;
    HardwareType hardware;
};

struct quantum_geometric_curvature_t {
    geometric_curvature_type_t type;
    size_t dimension;
    ComplexFloat* components;
    void* auxiliary_data;
    bool is_flat;
    HardwareType hardware;
};

/* The reference caps metric/curvature dimensions at 16 (QGT_MAX_DIMENSIONS,
 * quantum_geometric_types.h:97), which rejects every circuit with more than
 * 16 parameters; this library lifts the cap to QGT_MAX_PARAMETERS. */
#define QGT_MAX_PARAMETERS 65536
#endif
