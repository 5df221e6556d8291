/*
 * quantum_geometric_tensor.h -- tensor lifecycle of the reference ABI on this
 * path, same prototypes (reference: include/quantum_geometric/core/
 * quantum_geometric_tensor.h:13-27; behaviour of src/quantum_geometric/core/
 * quantum_geometric_tensor.c:158-340 and quantum_geometric_tensor_cpu.c:837-863:
 * zeroed ComplexFloat components, 8-element aligned storage, unit-modulus
 * random fills, identity for square rank-2 tensors).
 */
#ifndef QUANTUM_GEOMETRIC_TENSOR_H
#define QUANTUM_GEOMETRIC_TENSOR_H
#include <stdbool.h>
#include <stddef.h>
#include "quantum_geometric/core/quantum_geometric_types.h"
#ifdef __cplusplus
extern "C" {
#endif
qgt_error_t geometric_tensor_create(quantum_geometric_tensor_t** tensor, geometric_tensor_type_t type,
                                    const size_t* dimensions, size_t rank);
void geometric_tensor_destroy(quantum_geometric_tensor_t* tensor);
qgt_error_t geometric_tensor_clone(quantum_geometric_tensor_t** dest, const quantum_geometric_tensor_t* src);
qgt_error_t geometric_tensor_initialize(quantum_geometric_tensor_t* tensor, const ComplexFloat* data);
qgt_error_t geometric_tensor_initialize_zero(quantum_geometric_tensor_t* tensor);
qgt_error_t geometric_tensor_initialize_random(quantum_geometric_tensor_t* tensor, float min_val, float max_val);
qgt_error_t geometric_tensor_initialize_identity(quantum_geometric_tensor_t* tensor);
#ifdef __cplusplus
}
#endif
#endif
