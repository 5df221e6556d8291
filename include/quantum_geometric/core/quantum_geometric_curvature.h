/*
 * quantum_geometric_curvature.h -- Berry curvature and full-QGT entry points
 * of the reference ABI, same prototypes (reference: include/quantum_geometric/
 * core/quantum_geometric_curvature.h:15-103).  Convention of the core API:
 * Omega = +Im Q, stored in .real, antisymmetric, zero diagonal
 * (src/quantum_geometric/core/quantum_geometric_curvature.c:222-243).
 */
#ifndef QUANTUM_GEOMETRIC_CURVATURE_H
#define QUANTUM_GEOMETRIC_CURVATURE_H
#include "quantum_geometric/core/quantum_geometric_types.h"
#include "quantum_geometric/core/quantum_geometric_tensor_network.h"
#ifdef __cplusplus
extern "C" {
#endif
qgt_error_t geometric_create_curvature(quantum_geometric_curvature_t** curvature, geometric_curvature_type_t type,
                                       size_t dimension);
void geometric_destroy_curvature(quantum_geometric_curvature_t* curvature);
qgt_error_t geometric_clone_curvature(quantum_geometric_curvature_t** dest,
                                      const quantum_geometric_curvature_t* src);
qgt_error_t geometric_compute_berry_curvature(quantum_geometric_curvature_t* curvature,
                                              const quantum_geometric_tensor_network_t* qgtn, size_t num_params);
qgt_error_t geometric_compute_berry_curvature_element(const quantum_geometric_tensor_network_t* qgtn,
                                                      size_t param_mu, size_t param_nu, float* result);
qgt_error_t geometric_compose_qgt(ComplexFloat* qgt, const quantum_geometric_metric_t* metric,
                                  const quantum_geometric_curvature_t* curvature, size_t dimension);
qgt_error_t geometric_compute_full_qgt(ComplexFloat* qgt, const quantum_geometric_tensor_network_t* qgtn,
                                       size_t num_params);
#ifdef __cplusplus
}
#endif
#endif
