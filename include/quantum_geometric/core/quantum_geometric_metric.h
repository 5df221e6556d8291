/*
 * quantum_geometric_metric.h -- Fubini-Study metric entry points of the
 * reference ABI, same prototypes (reference: include/quantum_geometric/core/
 * quantum_geometric_metric.h:13-68).
 * Deviation: dimensions up to QGT_MAX_PARAMETERS (the reference caps at 16).
 */
#ifndef QUANTUM_GEOMETRIC_METRIC_H
#define QUANTUM_GEOMETRIC_METRIC_H
#include "quantum_geometric/core/quantum_geometric_types.h"
#include "quantum_geometric/core/quantum_geometric_tensor_network.h"
#ifdef __cplusplus
extern "C" {
#endif
qgt_error_t geometric_create_metric(quantum_geometric_metric_t** metric, geometric_metric_type_t type,
                                    size_t dimension);
void geometric_destroy_metric(quantum_geometric_metric_t* metric);
/* the state-space metric of a state: Euclidean unchanged, Fubini-Study
 * delta_ij - conj(psi_i) psi_j (dimension = the state's dimension) */
qgt_error_t geometric_compute_metric(quantum_geometric_metric_t* metric, const quantum_state_t* state);
qgt_error_t geometric_clone_metric(quantum_geometric_metric_t** dest, const quantum_geometric_metric_t* src);
qgt_error_t geometric_compute_fubini_study_metric(quantum_geometric_metric_t* metric,
                                                  const quantum_geometric_tensor_network_t* qgtn,
                                                  size_t num_params);
qgt_error_t geometric_compute_fubini_study_element(const quantum_geometric_tensor_network_t* qgtn,
                                                   size_t param_mu, size_t param_nu, float* result);
#ifdef __cplusplus
}
#endif
#endif
