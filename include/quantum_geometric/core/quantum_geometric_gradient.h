/*
 * quantum_geometric_gradient.h -- gradient / natural-gradient entry points of
 * the reference ABI, same prototypes and config struct (reference:
 * include/quantum_geometric/core/quantum_geometric_gradient.h:25-262).
 */
#ifndef QUANTUM_GEOMETRIC_GRADIENT_H
#define QUANTUM_GEOMETRIC_GRADIENT_H
#include <stdbool.h>
#include <stddef.h>
#include "quantum_geometric/core/quantum_geometric_tensor_network.h"
#ifdef __cplusplus
extern "C" {
#endif
bool compute_quantum_gradient(const quantum_geometric_tensor_network_t* qgtn, size_t param_idx,
                              ComplexFloat** gradient, size_t* dimension);
bool compute_quantum_natural_gradient(const quantum_geometric_tensor_network_t* qgtn, size_t param_idx,
                                      ComplexFloat** natural_gradient, size_t* dimension);
typedef struct {
    double shift_amount;
    bool use_centered_difference;
    bool use_higher_order;
    size_t num_points;
    bool accumulate_gradients;
    void* custom_options;
} gradient_options_t;
bool set_gradient_options(const gradient_options_t* options);
bool get_gradient_options(gradient_options_t* options);
size_t count_trainable_parameters(const quantum_geometric_tensor_network_t* qgtn);
typedef struct {
    float regularization_param;
    float condition_threshold;
    bool use_adaptive_regularization;
    bool use_pseudoinverse_fallback;
    float singular_value_cutoff;
} natural_gradient_config_t;
natural_gradient_config_t get_default_natural_gradient_config(void);
bool compute_complex_matrix_condition_number(const ComplexFloat* matrix, size_t dimension, float* condition_number);
bool compute_regularized_natural_gradient(const ComplexFloat* gradient, const ComplexFloat* metric,
                                          ComplexFloat* natural_gradient, size_t dimension,
                                          const natural_gradient_config_t* config);
bool compute_pseudoinverse_natural_gradient(const ComplexFloat* gradient, const ComplexFloat* metric,
                                            ComplexFloat* natural_gradient, size_t dimension, float singular_cutoff);
#ifdef __cplusplus
}
#endif
#endif
