/*
 * classical_optimization_engine.h -- the natural-gradient solve consumed by
 * the reference's optimiser (reference: src/quantum_geometric/hybrid/
 * classical_optimization_engine.c:613-623, where the GPU variant falls back
 * to the CPU CG).  Here it is an FP64 Cholesky solve of F x = g on the GPU
 * (lambda starts at 0 and grows x10 from 1e-12 * max diag(F) when F is not
 * positive definite).
 */
#ifndef QUANTUM_GEOMETRIC_CLASSICAL_OPTIMIZATION_ENGINE_H
#define QUANTUM_GEOMETRIC_CLASSICAL_OPTIMIZATION_ENGINE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
void compute_natural_gradient_gpu(const double* fisher_matrix, const double* gradients, double* natural_gradient,
                                  size_t num_parameters);
#ifdef __cplusplus
}
#endif
#endif
