/*
 * classical_optimization_engine.h -- the natural-gradient solve consumed by
 * the reference's optimiser (reference: src/quantum_geometric/hybrid/
 * classical_optimization_engine.c:613-623, where the GPU variant falls back
 * to the CPU CG of :543-611).  Here the same conjugate-gradient iteration
 * (x0 = 0, at most 100 steps, stop at |p^T F p| < 1e-15 or |r| < 1e-8) runs
 * on the GPU in FP64.
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
