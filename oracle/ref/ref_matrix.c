/*
 * ref_matrix.c -- wrappers over the reference's complex LU inverse and solve
 * (src/quantum_geometric/core/matrix_operations.c:55-217), the dense algebra
 * behind compute_regularized_natural_gradient
 * (src/quantum_geometric/core/quantum_geometric_gradient.c:2887-2964).
 * TEST INFRASTRUCTURE ONLY.
 */
#include "ref_common.h"
#pragma GCC visibility push(hidden)
#include "src/quantum_geometric/core/matrix_operations.c"
#pragma GCC visibility pop

/* inv = a^-1 for an n x n ComplexFloat matrix ({re, im} floats); 1 on success, 0 when singular */
REF_EXPORT int ref_matrix_inverse(const float* a, float* inv, size_t n)
{
    return matrix_inverse((const ComplexFloat*)a, (ComplexFloat*)inv, n) ? 1 : 0;
}

/* a x = b; 1 on success, 0 when singular */
REF_EXPORT int ref_solve_linear_system(const float* a, const float* b, float* x, size_t n)
{
    return solve_linear_system((const ComplexFloat*)a, (const ComplexFloat*)b, (ComplexFloat*)x, n) ? 1 : 0;
}
