/*
 * ref_optim.c -- wrapper over the reference's FP64 CG natural-gradient solve
 * compute_natural_gradient_cpu (src/quantum_geometric/hybrid/
 * classical_optimization_engine.c:543-611).  TEST INFRASTRUCTURE ONLY.
 */
#include "ref_common.h"
#pragma GCC visibility push(hidden)
#include "src/quantum_geometric/hybrid/classical_optimization_engine.c"
#pragma GCC visibility pop

REF_EXPORT void ref_natural_gradient_cg(const double* F, const double* g, double* x, size_t P)
{
    compute_natural_gradient_cpu(F, g, x, P);
}
