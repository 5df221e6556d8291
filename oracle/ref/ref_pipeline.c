/*
 * ref_pipeline.c -- wrapper over the reference's float Tikhonov + Cholesky
 * QFIM inverse invert_qfim_regularized (src/quantum_geometric/learning/
 * quantum_pipeline_impl.c:1601-1682).  TEST INFRASTRUCTURE ONLY.
 */
#include "ref_common.h"
#pragma GCC visibility push(hidden)
#include "src/quantum_geometric/learning/quantum_pipeline_impl.c"
#pragma GCC visibility pop

REF_EXPORT int ref_invert_qfim_regularized(const float* qfim, float* inv, size_t n, float lambda)
{
    return invert_qfim_regularized(qfim, inv, n, lambda);
}
