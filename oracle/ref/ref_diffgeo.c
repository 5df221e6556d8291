/*
 * ref_diffgeo.c -- wrappers over the reference's FP64 QGT contraction
 * (src/quantum_geometric/distributed/differential_geometry.c:2819-2906).
 * TEST INFRASTRUCTURE ONLY.
 */
#include "ref_common.h"
#pragma GCC visibility push(hidden)
#include "src/quantum_geometric/distributed/differential_geometry.c"
#pragma GCC visibility pop

/* g_ij = Re(<d_i|d_j> - <d_i|psi><psi|d_j>); D row-major [i*dim + k]. */
REF_EXPORT int ref_fubini_study(const double* state, size_t dim, const double* D, size_t P, double* out)
{
    diffgeo_engine_t* e = diffgeo_engine_create();
    if (!e) return -1;
    bool ok = diffgeo_compute_fubini_study(e, (const ComplexDouble*)state, dim,
                                           (const ComplexDouble*)D, P, out);
    diffgeo_engine_destroy(e);
    return ok ? 0 : -1;
}

/* F_ij = -2 Im(<d_i|d_j> - <d_i|psi><psi|d_j>) (differential_geometry.c:2899). */
REF_EXPORT int ref_berry_curvature(const double* state, size_t dim, const double* D, size_t P, double* out)
{
    diffgeo_engine_t* e = diffgeo_engine_create();
    if (!e) return -1;
    bool ok = diffgeo_compute_berry_curvature(e, (const ComplexDouble*)state, dim,
                                              (const ComplexDouble*)D, P, out);
    diffgeo_engine_destroy(e);
    return ok ? 0 : -1;
}

/* diffgeo_compute_berry_phase (differential_geometry.c:2908-2945): out = {re, im}. */
REF_EXPORT int ref_berry_phase(const double* const* states, size_t n, size_t dim, double* out)
{
    diffgeo_engine_t* e = diffgeo_engine_create();
    if (!e) return -1;
    ComplexDouble r = diffgeo_compute_berry_phase(e, (const ComplexDouble**)states, n, dim);
    diffgeo_engine_destroy(e);
    out[0] = r.real;
    out[1] = r.imag;
    return 0;
}
