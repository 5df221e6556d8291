/*
 * differential_geometry.h -- the reference's FP64 QGT contraction and loop
 * Berry phase from given states, same prototypes (reference:
 * include/quantum_geometric/distributed/differential_geometry.h:573-599;
 * src/quantum_geometric/distributed/differential_geometry.c:2819-2945),
 * computed on the GPU.
 * Normalisations: metric_out = Re Q; curvature_out = -2 Im Q.
 * diffgeo_compute_berry_phase returns prod_i <psi_i|psi_{i+1 mod n}> / |...|
 * (a unit complex number whose argument is the phase); {1, 0} for NULL
 * arguments, fewer than 2 states or dim 0; {0, 0} when a link has magnitude
 * <= 1e-14 or the GPU reports an error.
 */
#ifndef QUANTUM_GEOMETRIC_DIFFERENTIAL_GEOMETRY_H
#define QUANTUM_GEOMETRIC_DIFFERENTIAL_GEOMETRY_H
#include <stdbool.h>
#include <stddef.h>
#include "quantum_geometric/core/quantum_complex.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct diffgeo_engine diffgeo_engine_t;
diffgeo_engine_t* diffgeo_engine_create(void);
void diffgeo_engine_destroy(diffgeo_engine_t* engine);
bool diffgeo_compute_fubini_study(diffgeo_engine_t* engine, const ComplexDouble* state, size_t dim,
                                  const ComplexDouble* param_derivatives, size_t num_params, double* metric_out);
bool diffgeo_compute_berry_curvature(diffgeo_engine_t* engine, const ComplexDouble* state, size_t dim,
                                     const ComplexDouble* param_derivatives, size_t num_params,
                                     double* curvature_out);
ComplexDouble diffgeo_compute_berry_phase(diffgeo_engine_t* engine, const ComplexDouble** states, size_t num_states,
                                          size_t dim);
#ifdef __cplusplus
}
#endif
#endif
