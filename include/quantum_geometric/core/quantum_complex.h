/*
 * quantum_complex.h -- complex scalar types of the reference ABI
 * (reference: include/quantum_geometric/core/quantum_complex.h:13-23).
 * Same layout: {real, imag} pairs of float / double.
 */
#ifndef QUANTUM_COMPLEX_H
#define QUANTUM_COMPLEX_H
#ifndef COMPLEX_FLOAT_DEFINED
#define COMPLEX_FLOAT_DEFINED
typedef struct {
    float real;
    float imag;
} ComplexFloat;
typedef struct {
    double real;
    double imag;
} ComplexDouble;
#endif
#endif
