/*
 * ref_common.h -- shared prelude of the oracle/ref shims.
 *
 * TEST INFRASTRUCTURE ONLY.  Each shim compiles ONE source file of the
 * reference library where it lies in the read-only reference tree (the
 * Makefile passes -I<reference root>) and exports a few thin wrappers around
 * its functions, so the oracle and the golden fixtures can be checked
 * against the reference's own code.  The reference sources are included,
 * never copied; the reference's own symbols are kept hidden so that the
 * linker can drop everything the wrappers do not reach.
 */
#ifndef QGT_REF_COMMON_H
#define QGT_REF_COMMON_H
#include <complex.h>
#include <math.h>
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <float.h>
#include <unistd.h>
#define REF_EXPORT __attribute__((visibility("default")))
#endif
