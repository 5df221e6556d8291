/*
 * qgt_states.c -- QGT from caller-supplied states on the GPU, and the
 * reference's diffgeo contraction entry points on top of it.
 *
 * The reference computes g_ij = Re(<d_i|d_j> - <d_i|psi><psi|d_j>) and
 * F_ij = -2 Im(...) with a serial triple loop that recomputes both
 * projections for every (i, j) (src/quantum_geometric/distributed/
 * differential_geometry.c:2819-2906, 3 P^2 N complex MACs).  Here the states
 * are copied to HBM once, the Gram of [psi, 0, d_0 .. d_{P-1}] runs on the
 * GPU (FP64 SIMT, or split-FP16 / split-BF16 tcgen05 from complex64-rounded
 * states) and the projector is applied in FP64.
 */
#include <math.h>
#include <stdbool.h>
#include <stdlib.h>
#include <string.h>

#include "../qgt_internal.h"
#include "qgt_gb300.h"
#include "quantum_geometric/distributed/differential_geometry.h"

#define E_INVAL (-1)
#define E_NOMEM (-2)

int qgt_qgt_from_states(const double* psi, const double* D, int64_t dim, int32_t P, qgt_precision_t prec, double* Q)
{
    if (!psi || (P > 0 && !D) || !Q || dim <= 0 || P < 0) return qgt_set_error(E_INVAL, "qgt_qgt_from_states: bad argument");
    if (prec < QGT_PRECISION_FP64 || prec > QGT_PRECISION_MIXED_BF16X3)
        return qgt_set_error(E_INVAL, "qgt_qgt_from_states: unknown precision %d", (int)prec);
    if (P == 0) return 0;
    const int rows = P + 2;
    const int fp64 = prec == QGT_PRECISION_FP64;
    void* s = NULL;
    double *X = NULL, *part = NULL, *HG = NULL, *Qd = NULL;
    void* split = NULL;
    qgt_tc_gram_t* tc = NULL;
    int32_t *pptr = NULL, *pslots = NULL, *sparam = NULL;
    int32_t* hptr = (int32_t*)malloc(sizeof(int32_t) * ((size_t)P + 1));
    int32_t* hsl = (int32_t*)malloc(sizeof(int32_t) * (size_t)P);
    if (!hptr || !hsl) { free(hptr); free(hsl); return qgt_set_error(E_NOMEM, "qgt_qgt_from_states: oom"); }
    for (int i = 0; i <= P; i++) hptr[i] = i;
    for (int i = 0; i < P; i++) hsl[i] = i;
    const size_t rowb = (size_t)dim * 16;
    int rc = qgt_dev_stream_create(&s);
    if (!rc) rc = qgt_dev_malloc((void**)&X, rowb * rows);
    if (!rc) rc = qgt_dev_memset(X, 0, rowb * rows, s);
    if (!rc) rc = qgt_dev_memcpy_h2d(X, psi, rowb, s);
    if (!rc) rc = qgt_dev_memcpy_h2d((char*)X + 2 * rowb, D, rowb * (size_t)P, s);
    if (!rc) rc = qgt_dev_malloc((void**)&HG, sizeof(double) * 2 * (size_t)rows * rows);
    if (!rc) rc = qgt_dev_malloc((void**)&Qd, sizeof(double) * 2 * (size_t)P * P);
    if (!rc) rc = qgt_dev_malloc((void**)&pptr, sizeof(int32_t) * ((size_t)P + 1));
    if (!rc) rc = qgt_dev_malloc((void**)&pslots, sizeof(int32_t) * (size_t)P);
    if (!rc) rc = qgt_dev_malloc((void**)&sparam, sizeof(int32_t) * (size_t)P);
    if (!rc) rc = qgt_dev_memcpy_h2d(pptr, hptr, sizeof(int32_t) * ((size_t)P + 1), s);
    if (!rc) rc = qgt_dev_memcpy_h2d(pslots, hsl, sizeof(int32_t) * (size_t)P, s);
    if (!rc) rc = qgt_dev_memcpy_h2d(sparam, hsl, sizeof(int32_t) * (size_t)P, s);
    if (!rc && fp64) {
        int nt = (rows + 31) / 32, ntp = nt * (nt + 1) / 2;
        int ns = 4 * 152 / ntp;
        if (ns < 1) ns = 1;
        if (ns > dim / 16) ns = (int)(dim / 16 > 0 ? dim / 16 : 1);
        rc = qgt_dev_malloc((void**)&part, sizeof(double) * 2 * 1024 * (size_t)ntp * ns);
        if (!rc) rc = qgt_dev_gram_f64(X, dim, rows, part, ns, HG, 1, 0, s);
    } else if (!rc && prec == QGT_PRECISION_MIXED) {
        /* complex64 rows (row length padded to 16 with zeros), per-row maxima, digit Gram */
        int64_t ld = (dim + 15) / 16 * 16;
        float* Y = NULL;
        uint32_t* rmax = NULL;
        qgt_dg_gram_t* dg = NULL;
        rc = qgt_dev_malloc((void**)&Y, sizeof(float) * 2 * (size_t)ld * rows);
        if (!rc) rc = qgt_dev_memset(Y, 0, sizeof(float) * 2 * (size_t)ld * rows, s);
        for (int r = 0; !rc && r < rows; r++)
            rc = qgt_dev_c128_to_c64(X + 2 * (size_t)dim * r, 2 * dim, Y + 2 * (size_t)ld * r, s);
        if (!rc) rc = qgt_dev_malloc((void**)&rmax, sizeof(uint32_t) * (size_t)rows);
        if (!rc) rc = qgt_dev_memset(rmax, 0, sizeof(uint32_t) * (size_t)rows, s);
        if (!rc) rc = qgt_dev_rowmax(Y, ld, 0, rows, rmax, s);
        if (!rc) rc = qgt_dev_dg_gram_create(Y, ld, rows, rmax, 1, rows, &dg);
        if (!rc) rc = qgt_dev_dg_gram_run(dg, HG, s);
        if (!rc) rc = qgt_dev_stream_sync(s);
        if (!rc) {
            int st = qgt_dev_dg_gram_status(dg, s);
            if (st) rc = qgt_set_error(st, "tensor-core Gram reported device status %d", st);
        }
        qgt_dev_dg_gram_destroy(dg);
        qgt_dev_free(Y);
        qgt_dev_free(rmax);
    } else if (!rc) {
        /* power-of-two prescale so that max |x| * scale <= 2^14 */
        double mx = 0;
        for (int64_t i = 0; i < 2 * dim; i++) mx = fmax(mx, fabs(psi[i]));
        for (int64_t i = 0; i < 2 * dim * (int64_t)P; i++) mx = fmax(mx, fabs(D[i]));
        int e = 0;
        if (mx > 0) { frexp(mx, &e); }
        float scale = (float)ldexp(1.0, 14 - e);
        int64_t ld = dim < 32 ? 32 : (dim + 31) / 32 * 32;
        int rows_pad = (rows + 127) / 128 * 128;
        size_t sb = (size_t)4 * rows_pad * ld * 2;
        rc = qgt_dev_malloc(&split, sb);
        if (!rc) rc = qgt_dev_memset(split, 0, sb, s);
        if (!rc) rc = qgt_dev_split_rows(X, rows, dim, split, ld, (int64_t)rows_pad * ld, 0, scale,
                                         prec == QGT_PRECISION_MIXED_BF16X3, s);
        if (!rc) rc = qgt_dev_tc_gram_create(split, ld, rows, rows_pad, prec == QGT_PRECISION_MIXED_BF16X3, &tc);
        if (!rc) rc = qgt_dev_tc_gram_run(tc, 1.0 / ((double)scale * scale), HG, s);
    }
    if (!rc) {
        qgt_dev_post_args_t pa;
        memset(&pa, 0, sizeof pa);
        pa.HG = HG;
        pa.rows = rows;
        pa.P = P;
        pa.slot_param = sparam;
        pa.param_ptr = pptr;
        pa.param_slots = pslots;
        pa.hscale = 1.0;
        pa.Q = Qd;
        rc = qgt_dev_post(&pa, s);
    }
    if (!rc) rc = qgt_dev_memcpy_d2h(Q, Qd, sizeof(double) * 2 * (size_t)P * P, s);
    if (!rc) rc = qgt_dev_stream_sync(s);
    if (!rc && tc) {
        int st = qgt_dev_tc_gram_status(tc, s);
        if (st) rc = qgt_set_error(st, "tensor-core Gram reported device status %d", st);
    }
    qgt_dev_tc_gram_destroy(tc);
    qgt_dev_free(X); qgt_dev_free(part); qgt_dev_free(HG); qgt_dev_free(Qd); qgt_dev_free(split);
    qgt_dev_free(pptr); qgt_dev_free(pslots); qgt_dev_free(sparam);
    if (s) qgt_dev_stream_destroy(s);
    free(hptr);
    free(hsl);
    return rc;
}

/* ---- reference diffgeo entry points ---- */

struct diffgeo_engine {
    int precision;
    size_t metric_evaluations, curvature_evaluations, berry_phase_evaluations;
};

diffgeo_engine_t* diffgeo_engine_create(void)
{
    diffgeo_engine_t* e = (diffgeo_engine_t*)calloc(1, sizeof(diffgeo_engine_t));
    if (e) e->precision = QGT_PRECISION_FP64;
    return e;
}

void diffgeo_engine_destroy(diffgeo_engine_t* e) { free(e); }

static bool diffgeo_q(diffgeo_engine_t* e, const ComplexDouble* state, size_t dim, const ComplexDouble* d, size_t P,
                      double** Qout)
{
    if (!e || !state || !d || dim == 0 || P == 0 || P > 0x7fffffff) return false;
    double* Q = (double*)malloc(sizeof(double) * 2 * P * P);
    if (!Q) return false;
    if (qgt_qgt_from_states((const double*)state, (const double*)d, (int64_t)dim, (int32_t)P,
                            (qgt_precision_t)e->precision, Q) != 0) {
        free(Q);
        return false;
    }
    *Qout = Q;
    return true;
}

bool diffgeo_compute_fubini_study(diffgeo_engine_t* e, const ComplexDouble* state, size_t dim,
                                  const ComplexDouble* d, size_t P, double* metric_out)
{
    double* Q = NULL;
    if (!metric_out || !diffgeo_q(e, state, dim, d, P, &Q)) return false;
    for (size_t i = 0; i < P * P; i++) metric_out[i] = Q[2 * i];
    free(Q);
    e->metric_evaluations++;
    return true;
}

bool diffgeo_compute_berry_curvature(diffgeo_engine_t* e, const ComplexDouble* state, size_t dim,
                                     const ComplexDouble* d, size_t P, double* curvature_out)
{
    double* Q = NULL;
    if (!curvature_out || !diffgeo_q(e, state, dim, d, P, &Q)) return false;
    for (size_t i = 0; i < P * P; i++) curvature_out[i] = -2.0 * Q[2 * i + 1];
    free(Q);
    e->curvature_evaluations++;
    return true;
}

/* Berry phase of a closed loop of states (reference:
 * src/quantum_geometric/distributed/differential_geometry.c:2908-2945): the
 * product over i of <psi_i|psi_{i+1 mod n}> / |<psi_i|psi_{i+1 mod n}>|,
 * multiplied in loop order.  The n overlaps run as one GPU kernel over the
 * states copied to HBM; {0, 0} when a link magnitude is <= 1e-14 (orthogonal
 * neighbours, phase undefined) or the GPU fails (the last error says which). */
ComplexDouble diffgeo_compute_berry_phase(diffgeo_engine_t* e, const ComplexDouble** states, size_t num_states,
                                          size_t dim)
{
    ComplexDouble res = {1.0, 0.0};
    if (!e || !states || num_states < 2 || dim == 0) return res;
    const ComplexDouble zero = {0.0, 0.0};
    for (size_t i = 0; i < num_states; i++)
        if (!states[i]) { qgt_set_error(E_INVAL, "diffgeo_compute_berry_phase: state %zu is NULL", i); return zero; }
    if (num_states > 0x7fffffff || dim > ((size_t)1 << 40)) {
        qgt_set_error(E_INVAL, "diffgeo_compute_berry_phase: %zu states of %zu amplitudes too large", num_states, dim);
        return zero;
    }
    const int32_t n = (int32_t)num_states;
    const int32_t nch = qgt_overlap_chunks((int64_t)dim, n);
    void* s = NULL;
    double *X = NULL, *part = NULL;
    int64_t* off_d = NULL;
    int64_t* off = (int64_t*)malloc(sizeof(int64_t) * 2 * (size_t)n);
    double* part_h = (double*)malloc(sizeof(double) * 2 * (size_t)n * (size_t)nch);
    int rc = (!off || !part_h) ? qgt_set_error(E_NOMEM, "diffgeo_compute_berry_phase: out of memory") : 0;
    for (int32_t i = 0; !rc && i < n; i++) {
        off[i] = (int64_t)i * (int64_t)dim;
        off[n + i] = (int64_t)((i + 1) % n) * (int64_t)dim;
    }
    if (!rc) rc = qgt_dev_stream_create(&s);
    if (!rc) rc = qgt_dev_malloc((void**)&X, sizeof(ComplexDouble) * dim * num_states);
    for (size_t i = 0; !rc && i < num_states; i++)
        rc = qgt_dev_memcpy_h2d(X + 2 * dim * i, states[i], sizeof(ComplexDouble) * dim, s);
    if (!rc) rc = qgt_dev_malloc((void**)&off_d, sizeof(int64_t) * 2 * (size_t)n);
    if (!rc) rc = qgt_dev_malloc((void**)&part, sizeof(double) * 2 * (size_t)n * (size_t)nch);
    if (!rc) rc = qgt_dev_memcpy_h2d(off_d, off, sizeof(int64_t) * 2 * (size_t)n, s);
    if (!rc) rc = qgt_dev_overlaps(X, 1, (int64_t)dim, off_d, off_d + n, n, nch, part, s);
    if (!rc) rc = qgt_dev_memcpy_d2h(part_h, part, sizeof(double) * 2 * (size_t)n * (size_t)nch, s);
    if (!rc) rc = qgt_dev_stream_sync(s);
    for (int32_t i = 0; !rc && i < n; i++) {
        double re = 0, im = 0;
        for (int32_t q = 0; q < nch; q++) {
            re += part_h[2 * ((size_t)i * nch + q)];
            im += part_h[2 * ((size_t)i * nch + q) + 1];
        }
        const double mag = sqrt(re * re + im * im);
        if (!(mag > 1e-14)) {
            rc = qgt_set_error(E_INVAL, "diffgeo_compute_berry_phase: states %d and %d are orthogonal", i, (i + 1) % n);
            break;
        }
        re /= mag;
        im /= mag;
        const double r = res.real * re - res.imag * im;
        res.imag = res.real * im + res.imag * re;
        res.real = r;
    }
    qgt_dev_free(X);
    qgt_dev_free(part);
    qgt_dev_free(off_d);
    if (s) qgt_dev_stream_destroy(s);
    free(off);
    free(part_h);
    if (rc) return zero;
    e->berry_phase_evaluations++;
    return res;
}
