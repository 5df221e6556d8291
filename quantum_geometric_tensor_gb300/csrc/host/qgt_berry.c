/*
 * qgt_berry.c -- Berry phases of closed loops of states: the plaquette
 * (Wilson-loop) flux over a two-parameter lattice of circuit states.
 *
 * The reference's berry_curvature_kernel (src/cuda/quantum_phase_cuda.cu:
 * 245-313) takes one complex value per lattice site and forms, per plaquette,
 * W = U_01 U_12 U_23 U_30 with U_ij = conj(psi_i) psi_j and flux = arg W.  The
 * loop phase diffgeo_compute_berry_phase (src/quantum_geometric/distributed/
 * differential_geometry.c:2908-2945) multiplies the unit-normalised overlaps
 * <psi_i|psi_{i+1}> of full states around a loop.  Here the sites are full
 * circuit states: a theta-batched plan (forward transport, no Hamiltonian,
 * one derivative parameter, which the flux does not read) evolves a block of
 * lattice rows in one step, the 2 (R + 1) cols link overlaps of the block run
 * as one GPU kernel over the plan's vector buffer, and the host multiplies
 * the four links of each plaquette in the reference kernel's order.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../qgt_internal.h"
#include "qgt_gb300.h"

#define E_INVAL (-1)
#define E_NOMEM (-2)

/* device memory a block of lattice rows may hold in its plan */
#define FLUX_BLOCK_BYTES (48.0 * 1024 * 1024 * 1024)

int32_t qgt_overlap_chunks(int64_t N, int32_t n)
{
    /* about 4 CTAs per SM of 152 in total, each summing >= 4096 amplitudes */
    int64_t want = (4 * 152 + n - 1) / (n > 0 ? n : 1);
    int64_t most = N / 4096;
    if (want > most) want = most;
    if (want < 1) want = 1;
    if ((int64_t)n * want > 0x7fffffff) want = 1;
    return (int32_t)want;
}

void qgt_flux_default_options(qgt_flux_options_t* o)
{
    if (!o) return;
    memset(o, 0, sizeof *o);
    o->param_a = 0;
    o->param_b = 1;
    o->rows = o->cols = 32;
    o->a0 = o->b0 = 0.0;
    o->da = o->db = 2.0 * M_PI / 32;
    o->periodic = 1;
    o->precision = QGT_PRECISION_MIXED;
    o->device = 0;
}

static inline void cmul(double ar, double ai, double br, double bi, double* r, double* i)
{
    *r = ar * br - ai * bi;
    *i = ar * bi + ai * br;
}

int qgt_berry_flux_grid(const qgt_circuit_desc_t* c, const double* theta, const qgt_flux_options_t* opt,
                        double* flux, double* total)
{
    qgt_flux_options_t o;
    if (opt) o = *opt; else qgt_flux_default_options(&o);
    if (!c || !flux || (c->num_params > 0 && !theta)) return qgt_set_error(E_INVAL, "qgt_berry_flux_grid: NULL argument");
    if (o.param_a < 0 || o.param_b < 0 || o.param_a >= c->num_params || o.param_b >= c->num_params || o.param_a == o.param_b)
        return qgt_set_error(E_INVAL, "qgt_berry_flux_grid: parameters (%d, %d) not two distinct indices below %d",
                             o.param_a, o.param_b, c->num_params);
    if (o.rows < 2 || o.cols < 2 || o.rows > 4096 || o.cols > 4096)
        return qgt_set_error(E_INVAL, "qgt_berry_flux_grid: lattice %d x %d outside [2, 4096]^2", o.rows, o.cols);
    if (!isfinite(o.a0) || !isfinite(o.da) || !isfinite(o.b0) || !isfinite(o.db))
        return qgt_set_error(E_INVAL, "qgt_berry_flux_grid: lattice origin or spacing not finite");
    if (o.periodic != 0 && o.periodic != 1) return qgt_set_error(E_INVAL, "qgt_berry_flux_grid: periodic must be 0 or 1");
    if (o.precision != QGT_PRECISION_FP64 && o.precision != QGT_PRECISION_MIXED)
        return qgt_set_error(E_INVAL, "qgt_berry_flux_grid: precision %d (FP64 or MIXED only)", (int)o.precision);
    for (int k = 0; k < c->num_params; k++)
        if (!isfinite(theta[k])) return qgt_set_error(E_INVAL, "qgt_berry_flux_grid: theta[%d] is not finite", k);

    const int rows = o.rows, cols = o.cols;
    const int prow = o.periodic ? rows : rows - 1;   /* plaquette rows and columns */
    const int pcol = o.periodic ? cols : cols - 1;
    qgt_plan_options_t po;
    qgt_plan_default_options(&po);
    /* complex64 passes need 4 or more qubits */
    po.precision = (o.precision == QGT_PRECISION_MIXED && c->num_qubits >= 4) ? QGT_PRECISION_MIXED : QGT_PRECISION_FP64;
    po.hamiltonian = QGT_HAMILTONIAN_NONE;
    po.device = o.device;
    po.num_deriv_params = 1;
    po.transport = QGT_TRANSPORT_FORWARD;   /* psi after the last gate is row 0 of each point */

    /* size the block of lattice rows from the device bytes of a one-point plan */
    qgt_plan_t* p = NULL;
    qgt_plan_info_t info;
    po.batch = 1;
    int rc = qgt_plan_create(c, &po, &p);
    if (!rc) rc = qgt_plan_get_info(p, &info);
    qgt_plan_destroy(p);
    p = NULL;
    if (rc) return rc;
    int64_t fit = (int64_t)(FLUX_BLOCK_BYTES / (double)(info.device_bytes > 0 ? info.device_bytes : 1));
    if (fit > 65535) fit = 65535;
    int R = (int)(fit / cols) - 1;               /* plaquette rows per block (R + 1 site rows) */
    if (R < 1) R = 1;
    if (R > prow) R = prow;
    const int npts = (R + 1) * cols;
    const int na = R * cols, nb = (R + 1) * cols, npair = na + nb;

    po.batch = npts;
    double* th = (double*)malloc(sizeof(double) * (size_t)npts * (size_t)c->num_params);
    int64_t* off = (int64_t*)malloc(sizeof(int64_t) * 2 * (size_t)npair);
    double* link = NULL;
    int64_t* off_d = NULL;
    double* part_d = NULL;
    if (!th || !off) { rc = qgt_set_error(E_NOMEM, "qgt_berry_flux_grid: out of memory"); goto done; }
    if ((rc = qgt_plan_create(c, &po, &p)) != 0) goto done;
    int64_t ps = 0;
    int32_t fp64 = 0;
    const void* V = qgt_plan_dev_V(p, &ps, &fp64);
    int64_t N = (int64_t)1 << c->num_qubits;
    void* s = qgt_plan_stream(p);
    /* links of a block: a-links (k, j) -> (k + 1, j) for k < R, then b-links
     * (k, j) -> (k, j + 1 mod cols) for k <= R; the same for every block */
    for (int k = 0; k <= R; k++)
        for (int j = 0; j < cols; j++) {
            const int e = k * cols + j;
            if (k < R) {
                off[e] = (int64_t)e * ps;
                off[npair + e] = (int64_t)(e + cols) * ps;
            }
            off[na + e] = (int64_t)e * ps;
            off[npair + na + e] = (int64_t)(k * cols + (j + 1) % cols) * ps;
        }
    const int32_t nch = qgt_overlap_chunks(N, npair);
    link = (double*)malloc(sizeof(double) * 2 * (size_t)npair * (size_t)nch);
    if (!link) { rc = qgt_set_error(E_NOMEM, "qgt_berry_flux_grid: out of memory"); goto done; }
    if ((rc = qgt_dev_malloc((void**)&off_d, sizeof(int64_t) * 2 * (size_t)npair)) != 0) goto done;
    if ((rc = qgt_dev_malloc((void**)&part_d, sizeof(double) * 2 * (size_t)npair * (size_t)nch)) != 0) goto done;
    if ((rc = qgt_dev_memcpy_h2d(off_d, off, sizeof(int64_t) * 2 * (size_t)npair, s)) != 0) goto done;

    memset(flux, 0, sizeof(double) * (size_t)rows * cols);
    for (int r0 = 0; r0 < prow; r0 += R) {
        for (int k = 0; k <= R; k++) {
            int g = r0 + k;
            g = o.periodic ? g % rows : (g < rows ? g : rows - 1);   /* rows past the end only pad */
            for (int j = 0; j < cols; j++) {
                double* t = th + (size_t)(k * cols + j) * c->num_params;
                memcpy(t, theta, sizeof(double) * (size_t)c->num_params);
                t[o.param_a] = o.a0 + g * o.da;
                t[o.param_b] = o.b0 + j * o.db;
            }
        }
        if ((rc = qgt_plan_execute_host(p, th, NULL, NULL, NULL, NULL)) != 0) goto done;
        if ((rc = qgt_dev_overlaps(V, fp64, N, off_d, off_d + npair, npair, nch, part_d, s)) != 0) goto done;
        if ((rc = qgt_dev_memcpy_d2h(link, part_d, sizeof(double) * 2 * (size_t)npair * (size_t)nch, s)) != 0) goto done;
        if ((rc = qgt_dev_stream_sync(s)) != 0) goto done;
        for (int e = 0; e < npair; e++) {   /* partial sums in chunk order */
            double re = 0, im = 0;
            for (int q = 0; q < nch; q++) { re += link[2 * ((size_t)e * nch + q)]; im += link[2 * ((size_t)e * nch + q) + 1]; }
            link[2 * e] = re;
            link[2 * e + 1] = im;
        }
        for (int k = 0; k < R && r0 + k < prow; k++)
            for (int j = 0; j < pcol; j++) {
                const double* u01 = link + 2 * (size_t)(k * cols + j);                     /* <p00|p10> */
                const double* u12 = link + 2 * (size_t)(na + (k + 1) * cols + j);          /* <p10|p11> */
                const double* u32 = link + 2 * (size_t)(k * cols + (j + 1) % cols);        /* <p01|p11> */
                const double* u03 = link + 2 * (size_t)(na + k * cols + j);                /* <p00|p01> */
                double w1r, w1i, w2r, w2i, wr, wi;
                cmul(u01[0], u01[1], u12[0], u12[1], &w1r, &w1i);
                cmul(u32[0], -u32[1], u03[0], -u03[1], &w2r, &w2i);   /* <p11|p01> <p01|p00> */
                cmul(w1r, w1i, w2r, w2i, &wr, &wi);
                flux[(size_t)(r0 + k) * cols + j] = sqrt(wr * wr + wi * wi) > 1e-15 ? atan2(wi, wr) : 0.0;
            }
    }
    if (total) {
        double t = 0;
        for (size_t i = 0; i < (size_t)rows * cols; i++) t += flux[i];
        *total = t;
    }
done:
    qgt_dev_free(off_d);
    qgt_dev_free(part_d);
    qgt_plan_destroy(p);
    free(th);
    free(off);
    free(link);
    return rc;
}
