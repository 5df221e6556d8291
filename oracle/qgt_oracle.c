/*
 * qgt_oracle.c -- FP64 CPU oracle (TEST INFRASTRUCTURE ONLY; see qgt_oracle.h).
 *
 * Plain C11 + OpenMP restatement of the reference algorithms on the QGT hot
 * path.  Nothing here is shipped in or called by the product library.
 */
#include "qgt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct { double re, im; } cd;

static inline cd cmul(cd a, cd b) { cd r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline cd cadd(cd a, cd b) { cd r = {a.re + b.re, a.im + b.im}; return r; }

/* ------------------------------------------------------------------------ */
/* circuit construction                                                      */
/* ------------------------------------------------------------------------ */

/* learning/quantum_pipeline_impl.c:2499-2526: RY(q) for all q, RZ(q) for all
 * q, then CNOT(q -> q+1).  The CZ ring variant replaces the ladder by
 * CZ(q, q+1 mod n). */
int or_build_ansatz(int n, int layers, int entangler, og_gate_t* gates, int max_gates)
{
    if (n < 1 || layers < 0) return -1;
    int nent = entangler == 0 ? n - 1 : (n >= 3 ? n : n - 1);
    int need = layers * (2 * n + nent);
    if (!gates) return need;
    if (need > max_gates) return -1;
    int g = 0, p = 0;
    for (int l = 0; l < layers; l++) {
        for (int q = 0; q < n; q++) gates[g++] = (og_gate_t){OG_RY, q, -1, p++, 0.0};
        for (int q = 0; q < n; q++) gates[g++] = (og_gate_t){OG_RZ, q, -1, p++, 0.0};
        if (entangler == 0) {
            for (int q = 0; q + 1 < n; q++) gates[g++] = (og_gate_t){OG_CNOT, q, q + 1, -1, 0.0};
        } else {
            for (int q = 0; q < nent; q++) gates[g++] = (og_gate_t){OG_CZ, q, (q + 1) % n, -1, 0.0};
        }
    }
    return g;
}

uint64_t or_splitmix64(uint64_t* s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void or_seed_params(uint64_t seed, int count, double* theta)
{
    uint64_t s = seed;
    for (int i = 0; i < count; i++) {
        double u = (double)(or_splitmix64(&s) >> 11) * (1.0 / 9007199254740992.0);
        theta[i] = 2.0 * M_PI * u;
    }
}

/* ------------------------------------------------------------------------ */
/* gate application (hybrid/quantum_classical_algorithms.c:174-318)          */
/* ------------------------------------------------------------------------ */

static double gate_angle(const og_gate_t* g, const double* theta)
{
    return g->param >= 0 ? theta[g->param] : g->angle;
}

/* 2x2 row-major matrix of a single-qubit gate (a2; quantum_classical_algorithms.c:228-276). */
static void gate_matrix(int type, double a, cd m[4])
{
    double c = cos(a / 2.0), s = sin(a / 2.0), r = 1.0 / sqrt(2.0);
    switch (type) {
    case OG_RX: m[0] = (cd){c, 0}; m[1] = (cd){0, -s}; m[2] = (cd){0, -s}; m[3] = (cd){c, 0}; break;
    case OG_RY: m[0] = (cd){c, 0}; m[1] = (cd){-s, 0}; m[2] = (cd){s, 0}; m[3] = (cd){c, 0}; break;
    case OG_RZ: m[0] = (cd){c, -s}; m[1] = (cd){0, 0}; m[2] = (cd){0, 0}; m[3] = (cd){c, s}; break;
    case OG_X: m[0] = (cd){0, 0}; m[1] = (cd){1, 0}; m[2] = (cd){1, 0}; m[3] = (cd){0, 0}; break;
    case OG_Y: m[0] = (cd){0, 0}; m[1] = (cd){0, -1}; m[2] = (cd){0, 1}; m[3] = (cd){0, 0}; break;
    case OG_Z: m[0] = (cd){1, 0}; m[1] = (cd){0, 0}; m[2] = (cd){0, 0}; m[3] = (cd){-1, 0}; break;
    case OG_H: m[0] = (cd){r, 0}; m[1] = (cd){r, 0}; m[2] = (cd){r, 0}; m[3] = (cd){-r, 0}; break;
    case OG_S: m[0] = (cd){1, 0}; m[1] = (cd){0, 0}; m[2] = (cd){0, 0}; m[3] = (cd){0, 1}; break;
    case OG_T: m[0] = (cd){1, 0}; m[1] = (cd){0, 0}; m[2] = (cd){0, 0}; m[3] = (cd){r, r}; break;
    default: m[0] = (cd){1, 0}; m[1] = (cd){0, 0}; m[2] = (cd){0, 0}; m[3] = (cd){1, 0}; break;
    }
}

/* (-i/2) G for the generator G of a rotation gate (exact entries). */
static void generator_matrix(int type, cd m[4])
{
    switch (type) {
    case OG_RX: m[0] = (cd){0, 0}; m[1] = (cd){0, -0.5}; m[2] = (cd){0, -0.5}; m[3] = (cd){0, 0}; break;
    case OG_RY: m[0] = (cd){0, 0}; m[1] = (cd){-0.5, 0}; m[2] = (cd){0.5, 0}; m[3] = (cd){0, 0}; break;
    default: /* RZ */ m[0] = (cd){0, -0.5}; m[1] = (cd){0, 0}; m[2] = (cd){0, 0}; m[3] = (cd){0, 0.5}; break;
    }
}

/* The gate loops below run over the amplitudes in parallel when `par` is set
 * (large vectors, one vector at a time); callers that already run one vector
 * per thread pass 0.  Every iteration touches its own pair of amplitudes. */
static void apply_1q_p(cd* v, size_t dim, int q, const cd m[4], int par)
{
    size_t mask = (size_t)1 << q;
    #pragma omp parallel for if (par) schedule(static)
    for (size_t i = 0; i < dim; i++) {
        if (i & mask) continue;
        size_t j = i | mask;
        cd a0 = v[i], a1 = v[j];
        v[i] = cadd(cmul(m[0], a0), cmul(m[1], a1));
        v[j] = cadd(cmul(m[2], a0), cmul(m[3], a1));
    }
}

static void apply_gate_p(cd* v, int n, const og_gate_t* g, const double* theta, int par)
{
    size_t dim = (size_t)1 << n;
    if (g->type == OG_CNOT) {
        size_t cm = (size_t)1 << g->q0, tm = (size_t)1 << g->q1;
        #pragma omp parallel for if (par) schedule(static)
        for (size_t i = 0; i < dim; i++)
            if ((i & cm) && !(i & tm)) { cd t = v[i]; v[i] = v[i | tm]; v[i | tm] = t; }
    } else if (g->type == OG_CZ) {
        size_t am = (size_t)1 << g->q0, bm = (size_t)1 << g->q1;
        #pragma omp parallel for if (par) schedule(static)
        for (size_t i = 0; i < dim; i++)
            if ((i & am) && (i & bm)) { v[i].re = -v[i].re; v[i].im = -v[i].im; }
    } else if (g->type == OG_SWAP) {
        size_t am = (size_t)1 << g->q0, bm = (size_t)1 << g->q1;
        #pragma omp parallel for if (par) schedule(static)
        for (size_t i = 0; i < dim; i++)
            if ((i & am) && !(i & bm)) { size_t j = (i & ~am) | bm; cd t = v[i]; v[i] = v[j]; v[j] = t; }
    } else {
        cd m[4];
        gate_matrix(g->type, gate_angle(g, theta), m);
        apply_1q_p(v, dim, g->q0, m, par);
    }
}

static void apply_gate(cd* v, int n, const og_gate_t* g, const double* theta) { apply_gate_p(v, n, g, theta, 0); }

/* amplitude-parallel loops pay off from this many amplitudes on */
#define OR_PAR_DIM ((size_t)1 << 16)

static int is_rotation(int t) { return t == OG_RX || t == OG_RY || t == OG_RZ; }

int or_simulate(int n, const og_gate_t* gates, int ngates, const double* theta, double* psi)
{
    if (n < 1 || n > 30) return -1;
    size_t dim = (size_t)1 << n;
    cd* v = (cd*)psi;
    memset(v, 0, dim * sizeof(cd));
    v[0].re = 1.0;
    for (int g = 0; g < ngates; g++) apply_gate_p(v, n, &gates[g], theta, dim >= OR_PAR_DIM);
    return 0;
}

/* Exact derivative states: every live derivative vector is transported with
 * psi; at a parameterised gate for parameter k the vector (-i/2) G_k psi is
 * added to row k.  This is the exact form of core/quantum_geometric_gradient.c
 * compute_higher_order_gradient (a4): (psi(theta+pi/2) - psi(theta-pi/2))/(2 sqrt 2). */
int or_derivatives(int n, const og_gate_t* gates, int ngates, const double* theta,
                   int nparams, double* psi, double* D)
{
    if (n < 1 || n > 30 || nparams < 0) return -1;
    size_t dim = (size_t)1 << n;
    cd* v = (cd*)psi;
    cd* d = (cd*)D;
    memset(v, 0, dim * sizeof(cd));
    v[0].re = 1.0;
    memset(d, 0, (size_t)nparams * dim * sizeof(cd));
    char* live = (char*)calloc((size_t)nparams + 1, 1);
    int* live_list = (int*)malloc(sizeof(int) * ((size_t)nparams + 1));
    if (!live || !live_list) { free(live); free(live_list); return -1; }
    int nlive = 0;
    cd* tmp = (cd*)malloc(dim * sizeof(cd));
    if (!tmp) { free(live); free(live_list); return -1; }
    /* few vectors of many amplitudes: parallel over the amplitudes of each vector; otherwise one
     * vector per thread */
    const int big = dim >= OR_PAR_DIM;
    for (int g = 0; g < ngates; g++) {
        const og_gate_t* gt = &gates[g];
        apply_gate_p(v, n, gt, theta, big);
        if (big) {
            for (int j = 0; j < nlive; j++) apply_gate_p(d + (size_t)live_list[j] * dim, n, gt, theta, 1);
        } else {
            #pragma omp parallel for schedule(dynamic, 1)
            for (int j = 0; j < nlive; j++) apply_gate(d + (size_t)live_list[j] * dim, n, gt, theta);
        }
        if (is_rotation(gt->type) && gt->param >= 0) {
            int k = gt->param;
            if (k >= nparams) { free(live); free(live_list); free(tmp); return -1; }
            cd m[4];
            generator_matrix(gt->type, m);
            memcpy(tmp, v, dim * sizeof(cd));
            apply_1q_p(tmp, dim, gt->q0, m, big);
            cd* row = d + (size_t)k * dim;
            #pragma omp parallel for
            for (size_t i = 0; i < dim; i++) row[i] = cadd(row[i], tmp[i]);
            if (!live[k]) { live[k] = 1; live_list[nlive++] = k; }
        }
    }
    free(tmp);
    free(live);
    free(live_list);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* QGT contraction (a5)                                                      */
/* ------------------------------------------------------------------------ */

int or_qgt(size_t dim, int P, const double* psi, const double* D, double* Q)
{
    const cd* v = (const cd*)psi;
    const cd* d = (const cd*)D;
    cd* q = (cd*)Q;
    cd* proj = (cd*)malloc(sizeof(cd) * (size_t)(P > 0 ? P : 1));
    if (!proj) return -1;
    /* proj_m = <d_m|psi> */
    #pragma omp parallel for
    for (int m = 0; m < P; m++) {
        double re = 0, im = 0;
        const cd* a = d + (size_t)m * dim;
        for (size_t k = 0; k < dim; k++) {
            re += a[k].re * v[k].re + a[k].im * v[k].im;
            im += a[k].re * v[k].im - a[k].im * v[k].re;
        }
        proj[m] = (cd){re, im};
    }
    /* Q_mn = <d_m|d_n> - <d_m|psi><psi|d_n>, upper triangle then Hermitian mirror */
    #pragma omp parallel for schedule(dynamic, 1)
    for (int m = 0; m < P; m++) {
        const cd* a = d + (size_t)m * dim;
        for (int nn = m; nn < P; nn++) {
            const cd* b = d + (size_t)nn * dim;
            double re = 0, im = 0;
            for (size_t k = 0; k < dim; k++) {
                re += a[k].re * b[k].re + a[k].im * b[k].im;
                im += a[k].re * b[k].im - a[k].im * b[k].re;
            }
            cd pn = {proj[nn].re, -proj[nn].im}; /* <psi|d_n> */
            cd pr = cmul(proj[m], pn);
            cd val = {re - pr.re, im - pr.im};
            q[(size_t)m * P + nn] = val;
            q[(size_t)nn * P + m] = (cd){val.re, -val.im};
        }
    }
    free(proj);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* energy and gradient (a8)                                                  */
/* ------------------------------------------------------------------------ */

static int tfim_bonds(int n) { return n >= 3 ? n : n - 1; }

void or_tfim_apply(int n, double J, double h, const double* psi, double* out)
{
    size_t dim = (size_t)1 << n;
    const cd* v = (const cd*)psi;
    cd* o = (cd*)out;
    int nb = tfim_bonds(n);
    #pragma omp parallel for
    for (size_t i = 0; i < dim; i++) {
        /* diagonal: -J sum Z_a Z_b */
        double zz = 0;
        for (int b = 0; b < nb; b++) {
            int qa = b, qb = (b + 1) % n;
            int za = (i >> qa) & 1, zb = (i >> qb) & 1;
            zz += (za ^ zb) ? -1.0 : 1.0;
        }
        cd acc = {-J * zz * v[i].re, -J * zz * v[i].im};
        for (int q = 0; q < n; q++) {
            cd w = v[i ^ ((size_t)1 << q)];
            acc.re -= h * w.re;
            acc.im -= h * w.im;
        }
        o[i] = acc;
    }
}

/* H psi for H = sum_k c_k P_k, P_k a Pauli string (compute_pauli_expectation,
 * hybrid/quantum_classical_algorithms.c:320-382): character [n-1-q] of the
 * string acts on qubit q; X, Y, Z (either case), anything else is the
 * identity; a string whose length is not n contributes nothing.  Each
 * operator is applied qubit by qubit to a copy of psi, as the reference does. */
void or_pauli_apply(int n, int nterms, const char* const* strings, const double* coeffs, const double* psi,
                    double* out)
{
    size_t dim = (size_t)1 << n;
    cd* o = (cd*)out;
    cd* t = (cd*)malloc(dim * sizeof(cd));
    memset(out, 0, 2 * dim * sizeof(double));
    if (!t) return;
    for (int k = 0; k < nterms; k++) {
        const char* s = strings[k];
        if (!s || (int)strlen(s) != n) continue;
        memcpy(t, psi, dim * sizeof(cd));
        for (int q = 0; q < n; q++) {
            char c = s[n - 1 - q];
            size_t m = (size_t)1 << q;
            if (c == 'X' || c == 'x') {
                for (size_t i = 0; i < dim; i++)
                    if (!(i & m)) { cd a = t[i]; t[i] = t[i | m]; t[i | m] = a; }
            } else if (c == 'Y' || c == 'y') {
                /* Y = [[0, -i], [i, 0]]: new0 = -i old1, new1 = i old0 */
                for (size_t i = 0; i < dim; i++)
                    if (!(i & m)) {
                        cd a0 = t[i], a1 = t[i | m];
                        t[i].re = a1.im; t[i].im = -a1.re;
                        t[i | m].re = -a0.im; t[i | m].im = a0.re;
                    }
            } else if (c == 'Z' || c == 'z') {
                for (size_t i = 0; i < dim; i++)
                    if (i & m) { t[i].re = -t[i].re; t[i].im = -t[i].im; }
            }
        }
        for (size_t i = 0; i < dim; i++) { o[i].re += coeffs[k] * t[i].re; o[i].im += coeffs[k] * t[i].im; }
    }
    free(t);
}

double or_tfim_energy(int n, double J, double h, const double* psi)
{
    size_t dim = (size_t)1 << n;
    double* hp = (double*)malloc(2 * dim * sizeof(double));
    if (!hp) return NAN;
    or_tfim_apply(n, J, h, psi, hp);
    double e = 0;
    for (size_t i = 0; i < dim; i++) e += psi[2 * i] * hp[2 * i] + psi[2 * i + 1] * hp[2 * i + 1];
    free(hp);
    return e;
}

void or_energy_grad(size_t dim, int P, const double* D, const double* Hpsi, double* grad)
{
    #pragma omp parallel for
    for (int k = 0; k < P; k++) {
        const double* a = D + 2 * (size_t)k * dim;
        double re = 0;
        for (size_t i = 0; i < dim; i++) re += a[2 * i] * Hpsi[2 * i] + a[2 * i + 1] * Hpsi[2 * i + 1];
        grad[k] = 2.0 * re;
    }
}

int or_param_shift_grad(int n, const og_gate_t* gates, int ngates, const double* theta,
                        int P, double J, double h, double* grad)
{
    size_t dim = (size_t)1 << n;
    double* th = (double*)malloc(sizeof(double) * (size_t)(P > 0 ? P : 1));
    double* psi = (double*)malloc(2 * dim * sizeof(double));
    if (!th || !psi) { free(th); free(psi); return -1; }
    memcpy(th, theta, sizeof(double) * (size_t)P);
    for (int k = 0; k < P; k++) {
        double o = th[k];
        th[k] = o + M_PI / 2;
        or_simulate(n, gates, ngates, th, psi);
        double ep = or_tfim_energy(n, J, h, psi);
        th[k] = o - M_PI / 2;
        or_simulate(n, gates, ngates, th, psi);
        double em = or_tfim_energy(n, J, h, psi);
        th[k] = o;
        grad[k] = (ep - em) / 2.0;
    }
    free(th);
    free(psi);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* natural-gradient solves (a7)                                              */
/* ------------------------------------------------------------------------ */

int or_cholesky_solve(int P, const double* A, double lambda, const double* b, double* x,
                      double* lambda_used)
{
    double* L = (double*)calloc((size_t)P * P, sizeof(double));
    double* y = (double*)malloc(sizeof(double) * (size_t)P);
    if (!L || !y) { free(L); free(y); return -1; }
    for (int attempt = 0; attempt < 12; attempt++) {
        int ok = 1;
        memset(L, 0, sizeof(double) * (size_t)P * P);
        for (int i = 0; i < P && ok; i++) {
            for (int j = 0; j <= i; j++) {
                double s = A[(size_t)i * P + j] + (i == j ? lambda : 0.0);
                for (int k = 0; k < j; k++) s -= L[(size_t)i * P + k] * L[(size_t)j * P + k];
                if (i == j) {
                    if (s <= 0) { ok = 0; break; }
                    L[(size_t)i * P + i] = sqrt(s);
                } else {
                    L[(size_t)i * P + j] = s / L[(size_t)j * P + j];
                }
            }
        }
        if (!ok) { lambda *= 10.0; continue; }
        for (int i = 0; i < P; i++) {
            double s = b[i];
            for (int k = 0; k < i; k++) s -= L[(size_t)i * P + k] * y[k];
            y[i] = s / L[(size_t)i * P + i];
        }
        for (int i = P - 1; i >= 0; i--) {
            double s = y[i];
            for (int k = i + 1; k < P; k++) s -= L[(size_t)k * P + i] * x[k];
            x[i] = s / L[(size_t)i * P + i];
        }
        if (lambda_used) *lambda_used = lambda;
        free(L);
        free(y);
        return 0;
    }
    free(L);
    free(y);
    return -1;
}

static double dot(const double* a, const double* b, int n)
{
    double s = 0;
    for (int i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

static void matvec(int P, const double* A, const double* x, double* y)
{
    #pragma omp parallel for
    for (int i = 0; i < P; i++) {
        double s = 0;
        for (int j = 0; j < P; j++) s += A[(size_t)i * P + j] * x[j];
        y[i] = s;
    }
}

int or_cg_solve(int P, const double* A, const double* b, double* x, int max_iter, double tol)
{
    return or_pcg_solve(P, A, b, x, max_iter, tol, NULL, NULL, 0);
}

/* Woodbury: (D + U U^T)^{-1} r = D^{-1} r - D^{-1} U (I + U^T D^{-1} U)^{-1} U^T D^{-1} r */
typedef struct { int P, r; const double* d; const double* U; double* Sinv; double* t; double* w; } wb_t;

static int wb_init(wb_t* w, int P, const double* d, const double* U, int r)
{
    w->P = P; w->r = r; w->d = d; w->U = U;
    w->Sinv = (double*)calloc((size_t)r * r + 1, sizeof(double));
    w->t = (double*)calloc((size_t)r + 1, sizeof(double));
    w->w = (double*)calloc((size_t)r + 1, sizeof(double));
    if (!w->Sinv || !w->t || !w->w) return -1;
    /* S = I + U^T D^{-1} U, then invert by Gauss-Jordan (SPD, small r) */
    double* S = (double*)calloc((size_t)r * r + 1, sizeof(double));
    if (!S) return -1;
    for (int a = 0; a < r; a++)
        for (int c = 0; c < r; c++) {
            double s = (a == c) ? 1.0 : 0.0;
            for (int i = 0; i < P; i++) s += U[(size_t)i * r + a] * U[(size_t)i * r + c] / d[i];
            S[a * r + c] = s;
        }
    for (int a = 0; a < r; a++) w->Sinv[a * r + a] = 1.0;
    for (int c = 0; c < r; c++) {
        double piv = S[c * r + c];
        for (int j = 0; j < r; j++) { S[c * r + j] /= piv; w->Sinv[c * r + j] /= piv; }
        for (int a = 0; a < r; a++) {
            if (a == c) continue;
            double f = S[a * r + c];
            for (int j = 0; j < r; j++) { S[a * r + j] -= f * S[c * r + j]; w->Sinv[a * r + j] -= f * w->Sinv[c * r + j]; }
        }
    }
    free(S);
    return 0;
}

static void wb_apply(wb_t* w, const double* rin, double* z)
{
    int P = w->P, r = w->r;
    for (int i = 0; i < P; i++) z[i] = rin[i] / w->d[i];
    if (r == 0) return;
    for (int a = 0; a < r; a++) {
        double s = 0;
        for (int i = 0; i < P; i++) s += w->U[(size_t)i * r + a] * z[i];
        w->t[a] = s;
    }
    for (int a = 0; a < r; a++) {
        double s = 0;
        for (int c = 0; c < r; c++) s += w->Sinv[a * r + c] * w->t[c];
        w->w[a] = s;
    }
    for (int i = 0; i < P; i++) {
        double s = 0;
        for (int a = 0; a < r; a++) s += w->U[(size_t)i * r + a] * w->w[a];
        z[i] -= s / w->d[i];
    }
}

int or_pcg_solve(int P, const double* A, const double* b, double* x, int max_iter, double tol,
                 const double* d, const double* U, int r)
{
    double* rr = (double*)malloc(sizeof(double) * (size_t)P);
    double* p = (double*)malloc(sizeof(double) * (size_t)P);
    double* Ap = (double*)malloc(sizeof(double) * (size_t)P);
    double* z = (double*)malloc(sizeof(double) * (size_t)P);
    wb_t w = {0};
    int pre = d != NULL;
    if (!rr || !p || !Ap || !z || (pre && wb_init(&w, P, d, U, r) != 0)) {
        free(rr); free(p); free(Ap); free(z); free(w.Sinv); free(w.t); free(w.w);
        return -1;
    }
    memset(x, 0, sizeof(double) * (size_t)P);
    memcpy(rr, b, sizeof(double) * (size_t)P);
    if (pre) wb_apply(&w, rr, z); else memcpy(z, rr, sizeof(double) * (size_t)P);
    memcpy(p, z, sizeof(double) * (size_t)P);
    double rz = dot(rr, z, P);
    int it = 0;
    if (sqrt(dot(rr, rr, P)) < tol) max_iter = 0;
    for (it = 0; it < max_iter;) {
        matvec(P, A, p, Ap);
        double pAp = dot(p, Ap, P);
        if (fabs(pAp) < 1e-15) break;
        double alpha = rz / pAp;
        for (int i = 0; i < P; i++) { x[i] += alpha * p[i]; rr[i] -= alpha * Ap[i]; }
        it++;
        if (sqrt(dot(rr, rr, P)) < tol) break;
        if (pre) wb_apply(&w, rr, z); else memcpy(z, rr, sizeof(double) * (size_t)P);
        double rznew = dot(rr, z, P);
        double beta = rznew / rz;
        for (int i = 0; i < P; i++) p[i] = z[i] + beta * p[i];
        rz = rznew;
    }
    free(rr); free(p); free(Ap); free(z); free(w.Sinv); free(w.t); free(w.w);
    return it;
}

/* ------------------------------------------------------------------------ */
/* Berry-curvature map over two parameters (a10)                             */
/* ------------------------------------------------------------------------ */

int or_berry_map(int n, const og_gate_t* gates, int ngates, const double* theta, int P,
                 int pa, int pb, int grid, double* out)
{
    if (pa < 0 || pb < 0 || pa >= P || pb >= P || pa == pb || grid < 1) return -1;
    size_t dim = (size_t)1 << n;
    int fail = 0;
    #pragma omp parallel
    {
        /* a private gate list in which only (pa, pb) stay parameters (as 0, 1) */
        og_gate_t* g2 = (og_gate_t*)malloc(sizeof(og_gate_t) * (size_t)(ngates > 0 ? ngates : 1));
        double* psi = (double*)malloc(2 * dim * sizeof(double));
        double* D = (double*)malloc(4 * dim * sizeof(double));
        double Q[8];
        if (!g2 || !psi || !D) {
            #pragma omp atomic write
            fail = 1;
        } else {
            #pragma omp for schedule(dynamic, 1)
            for (int ij = 0; ij < grid * grid; ij++) {
                int i = ij / grid, j = ij % grid;
                double th2[2] = {2.0 * M_PI * i / grid, 2.0 * M_PI * j / grid};
                for (int g = 0; g < ngates; g++) {
                    g2[g] = gates[g];
                    if (gates[g].param >= 0) {
                        if (gates[g].param == pa) g2[g].param = 0;
                        else if (gates[g].param == pb) g2[g].param = 1;
                        else { g2[g].param = -1; g2[g].angle = theta[gates[g].param]; }
                    }
                }
                or_derivatives(n, g2, ngates, th2, 2, psi, D);
                or_qgt(dim, 2, psi, D, Q);
                out[ij] = Q[3]; /* Im Q_{ab} */
            }
        }
        free(g2); free(psi); free(D);
    }
    return fail ? -1 : 0;
}

/* ---- Berry phases of loops (distributed/differential_geometry.c:2908-2945;
 *      cuda/quantum_phase_cuda.cu:245-313) ---- */

static void or_inner(const double* a, const double* b, size_t dim, double* re, double* im)
{
    double r = 0, i = 0;
    for (size_t k = 0; k < dim; k++) {
        r += a[2 * k] * b[2 * k] + a[2 * k + 1] * b[2 * k + 1];
        i += a[2 * k] * b[2 * k + 1] - a[2 * k + 1] * b[2 * k];
    }
    *re = r;
    *im = i;
}

int or_berry_phase(const double* const* states, size_t n, size_t dim, double* out)
{
    out[0] = 1.0;
    out[1] = 0.0;
    if (!states || n < 2 || dim == 0) return 0;
    for (size_t i = 0; i < n; i++) {
        double re, im;
        or_inner(states[i], states[(i + 1) % n], dim, &re, &im);
        double mag = sqrt(re * re + im * im);
        if (!(mag > 1e-14)) { out[0] = out[1] = 0.0; return -1; }
        re /= mag;
        im /= mag;
        double r = out[0] * re - out[1] * im;
        out[1] = out[0] * im + out[1] * re;
        out[0] = r;
    }
    return 0;
}

int or_berry_flux(int n, const og_gate_t* gates, int ngates, const double* theta, int P, int pa, int pb,
                  int rows, int cols, double a0, double da, double b0, double db, int periodic, double* flux)
{
    if (pa < 0 || pb < 0 || pa >= P || pb >= P || pa == pb || rows < 2 || cols < 2) return -1;
    const size_t dim = (size_t)1 << n, S = (size_t)rows * cols;
    double* st = (double*)malloc(sizeof(double) * 2 * dim * S);
    if (!st) return -1;
    int fail = 0;
    #pragma omp parallel
    {
        double* th = (double*)malloc(sizeof(double) * (size_t)(P > 0 ? P : 1));
        if (!th) {
            #pragma omp atomic write
            fail = 1;
        } else {
            #pragma omp for schedule(dynamic, 4)
            for (long ij = 0; ij < (long)S; ij++) {
                memcpy(th, theta, sizeof(double) * (size_t)P);
                th[pa] = a0 + (double)(ij / cols) * da;
                th[pb] = b0 + (double)(ij % cols) * db;
                if (or_simulate(n, gates, ngates, th, st + 2 * dim * (size_t)ij) != 0) {
                    #pragma omp atomic write
                    fail = 1;
                }
            }
        }
        free(th);
    }
    if (fail) { free(st); return -1; }
    #pragma omp parallel for schedule(dynamic, 4)
    for (long ij = 0; ij < (long)S; ij++) {
        const int i = (int)(ij / cols), j = (int)(ij % cols);
        if (!periodic && (i == rows - 1 || j == cols - 1)) { flux[ij] = 0.0; continue; }
        const int i1 = (i + 1) % rows, j1 = (j + 1) % cols;
        const double* p00 = st + 2 * dim * ((size_t)i * cols + j);
        const double* p10 = st + 2 * dim * ((size_t)i1 * cols + j);
        const double* p01 = st + 2 * dim * ((size_t)i * cols + j1);
        const double* p11 = st + 2 * dim * ((size_t)i1 * cols + j1);
        double u[4][2];
        or_inner(p00, p10, dim, &u[0][0], &u[0][1]);
        or_inner(p10, p11, dim, &u[1][0], &u[1][1]);
        or_inner(p11, p01, dim, &u[2][0], &u[2][1]);
        or_inner(p01, p00, dim, &u[3][0], &u[3][1]);
        double w1r = u[0][0] * u[1][0] - u[0][1] * u[1][1], w1i = u[0][0] * u[1][1] + u[0][1] * u[1][0];
        double w2r = u[2][0] * u[3][0] - u[2][1] * u[3][1], w2i = u[2][0] * u[3][1] + u[2][1] * u[3][0];
        double wr = w1r * w2r - w1i * w2i, wi = w1r * w2i + w1i * w2r;
        flux[ij] = sqrt(wr * wr + wi * wi) > 1e-15 ? atan2(wi, wr) : 0.0;
    }
    free(st);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* one full QGT step in slices (CPU baseline)                                */
/* ------------------------------------------------------------------------ */

/* The whole step (psi, every derivative state, Gram, projector, TFIM energy
 * and gradient, Cholesky natural-gradient solve) cut into `nslices` calls
 * that together do each piece of work exactly once: slice s carries psi up
 * to the gate of its last derivative row (spawning its rows on the way, as
 * or_derivatives does), transports its rows to the end of the circuit, and
 * adds their Gram rows against every row made so far; the last slice also
 * finishes psi and forms Q, energy, gradient and natural gradient. */
struct or_qgt_job {
    int n, ngates, P, nrows, nslices, next, gpsi;
    size_t dim;
    og_gate_t* gates;
    double* theta;
    int* row_gate;
    int* row_param;
    cd* psi;
    cd* D;
    cd* B;            /* nrows x nrows: B[i][j] = <D_i|D_j>, filled for j <= i */
    double J, h, lambda;
    double *Q, *grad, *energy, *natgrad;
};

void or_qgt_job_destroy(or_qgt_job_t* j)
{
    if (!j) return;
    free(j->gates); free(j->theta); free(j->row_gate); free(j->row_param);
    free(j->psi); free(j->D); free(j->B);
    free(j);
}

or_qgt_job_t* or_qgt_job_create(int n, const og_gate_t* gates, int ngates, const double* theta, int P, int nslices,
                                double J, double h, double lambda, double* Q, double* grad, double* energy,
                                double* natgrad)
{
    if (n < 1 || n > 30 || ngates < 0 || P < 1 || nslices < 1) return NULL;
    or_qgt_job_t* j = (or_qgt_job_t*)calloc(1, sizeof(*j));
    if (!j) return NULL;
    j->n = n;
    j->dim = (size_t)1 << n;
    j->ngates = ngates;
    j->P = P;
    j->J = J; j->h = h; j->lambda = lambda;
    j->Q = Q; j->grad = grad; j->energy = energy; j->natgrad = natgrad;
    j->gates = (og_gate_t*)malloc(sizeof(og_gate_t) * (size_t)(ngates > 0 ? ngates : 1));
    j->theta = (double*)malloc(sizeof(double) * (size_t)P);
    j->row_gate = (int*)malloc(sizeof(int) * (size_t)(ngates > 0 ? ngates : 1));
    j->row_param = (int*)malloc(sizeof(int) * (size_t)(ngates > 0 ? ngates : 1));
    j->psi = (cd*)malloc(sizeof(cd) * j->dim);
    if (!j->gates || !j->theta || !j->row_gate || !j->row_param || !j->psi) { or_qgt_job_destroy(j); return NULL; }
    memcpy(j->gates, gates, sizeof(og_gate_t) * (size_t)ngates);
    memcpy(j->theta, theta, sizeof(double) * (size_t)P);
    for (int g = 0; g < ngates; g++)
        if (is_rotation(gates[g].type) && gates[g].param >= 0) {
            if (gates[g].param >= P) { or_qgt_job_destroy(j); return NULL; }
            j->row_gate[j->nrows] = g;
            j->row_param[j->nrows] = gates[g].param;
            j->nrows++;
        }
    j->nslices = nslices > j->nrows ? (j->nrows > 0 ? j->nrows : 1) : nslices;
    j->D = (cd*)calloc((size_t)(j->nrows > 0 ? j->nrows : 1) * j->dim, sizeof(cd));
    j->B = (cd*)calloc((size_t)(j->nrows > 0 ? j->nrows : 1) * (size_t)(j->nrows > 0 ? j->nrows : 1), sizeof(cd));
    if (!j->D || !j->B) { or_qgt_job_destroy(j); return NULL; }
    memset(j->psi, 0, sizeof(cd) * j->dim);
    j->psi[0].re = 1.0;
    return j;
}

int or_qgt_job_slices(const or_qgt_job_t* j) { return j ? j->nslices : 0; }

static void job_finish(or_qgt_job_t* j)
{
    const size_t dim = j->dim;
    const int R = j->nrows, P = j->P;
    for (int g = j->gpsi; g < j->ngates; g++) apply_gate_p(j->psi, j->n, &j->gates[g], j->theta, dim >= OR_PAR_DIM);
    j->gpsi = j->ngates;
    cd* v = (cd*)calloc((size_t)(R > 0 ? R : 1), sizeof(cd));
    double* gr = (double*)calloc((size_t)(R > 0 ? R : 1), sizeof(double));
    cd* hp = (cd*)malloc(sizeof(cd) * dim);
    if (!v || !gr || !hp) { free(v); free(gr); free(hp); return; }
    or_tfim_apply(j->n, j->J, j->h, (const double*)j->psi, (double*)hp);
    double e = 0;
    #pragma omp parallel for reduction(+:e) schedule(static)
    for (size_t k = 0; k < dim; k++) e += j->psi[k].re * hp[k].re + j->psi[k].im * hp[k].im;
    /* v_i = <D_i|psi>, g_i = 2 Re <D_i|H psi> */
    #pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < R; i++) {
        const cd* a = j->D + (size_t)i * dim;
        double vr = 0, vi = 0, g = 0;
        for (size_t k = 0; k < dim; k++) {
            vr += a[k].re * j->psi[k].re + a[k].im * j->psi[k].im;
            vi += a[k].re * j->psi[k].im - a[k].im * j->psi[k].re;
            g += a[k].re * hp[k].re + a[k].im * hp[k].im;
        }
        v[i] = (cd){vr, vi};
        gr[i] = 2.0 * g;
    }
    cd* q = (cd*)j->Q;
    memset(q, 0, sizeof(cd) * (size_t)P * P);
    memset(j->grad, 0, sizeof(double) * (size_t)P);
    for (int a = 0; a < R; a++) {
        j->grad[j->row_param[a]] += gr[a];
        for (int b = 0; b < R; b++) {
            /* <D_a|D_b> from the filled lower part (Hermitian) */
            cd bab = a >= b ? j->B[(size_t)a * R + b] : (cd){j->B[(size_t)b * R + a].re, -j->B[(size_t)b * R + a].im};
            cd vv = cmul(v[a], (cd){v[b].re, -v[b].im});
            cd* t = &q[(size_t)j->row_param[a] * P + j->row_param[b]];
            t->re += bab.re - vv.re;
            t->im += bab.im - vv.im;
        }
    }
    *j->energy = e;
    double* A = (double*)malloc(sizeof(double) * (size_t)P * P);
    if (A) {
        for (size_t k = 0; k < (size_t)P * P; k++) A[k] = q[k].re;
        double used;
        if (or_cholesky_solve(P, A, j->lambda, j->grad, j->natgrad, &used) != 0)
            for (int k = 0; k < P; k++) j->natgrad[k] = NAN;
        free(A);
    }
    free(v); free(gr); free(hp);
}

/* runs the next slice; returns the number of slices left (0 after the last), -1 on error */
int or_qgt_job_step(or_qgt_job_t* j)
{
    if (!j || j->next >= j->nslices) return -1;
    const int s = j->next;
    const size_t dim = j->dim;
    const int R = j->nrows;
    const int r0 = (int)((int64_t)s * R / j->nslices), r1 = (int)((int64_t)(s + 1) * R / j->nslices);
    const int big = dim >= OR_PAR_DIM;
    if (r1 > r0) {
        /* psi up to the last row's gate, spawning and carrying this slice's rows */
        const int gl = j->row_gate[r1 - 1];
        int live0 = r0, live1 = r0;   /* rows [live0, live1) are spawned */
        for (int g = j->gpsi; g <= gl; g++) {
            const og_gate_t* gt = &j->gates[g];
            apply_gate_p(j->psi, j->n, gt, j->theta, big);
            if (big) {
                for (int r = live0; r < live1; r++) apply_gate_p(j->D + (size_t)r * dim, j->n, gt, j->theta, 1);
            } else {
                #pragma omp parallel for schedule(dynamic, 1)
                for (int r = live0; r < live1; r++) apply_gate(j->D + (size_t)r * dim, j->n, gt, j->theta);
            }
            if (live1 < r1 && j->row_gate[live1] == g) {
                cd m[4];
                generator_matrix(gt->type, m);
                cd* row = j->D + (size_t)live1 * dim;
                memcpy(row, j->psi, sizeof(cd) * dim);
                apply_1q_p(row, dim, gt->q0, m, big);
                live1++;
            }
        }
        j->gpsi = gl + 1;
        /* the slice's rows to the end of the circuit: one row per thread */
        #pragma omp parallel for schedule(dynamic, 1)
        for (int r = r0; r < r1; r++)
            for (int g = gl + 1; g < j->ngates; g++) apply_gate(j->D + (size_t)r * dim, j->n, &j->gates[g], j->theta);
        /* Gram rows i in [r0, r1) against j <= i, over amplitude chunks */
        const int m = r1 - r0;
        const size_t chunk = 256;
        const size_t nch = (dim + chunk - 1) / chunk;
        #pragma omp parallel
        {
            cd* acc = (cd*)calloc((size_t)m * (size_t)r1, sizeof(cd));
            #pragma omp for schedule(static)
            for (size_t c = 0; c < nch; c++) {
                const size_t k0 = c * chunk, k1 = k0 + chunk < dim ? k0 + chunk : dim;
                for (int i = r0; i < r1; i++) {
                    const cd* a = j->D + (size_t)i * dim;
                    for (int jj = 0; jj <= i; jj++) {
                        const cd* b = j->D + (size_t)jj * dim;
                        double re = 0, im = 0;
                        for (size_t k = k0; k < k1; k++) {
                            re += a[k].re * b[k].re + a[k].im * b[k].im;
                            im += a[k].re * b[k].im - a[k].im * b[k].re;
                        }
                        if (acc) {
                            acc[(size_t)(i - r0) * r1 + jj].re += re;
                            acc[(size_t)(i - r0) * r1 + jj].im += im;
                        }
                    }
                }
            }
            #pragma omp critical
            {
                if (acc)
                    for (int i = r0; i < r1; i++)
                        for (int jj = 0; jj <= i; jj++) {
                            j->B[(size_t)i * R + jj].re += acc[(size_t)(i - r0) * r1 + jj].re;
                            j->B[(size_t)i * R + jj].im += acc[(size_t)(i - r0) * r1 + jj].im;
                        }
            }
            free(acc);
        }
    }
    j->next++;
    if (j->next == j->nslices) job_finish(j);
    return j->nslices - j->next;
}
