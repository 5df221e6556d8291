/*
 * qgt_batch.c -- ragged batches of circuits in one CUDA-graph launch.
 *
 * The reference evaluates circuits one at a time, each QGT element by its own
 * network contractions (src/quantum_geometric/core/quantum_geometric_curvature.c:
 * 289-320), and the Berry curvature pointwise from a 2 x 2 QGT
 * (quantum_geometric_curvature.c:181-198).  Here a batch is compiled once:
 *
 *   - circuits with the same structure (qubits, gate list, fixed angles) form
 *     a group and share ONE batched plan: the parameter point is a grid
 *     dimension of every kernel, so a group costs one launch per kernel;
 *   - a Berry map Omega_ab = Im Q_ab on a G x G lattice over [0, 2pi)^2 (the
 *     other parameters at the circuit's theta) runs as a second batched plan
 *     per (pair, truncated circuit): the circuit truncated after the last gate
 *     of a or b, parameters permuted so that a, b are derivative parameters
 *     0, 1; groups whose gates agree up to that gate (an ansatz with more
 *     layers after a and b) share one plan;
 *   - all plans, with the uploads of theta and downloads of Q, are captured
 *     into one CUDA graph over a few streams (independent groups overlap).
 *
 * Closed form used for the maps: when a and b each drive one rotation
 * R(t) = cos(t/2) I - i sin(t/2) G, the truncated circuit's state is
 * sum_{r,s} c_r(ta) c_s(tb) v_rs with v_rs the circuit with G_a^r, G_b^s in
 * place of the rotations, so psi, d_a psi and d_b psi at every lattice point
 * are combinations of four vectors: the plan evaluates the states at
 * (ta, tb) in {0, pi}^2 (v_rs up to phases), one overlap kernel forms their
 * 4 x 4 Gram and one kernel evaluates Omega_ab at all G^2 points from it
 * (qgt_dev_berry_closed).  Parameters shared by several gates get all G^2
 * points as separate 2 x 2 QGTs.
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../qgt_internal.h"
#include "qgt_gb300.h"

#define E_INVAL (-1)
#define E_NOMEM (-2)
#define MAX_STREAMS 16

typedef struct {
    int berry;              /* 0: full QGT plan, 1: Berry-map plan */
    qgt_plan_t* plan;
    int P, Pd;              /* theta width; output width */
    int nmem, per;          /* circuits in the plan; points per circuit */
    int* mem;               /* circuit indices */
    int pa, pb;             /* Berry parameters (circuit numbering) */
    int compact;            /* G points per circuit (exact reduction) instead of G^2 */
    int early_is_a;         /* a's gate precedes b's */
    int* perm;              /* circuit parameter k -> plan parameter perm[k], k < nperm */
    int nperm;
    size_t th_off, out_off; /* doubles into the pinned staging buffers */
    /* closed form (compact pairs): 4 points per circuit, (theta_a, theta_b) in {0, pi}^2; their 10
     * overlaps per circuit (offsets off_d: a then b, 10 nmem each) -> partial sums part_d -> maps_d */
    int64_t* off_d;
    double* part_d;
    double* maps_d;
    int nchunk;
} bplan_t;

struct qgt_batch {
    qgt_batch_options_t opt;
    int count, G;
    int* P;                 /* per circuit */
    size_t *th_at, *q_at;   /* per circuit offsets into the caller's theta / Q arrays */
    bplan_t* bp;
    int nbp, ngroups, nberry;
    double *th_pin, *out_pin;
    size_t th_len, out_len;
    int nstreams;
    void* s[MAX_STREAMS];
    void* ev[MAX_STREAMS + 1];
    void* graph;            /* with the theta uploads and result downloads */
    void* graph_dev;        /* the same work without them */
    int nodes;
    int64_t device_bytes;
};

void qgt_batch_default_options(qgt_batch_options_t* o)
{
    memset(o, 0, sizeof *o);
    o->precision = QGT_PRECISION_MIXED;
    o->berry_grid = 32;
    o->device = 0;
    o->streams = 4;
}

/* gates [0, ng) of a and b equal (types, qubits, parameter indices, fixed angles) */
static int same_gates(const qgt_circuit_desc_t* a, const qgt_circuit_desc_t* b, int ng)
{
    if (a->num_qubits != b->num_qubits || a->num_gates < ng || b->num_gates < ng) return 0;
    for (int g = 0; g < ng; g++) {
        const qgt_gate_desc_t *x = &a->gates[g], *y = &b->gates[g];
        if (x->type != y->type || x->qubits[0] != y->qubits[0] || x->param != y->param) return 0;
        int two = x->type == QGT_GATE_CNOT || x->type == QGT_GATE_CZ || x->type == QGT_GATE_SWAP;
        if (two && x->qubits[1] != y->qubits[1]) return 0;
        if (x->param < 0 && memcmp(&x->angle, &y->angle, sizeof(double)) != 0) return 0;
    }
    return 1;
}

static int same_structure(const qgt_circuit_desc_t* a, const qgt_circuit_desc_t* b)
{
    return a->num_gates == b->num_gates && a->num_params == b->num_params && same_gates(a, b, a->num_gates);
}

/* last gate driven by parameter pa or pb (-1 if none) */
static int last_gate_of(const qgt_circuit_desc_t* c, int pa, int pb)
{
    int gl = -1;
    for (int g = 0; g < c->num_gates; g++)
        if (c->gates[g].param == pa || c->gates[g].param == pb) gl = g;
    return gl;
}

static int make_plan(const qgt_circuit_desc_t* c, const qgt_batch_options_t* bo, int batch, int Pd, qgt_plan_t** out)
{
    qgt_plan_options_t o;
    qgt_plan_default_options(&o);
    o.precision = bo->precision;
    o.hamiltonian = QGT_HAMILTONIAN_NONE;
    o.device = bo->device;
    o.use_graph = 0;
    o.batch = batch;
    o.num_deriv_params = Pd;
    if (bo->tune_cache) {
        /* the fastest measured configuration of this group's plan (timed once, then read from the cache) */
        qgt_plan_options_t t;
        int rc = qgt_plan_autotune(c, &o, bo->tune_cache, 3, &t, NULL);
        if (rc) return rc;
        o.tile_bits = t.tile_bits;
        o.pass_kernels = t.pass_kernels;
    }
    return qgt_plan_create(c, &o, out);
}

void qgt_batch_destroy(qgt_batch_t* b)
{
    if (!b) return;
    if (b->nstreams > 0 && b->s[0]) qgt_dev_stream_sync(b->s[0]);
    qgt_dev_graph_destroy(b->graph);
    qgt_dev_graph_destroy(b->graph_dev);
    for (int i = 0; i < b->nbp; i++) {
        qgt_plan_destroy(b->bp[i].plan);
        free(b->bp[i].mem);
        free(b->bp[i].perm);
        qgt_dev_free(b->bp[i].off_d);
        qgt_dev_free(b->bp[i].part_d);
        qgt_dev_free(b->bp[i].maps_d);
    }
    for (int k = 0; k < MAX_STREAMS; k++) if (b->s[k]) qgt_dev_stream_destroy(b->s[k]);
    for (int k = 0; k <= MAX_STREAMS; k++) if (b->ev[k]) qgt_dev_event_destroy(b->ev[k]);
    qgt_dev_host_free(b->th_pin);
    qgt_dev_host_free(b->out_pin);
    free(b->bp); free(b->P); free(b->th_at); free(b->q_at);
    free(b);
}

/* one graph: fork over the streams, per plan [upload theta ->] step [-> download Q or the map], join */
static int capture(qgt_batch_t* b, const qgt_circuit_desc_t* circuits, int copies, void** graph)
{
    const int K = b->nstreams;
    int cr = qgt_dev_graph_begin(b->s[0]);
    if (!cr) cr = qgt_dev_event_record(b->ev[K], b->s[0]);
    for (int k = 1; k < K && !cr; k++) cr = qgt_dev_stream_wait_event(b->s[k], b->ev[K]);
    int nodes = 0;
    for (int i = 0; i < b->nbp && !cr; i++) {
        bplan_t* bp = &b->bp[i];
        void* st = b->s[i % K];
        const size_t pts = (size_t)bp->nmem * bp->per;
        if (bp->P > 0 && copies)
            cr = qgt_dev_memcpy_h2d(qgt_plan_dev_theta(bp->plan), b->th_pin + bp->th_off,
                                    sizeof(double) * pts * (size_t)bp->P, st);
        if (!cr) cr = qgt_plan_enqueue_step(bp->plan, st);
        if (!cr && bp->berry && bp->compact) {
            int64_t pstride = 0;
            int32_t f64 = 0;
            const void* V = qgt_plan_dev_V(bp->plan, &pstride, &f64);
            const int npair = 10 * bp->nmem;
            const int64_t N = (int64_t)1 << circuits[bp->mem[0]].num_qubits;
            cr = qgt_dev_overlaps(V, f64, N, bp->off_d, bp->off_d + npair, npair, bp->nchunk, bp->part_d, st);
            if (!cr) cr = qgt_dev_berry_closed(bp->part_d, bp->nchunk, bp->nmem, b->G, bp->maps_d, st);
            if (!cr && copies)
                cr = qgt_dev_memcpy_d2h(b->out_pin + bp->out_off, bp->maps_d,
                                        sizeof(double) * (size_t)bp->nmem * b->G * b->G, st);
            nodes += 2;
        } else if (!cr && bp->Pd > 0 && copies) {
            cr = qgt_dev_memcpy_d2h(b->out_pin + bp->out_off, qgt_plan_dev_Q(bp->plan),
                                    sizeof(double) * pts * 2 * (size_t)bp->Pd * bp->Pd, st);
        }
        nodes += qgt_plan_launches(bp->plan) + (copies ? 2 : 0);
    }
    for (int k = 1; k < K && !cr; k++) {
        cr = qgt_dev_event_record(b->ev[k], b->s[k]);
        if (!cr) cr = qgt_dev_stream_wait_event(b->s[0], b->ev[k]);
    }
    void* exec = NULL;
    int re = qgt_dev_graph_end(b->s[0], &exec);
    if (cr) { qgt_dev_graph_destroy(exec); return cr; }
    if (re) return re;
    *graph = exec;
    if (copies) b->nodes = nodes;
    return 0;
}

int qgt_batch_create(const qgt_circuit_desc_t* circuits, int32_t count, const int32_t* berry_params,
                     const qgt_batch_options_t* opt, qgt_batch_t** out)
{
    if (!out) return qgt_set_error(E_INVAL, "qgt_batch_create: NULL output");
    *out = NULL;
    if (!circuits || count < 1) return qgt_set_error(E_INVAL, "qgt_batch_create: no circuits");
    qgt_batch_t* b = (qgt_batch_t*)calloc(1, sizeof *b);
    if (!b) return qgt_set_error(E_NOMEM, "qgt_batch_create: out of memory");
    if (opt) b->opt = *opt; else qgt_batch_default_options(&b->opt);
    int rc = 0;
    b->count = count;
    b->G = b->opt.berry_grid;
    if (b->G < 0 || b->G > 1024) { rc = qgt_set_error(E_INVAL, "qgt_batch_create: berry_grid %d outside [0, 1024]", b->G); goto fail; }
    if (b->opt.precision != QGT_PRECISION_FP64 && b->opt.precision != QGT_PRECISION_MIXED) {
        rc = qgt_set_error(E_INVAL, "qgt_batch_create: batches run FP64 or MIXED precision");
        goto fail;
    }
    if (b->G > 0 && !berry_params) { rc = qgt_set_error(E_INVAL, "qgt_batch_create: berry_grid > 0 needs berry_params"); goto fail; }
    b->nstreams = b->opt.streams < 1 ? 1 : (b->opt.streams > MAX_STREAMS ? MAX_STREAMS : b->opt.streams);
    b->P = (int*)calloc((size_t)count, sizeof(int));
    b->th_at = (size_t*)calloc((size_t)count + 1, sizeof(size_t));
    b->q_at = (size_t*)calloc((size_t)count + 1, sizeof(size_t));
    int* group = (int*)malloc(sizeof(int) * (size_t)count);
    int* rep = (int*)malloc(sizeof(int) * (size_t)count);
    b->bp = (bplan_t*)calloc(2 * (size_t)count, sizeof(bplan_t));
    if (!b->P || !b->th_at || !b->q_at || !group || !rep || !b->bp) {
        free(group); free(rep);
        rc = qgt_set_error(E_NOMEM, "qgt_batch_create: out of memory");
        goto fail;
    }
    for (int c = 0; c < count; c++) {
        b->P[c] = circuits[c].num_params;
        b->th_at[c + 1] = b->th_at[c] + (size_t)b->P[c];
        b->q_at[c + 1] = b->q_at[c] + 2 * (size_t)b->P[c] * b->P[c];
        if (b->G > 0) {
            int pa = berry_params[2 * c], pb = berry_params[2 * c + 1];
            if (pa < 0 || pb < 0 || pa >= b->P[c] || pb >= b->P[c] || pa == pb) {
                free(group); free(rep);
                rc = qgt_set_error(E_INVAL, "qgt_batch_create: circuit %d: Berry parameters (%d, %d) invalid", c, pa, pb);
                goto fail;
            }
        }
    }
    /* structural groups */
    int ng = 0;
    for (int c = 0; c < count; c++) {
        int g = -1;
        for (int k = 0; k < ng && g < 0; k++)
            if (same_structure(&circuits[rep[k]], &circuits[c])) g = k;
        if (g < 0) { g = ng; rep[ng++] = c; }
        group[c] = g;
    }
    b->ngroups = ng;
    for (int g = 0; g < ng; g++) {
        bplan_t* bp = &b->bp[b->nbp];
        const qgt_circuit_desc_t* rc0 = &circuits[rep[g]];
        bp->berry = 0;
        bp->P = bp->Pd = rc0->num_params;
        bp->per = 1;
        bp->mem = (int*)malloc(sizeof(int) * (size_t)count);
        if (!bp->mem) { free(group); free(rep); rc = qgt_set_error(E_NOMEM, "qgt_batch_create: oom"); goto fail; }
        for (int c = 0; c < count; c++) if (group[c] == g) bp->mem[bp->nmem++] = c;
        b->nbp++;
        if ((rc = make_plan(rc0, &b->opt, bp->nmem, 0, &bp->plan)) != 0) { free(group); free(rep); goto fail; }
    }
    /* Berry plans: one per (group, parameter pair) */
    if (b->G > 0) {
        char* done = (char*)calloc((size_t)count, 1);
        qgt_gate_desc_t* tg = NULL;
        if (!done) { free(group); free(rep); rc = qgt_set_error(E_NOMEM, "qgt_batch_create: oom"); goto fail; }
        for (int c = 0; c < count && !rc; c++) {
            if (done[c]) continue;
            const int pa = berry_params[2 * c], pb = berry_params[2 * c + 1];
            const qgt_circuit_desc_t* cc = &circuits[c];
            bplan_t* bp = &b->bp[b->nbp];
            bp->berry = 1;
            bp->pa = pa;
            bp->pb = pb;
            bp->Pd = 2;
            bp->mem = (int*)malloc(sizeof(int) * (size_t)count);
            bp->perm = (int*)malloc(sizeof(int) * (size_t)cc->num_params);
            tg = (qgt_gate_desc_t*)malloc(sizeof(qgt_gate_desc_t) * (size_t)(cc->num_gates + 1));
            if (!bp->mem || !bp->perm || !tg) { rc = qgt_set_error(E_NOMEM, "qgt_batch_create: oom"); break; }
            /* circuits whose gates up to the last one of a or b equal this circuit's (e.g. the
             * same ansatz with more layers after a and b) share the truncated circuit's plan */
            const int gl = last_gate_of(cc, pa, pb);
            for (int d = c; d < count; d++)
                if (!done[d] && berry_params[2 * d] == pa && berry_params[2 * d + 1] == pb &&
                    (group[d] == group[c] || (gl >= 0 && last_gate_of(&circuits[d], pa, pb) == gl &&
                                              same_gates(cc, &circuits[d], gl + 1)))) {
                    bp->mem[bp->nmem++] = d;
                    done[d] = 1;
                }
            b->nbp++;
            int na = 0, nb = 0, ga = -1, gb = -1;
            for (int g = 0; g < cc->num_gates; g++) {
                if (cc->gates[g].param == pa) { na++; if (ga < 0) ga = g; }
                if (cc->gates[g].param == pb) { nb++; if (gb < 0) gb = g; }
            }
            if (na == 0 || nb == 0) {
                rc = qgt_set_error(E_INVAL, "qgt_batch_create: Berry parameter %d drives no gate", na == 0 ? pa : pb);
                break;
            }
            int glast = -1;
            for (int g = 0; g < cc->num_gates; g++)
                if (cc->gates[g].param == pa || cc->gates[g].param == pb) glast = g;
            /* one gate each: the closed form over the states at (theta_a, theta_b) in {0, pi}^2 */
            bp->compact = (na == 1 && nb == 1);
            bp->early_is_a = ga < gb;
            bp->per = bp->compact ? 4 : b->G * b->G;
            bp->nperm = cc->num_params;   /* members with more parameters map the rest beyond bp->P */
            for (int k = 0, nxt = 2; k < cc->num_params; k++)
                bp->perm[k] = (k == pa) ? 0 : (k == pb) ? 1 : nxt++;
            bp->P = 2;   /* plan parameters: a, b, then those of the truncated gates */
            for (int g = 0; g <= glast; g++) {
                tg[g] = cc->gates[g];
                if (tg[g].param >= 0) {
                    tg[g].param = bp->perm[tg[g].param];
                    if (tg[g].param + 1 > bp->P) bp->P = tg[g].param + 1;
                }
            }
            qgt_circuit_desc_t tc = {cc->num_qubits, glast + 1, tg, bp->P};
            if (bp->nmem * bp->per > 65535) {
                rc = qgt_set_error(E_INVAL, "qgt_batch_create: %d Berry points in one group exceed 65535", bp->nmem * bp->per);
                break;
            }
            rc = make_plan(&tc, &b->opt, bp->nmem * bp->per, 2, &bp->plan);
            free(tg);
            tg = NULL;
            b->nberry++;
            if (!rc && bp->compact) {
                /* offsets of the 10 state pairs of every member (points m 4 + t, row 0 = psi) */
                int64_t pstride = 0;
                int32_t f64 = 0;
                (void)qgt_plan_dev_V(bp->plan, &pstride, &f64);
                const int npair = 10 * bp->nmem;
                int64_t* off = (int64_t*)malloc(sizeof(int64_t) * 2 * (size_t)npair);
                if (!off) { rc = qgt_set_error(E_NOMEM, "qgt_batch_create: oom"); break; }
                static const int pi_[10] = {0, 0, 0, 0, 1, 1, 1, 2, 2, 3}, pj_[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};
                for (int m = 0; m < bp->nmem; m++)
                    for (int k = 0; k < 10; k++) {
                        off[m * 10 + k] = (int64_t)(4 * m + pi_[k]) * pstride;
                        off[npair + m * 10 + k] = (int64_t)(4 * m + pj_[k]) * pstride;
                    }
                const int64_t N = (int64_t)1 << cc->num_qubits;
                bp->nchunk = qgt_overlap_chunks(N, npair);
                rc = qgt_dev_malloc((void**)&bp->off_d, sizeof(int64_t) * 2 * (size_t)npair);
                if (!rc) rc = qgt_dev_memcpy_h2d(bp->off_d, off, sizeof(int64_t) * 2 * (size_t)npair, NULL);
                if (!rc) rc = qgt_dev_malloc((void**)&bp->part_d, sizeof(double) * 2 * (size_t)npair * bp->nchunk);
                if (!rc) rc = qgt_dev_malloc((void**)&bp->maps_d, sizeof(double) * (size_t)bp->nmem * b->G * b->G);
                if (!rc) rc = qgt_dev_stream_sync(NULL);
                free(off);
            }
        }
        free(tg);
        free(done);
    }
    free(group);
    free(rep);
    if (rc) goto fail;
    /* pinned staging */
    for (int i = 0; i < b->nbp; i++) {
        bplan_t* bp = &b->bp[i];
        const size_t pts = (size_t)bp->nmem * bp->per;
        bp->th_off = b->th_len;
        bp->out_off = b->out_len;
        b->th_len += pts * (size_t)bp->P;
        if (bp->berry && bp->compact) b->out_len += (size_t)bp->nmem * b->G * b->G;   /* the maps */
        else b->out_len += pts * 2 * (size_t)bp->Pd * bp->Pd;
        qgt_plan_info_t in;
        if (qgt_plan_get_info(bp->plan, &in) == 0) b->device_bytes += in.device_bytes;
    }
    if ((rc = qgt_dev_host_alloc((void**)&b->th_pin, sizeof(double) * (b->th_len + 1))) != 0) goto fail;
    if ((rc = qgt_dev_host_alloc((void**)&b->out_pin, sizeof(double) * (b->out_len + 1))) != 0) goto fail;
    memset(b->th_pin, 0, sizeof(double) * (b->th_len + 1));
    for (int k = 0; k < b->nstreams; k++)
        if ((rc = qgt_dev_stream_create(&b->s[k])) != 0) goto fail;
    for (int k = 0; k <= b->nstreams; k++)
        if ((rc = qgt_dev_event_create(&b->ev[k])) != 0) goto fail;
    /* two graphs: the batch with its copies (execute_host) and the same work on the device-resident
     * inputs and outputs alone (execute_device) */
    if ((rc = capture(b, circuits, 1, &b->graph)) != 0) goto fail;
    if ((rc = capture(b, circuits, 0, &b->graph_dev)) != 0) goto fail;
    *out = b;
    return 0;
fail:
    qgt_batch_destroy(b);
    return rc ? rc : qgt_set_error(E_INVAL, "qgt_batch_create failed");
}

/* host copies of a batch's results, cut into chunks that a few threads take in turn */
typedef struct {
    void* dst;
    const void* src;
    size_t n;
} ucopy_t;
typedef struct {
    ucopy_t* t;
    int n, cap;
    int next;   /* next chunk to take (atomic) */
} unpack_t;

#define UNPACK_CHUNK ((size_t)4 << 20)
#define UNPACK_THREADS 8

static int unpack_add(unpack_t* u, void* dst, const void* src, size_t n)
{
    for (size_t at = 0; at < n; at += UNPACK_CHUNK) {
        if (u->n == u->cap) {
            const int nc = u->cap ? 2 * u->cap : 1024;
            ucopy_t* t = (ucopy_t*)realloc(u->t, sizeof(ucopy_t) * (size_t)nc);
            if (!t) return qgt_set_error(E_NOMEM, "qgt_batch_execute_host: out of host memory");
            u->t = t;
            u->cap = nc;
        }
        const size_t k = n - at < UNPACK_CHUNK ? n - at : UNPACK_CHUNK;
        u->t[u->n++] = (ucopy_t){(char*)dst + at, (const char*)src + at, k};
    }
    return 0;
}

static void* unpack_worker(void* arg)
{
    unpack_t* u = (unpack_t*)arg;
    for (;;) {
        const int i = __atomic_fetch_add(&u->next, 1, __ATOMIC_RELAXED);
        if (i >= u->n) return NULL;
        memcpy(u->t[i].dst, u->t[i].src, u->t[i].n);
    }
}

static void unpack_run(unpack_t* u)
{
    pthread_t th[UNPACK_THREADS - 1];
    int started[UNPACK_THREADS - 1] = {0};
    const int nt = u->n < UNPACK_THREADS ? u->n : UNPACK_THREADS;
    for (int k = 0; k + 1 < nt; k++) started[k] = pthread_create(&th[k], NULL, unpack_worker, u) == 0;
    unpack_worker(u);   /* the calling thread takes chunks too, so every chunk is copied */
    for (int k = 0; k + 1 < nt; k++)
        if (started[k]) pthread_join(th[k], NULL);
}

int qgt_batch_execute_host(qgt_batch_t* b, const double* theta, double* Q, double* berry)
{
    if (!b || !theta) return qgt_set_error(E_INVAL, "qgt_batch_execute_host: NULL argument");
    if (berry && b->G == 0) return qgt_set_error(E_INVAL, "qgt_batch_execute_host: batch built without Berry maps");
    for (size_t k = 0; k < b->th_at[b->count]; k++)
        if (!isfinite(theta[k])) return qgt_set_error(E_INVAL, "qgt_batch_execute_host: theta[%zu] is not finite", k);
    const double step = 2.0 * M_PI / (b->G > 0 ? b->G : 1);
    for (int i = 0; i < b->nbp; i++) {
        const bplan_t* bp = &b->bp[i];
        for (int m = 0; m < bp->nmem; m++) {
            const double* th = theta + b->th_at[bp->mem[m]];
            for (int t = 0; t < bp->per; t++) {
                double* dst = b->th_pin + bp->th_off + ((size_t)m * bp->per + t) * (size_t)bp->P;
                if (!bp->berry) { memcpy(dst, th, sizeof(double) * (size_t)bp->P); continue; }
                const int np = b->P[bp->mem[m]] < bp->nperm ? b->P[bp->mem[m]] : bp->nperm;
                for (int k = 0; k < np; k++)
                    if (bp->perm[k] < bp->P) dst[bp->perm[k]] = th[k];
                if (bp->compact) {
                    dst[0] = (t & 1) ? M_PI : 0.0;   /* the closed form's four states */
                    dst[1] = (t & 2) ? M_PI : 0.0;
                } else {
                    dst[0] = step * (t / b->G);
                    dst[1] = step * (t % b->G);
                }
            }
        }
    }
    int rc = qgt_dev_graph_launch(b->graph, b->s[0]);
    if (!rc) rc = qgt_dev_stream_sync(b->s[0]);
    if (rc) return rc;
    for (int i = 0; i < b->nbp; i++) {
        int st = qgt_plan_device_status(b->bp[i].plan, NULL);
        if (st) return qgt_set_error(st, "qgt_batch_execute_host: plan %d reported device status %d", i, st);
    }
    /* results from the pinned staging buffer into the caller's arrays: contiguous blocks are copied
     * in chunks by a few host threads (one thread copies ~10-20 GB/s, the batch returns ~300 MB);
     * the per-point Berry maps of non-compact plans are gathered by the calling thread */
    const size_t G = (size_t)b->G;
    unpack_t u = {NULL, 0, 0, 0};
    int rc2 = 0;
    for (int i = 0; i < b->nbp && !rc2; i++) {
        const bplan_t* bp = &b->bp[i];
        const size_t blk = 2 * (size_t)bp->Pd * bp->Pd;
        for (int m = 0; m < bp->nmem && !rc2; m++) {
            const int c = bp->mem[m];
            const double* src = b->out_pin + bp->out_off + (size_t)m * bp->per * blk;
            if (!bp->berry) {
                if (Q) rc2 = unpack_add(&u, Q + b->q_at[c], src, sizeof(double) * blk);
                continue;
            }
            if (!berry) continue;
            double* map = berry + (size_t)c * G * G;
            if (bp->compact) {   /* maps formed on the device from the closed form */
                rc2 = unpack_add(&u, map, b->out_pin + bp->out_off + (size_t)m * G * G, sizeof(double) * G * G);
                continue;
            }
            /* Omega_ab = Im Q_01 of the 2 x 2 block (imaginary part at double index 3) */
            for (size_t x = 0; x < G; x++)
                for (size_t y = 0; y < G; y++) map[x * G + y] = src[(x * G + y) * blk + 3];
        }
    }
    if (!rc2) unpack_run(&u);
    free(u.t);
    return rc2;
}

int qgt_batch_execute_device(qgt_batch_t* b)
{
    if (!b) return qgt_set_error(E_INVAL, "qgt_batch_execute_device: NULL batch");
    return qgt_dev_graph_launch(b->graph_dev, b->s[0]);
}

void* qgt_batch_stream(const qgt_batch_t* b)
{
    return b ? b->s[0] : NULL;
}

int qgt_batch_get_info(const qgt_batch_t* b, qgt_batch_info_t* info)
{
    if (!b || !info) return qgt_set_error(E_INVAL, "qgt_batch_get_info: NULL argument");
    memset(info, 0, sizeof *info);
    info->num_circuits = b->count;
    info->num_groups = b->ngroups;
    info->num_berry_plans = b->nberry;
    info->graph_kernels = b->nodes;
    info->device_bytes = b->device_bytes;
    return 0;
}
