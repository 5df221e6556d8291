/*
 * qgt_plan.c -- circuit -> tile-pass schedule compiler and the plan driver.
 *
 * The reference evaluates every Q element separately, re-contracting its
 * tensor network 13 times per element (src/quantum_geometric/core/
 * quantum_geometric_curvature.c:300-317, quantum_geometric_tensor_network.c:
 * 1058-1181).  A plan instead runs one step per parameter point:
 *
 *   prepare      theta -> gate matrices (FP64, on the device)
 *   passes       psi and every derivative slot d_s = d psi / d a_s through
 *                the tile passes (exact generator insertion, in-place
 *                transport); the last pass writes the Gram operands
 *   H psi        TFIM ring, one extra row
 *   Gram         HG = <V_i|V_j> over rows (psi, H psi, d_0 .. d_{S-1})
 *   post         FP64: renormalisation, slot -> parameter sums, projector,
 *                energy and gradient
 *   solve        FP64 Cholesky of (Re Q + lambda I) x = grad E
 *
 * all captured in one CUDA graph.
 *
 * Schedule: gates are packed greedily into passes.  A pass holds a tile set S
 * of at most QGT_TILE_MAX qubits (qubits 0..4 always included); a gate joins
 * the current pass if it commutes with every earlier gate left out of the
 * pass and its non-diagonal qubits fit in S (S may still grow).  Diagonal
 * gates (RZ, Z, S, T, CZ) and CNOT controls never need to be tile bits.
 * Commutation is decided per shared qubit: both gates must act there as
 * functions of the same Pauli (Z-type, X-type or Y-type).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../qgt_internal.h"
#include "qgt_gb300.h"

#define E_INVAL (-1)
#define E_NOMEM (-2)
#define E_STATE (-4)
#define E_HW (-6)

/* per-qubit action type of a gate, for commutation */
enum { AT_NONE = 0, AT_Z = 1, AT_X = 2, AT_Y = 3, AT_G = 4 };

typedef struct {
    int type, q0, q1, param;
    double angle;
    int slot;        /* derivative slot, -1 */
    int coef;        /* coefficient index, -1 */
    int diag;        /* diagonal in the computational basis */
    uint32_t need;   /* qubits that must be tile bits */
    uint32_t touch;  /* all qubits touched */
    int at0, at1;    /* action types on q0 / q1 */
} sgate_t;

typedef struct {
    int op_begin, op_count;
    int ent_begin, ent_count;
    int tile_bits;
    uint32_t tile_mask;
    int8_t l2p[16];
} spass_t;

struct qgt_plan {
    qgt_plan_options_t opt;
    int n, P, nslots, rows, rows_pad;
    int64_t N, split_ld;
    int fp64;
    /* schedule */
    int ngates;
    sgate_t* gates;
    int npasses;
    spass_t* passes;
    qgt_dev_op_t* ops_h;
    int nops;
    qgt_dev_entry_t* ents_h;
    int nents;
    qgt_dev_coef_desc_t* coef_h;
    int ncoef;
    int32_t *slot_param_h, *param_ptr_h, *param_slots_h;
    /* device */
    void* stream;
    void* graph;
    void* V;
    void* split;
    qgt_dev_op_t* ops_d;
    qgt_dev_entry_t* ents_d;
    qgt_dev_coef_desc_t* coef_desc_d;
    double* coef_d;
    double* theta_d;
    double* HG_d;
    double* part_d;
    int part_nsplit;
    qgt_tc_gram_t* tc;            /* split-BF16 x3 Gram (operands written by the last pass) */
    qgt_dg_gram_t* dg;            /* integer-digit FP16 Gram (mixed default) */
    uint32_t* rowmax_d;           /* per-row max |amplitude| (float bits) for the digit Gram */
    double *Q_d, *grad_d, *energy_d, *natgrad_d, *chol_work_d, *status_d;
    int32_t *slot_param_d, *param_ptr_d, *param_slots_d;
    /* pinned host staging */
    double *theta_pin, *Q_pin, *grad_pin, *energy_pin, *natgrad_pin, *status_pin;
    double hscale;
    float split_scale;
    int64_t device_bytes;
    int64_t vector_passes, gate_bytes;
    int launches;
    int has_run;
};

static int popcount32(uint32_t x) { return __builtin_popcount(x); }

void qgt_plan_default_options(qgt_plan_options_t* o)
{
    memset(o, 0, sizeof *o);
    o->precision = QGT_PRECISION_MIXED;
    o->hamiltonian = QGT_HAMILTONIAN_TFIM;
    o->tfim_J = 1.0;
    o->tfim_h = 1.0;
    o->lambda = 1e-3;
    o->device = 0;
    o->use_graph = 1;
}

/* ------------------------------------------------------------------------ */
/* gate classification                                                       */
/* ------------------------------------------------------------------------ */

static int classify(const qgt_gate_desc_t* d, int n, int nparams, sgate_t* g)
{
    memset(g, 0, sizeof *g);
    g->type = d->type;
    g->q0 = d->qubits[0];
    g->q1 = d->qubits[1];
    g->param = d->param;
    g->angle = d->angle;
    g->slot = -1;
    g->coef = -1;
    int two = (d->type == QGT_GATE_CNOT || d->type == QGT_GATE_CZ || d->type == QGT_GATE_SWAP);
    if (g->q0 < 0 || g->q0 >= n) return qgt_set_error(E_INVAL, "gate qubit %d out of range [0,%d)", g->q0, n);
    if (two) {
        if (g->q1 < 0 || g->q1 >= n || g->q1 == g->q0)
            return qgt_set_error(E_INVAL, "two-qubit gate needs two distinct qubits in range (got %d, %d)", g->q0, g->q1);
    } else {
        g->q1 = -1;
    }
    int rot = (d->type == QGT_GATE_RX || d->type == QGT_GATE_RY || d->type == QGT_GATE_RZ);
    if (rot && d->param >= nparams) return qgt_set_error(E_INVAL, "gate parameter %d >= num_params %d", d->param, nparams);
    if (!rot && d->param >= 0) return qgt_set_error(E_INVAL, "gate type %d takes no parameter", d->type);
    if (rot && d->param < 0 && !isfinite(d->angle)) return qgt_set_error(E_INVAL, "non-finite fixed angle");
    uint32_t b0 = 1u << g->q0, b1 = two ? (1u << g->q1) : 0;
    g->touch = b0 | b1;
    switch (d->type) {
    case QGT_GATE_RX: case QGT_GATE_X: g->need = b0; g->at0 = AT_X; break;
    case QGT_GATE_RY: case QGT_GATE_Y: g->need = b0; g->at0 = AT_Y; break;
    case QGT_GATE_H: g->need = b0; g->at0 = AT_G; break;
    case QGT_GATE_RZ: case QGT_GATE_Z: case QGT_GATE_S: case QGT_GATE_T: g->diag = 1; g->at0 = AT_Z; break;
    case QGT_GATE_I: g->diag = 1; g->touch = 0; break;
    case QGT_GATE_CNOT: g->need = b1; g->at0 = AT_Z; g->at1 = AT_X; break;
    case QGT_GATE_CZ: g->diag = 1; g->at0 = AT_Z; g->at1 = AT_Z; break;
    case QGT_GATE_SWAP: g->need = b0 | b1; g->at0 = AT_G; g->at1 = AT_G; break;
    default: return qgt_set_error(E_INVAL, "unsupported gate type %d", d->type);
    }
    return 0;
}

static int action_on(const sgate_t* g, int q)
{
    if (g->q0 == q) return g->at0;
    if (g->q1 == q) return g->at1;
    return AT_NONE;
}

static int commute(const sgate_t* a, const sgate_t* b)
{
    uint32_t sh = a->touch & b->touch;
    while (sh) {
        int q = __builtin_ctz(sh);
        sh &= sh - 1;
        int ta = action_on(a, q), tb = action_on(b, q);
        if (ta != tb || ta == AT_G) return 0;
    }
    return 1;
}

/* ------------------------------------------------------------------------ */
/* schedule                                                                  */
/* ------------------------------------------------------------------------ */

static int compile_schedule(qgt_plan_t* p)
{
    const int n = p->n, G = p->ngates;
    const int tmax = n < (p->fp64 ? QGT_TILE_MAX_F64 : QGT_TILE_MAX_F32) ? n : (p->fp64 ? QGT_TILE_MAX_F64 : QGT_TILE_MAX_F32);
    const int lane = n < QGT_LANE_BITS ? n : QGT_LANE_BITS;
    char* placed = (char*)calloc((size_t)G + 1, 1);
    int* blocked = (int*)malloc(sizeof(int) * ((size_t)G + 1));
    int* order = (int*)malloc(sizeof(int) * ((size_t)G + 1));  /* gate order within passes */
    int cap = 16;
    p->passes = (spass_t*)calloc((size_t)cap, sizeof(spass_t));
    p->ops_h = (qgt_dev_op_t*)calloc((size_t)G + 1, sizeof(qgt_dev_op_t));
    if (!placed || !blocked || !order || !p->passes || !p->ops_h) {
        free(placed); free(blocked); free(order);
        return qgt_set_error(E_NOMEM, "schedule: out of memory");
    }
    int remaining = 0;
    for (int g = 0; g < G; g++) {
        if (p->gates[g].type == QGT_GATE_I && p->gates[g].slot < 0) placed[g] = 1;
        else remaining++;
    }
    int nord = 0, np = 0, first = 0;
    while (remaining > 0) {
        uint32_t S = (lane >= 32) ? 0xffffffffu : ((1u << lane) - 1u);
        int nb = 0, start = nord;
        while (first < G && placed[first]) first++;
        for (int g = first; g < G; g++) {
            if (placed[g]) continue;
            const sgate_t* cg = &p->gates[g];
            int ok = 1;
            for (int b = 0; b < nb && ok; b++) ok = commute(&p->gates[blocked[b]], cg);
            if (ok) {
                uint32_t need = cg->need;
                if ((need & ~S) == 0) { /* fits */ }
                else if (popcount32(S | need) <= tmax) S |= need;
                else ok = 0;
            }
            if (ok) { placed[g] = 1; order[nord++] = g; remaining--; }
            else blocked[nb++] = g;
        }
        if (nord == start) {
            free(placed); free(blocked); free(order);
            return qgt_set_error(E_STATE, "schedule: no progress (internal error)");
        }
        /* widen S to tmax with the lowest free qubits: larger, more contiguous tiles */
        for (int q = 0; q < n && popcount32(S) < tmax; q++) S |= 1u << q;
        if (np == cap) {
            cap *= 2;
            spass_t* nps = (spass_t*)realloc(p->passes, sizeof(spass_t) * (size_t)cap);
            if (!nps) { free(placed); free(blocked); free(order); return qgt_set_error(E_NOMEM, "schedule: oom"); }
            p->passes = nps;
        }
        spass_t* ps = &p->passes[np++];
        memset(ps, 0, sizeof *ps);
        ps->tile_mask = S;
        ps->tile_bits = popcount32(S);
        int8_t p2l[32];
        for (int q = 0, l = 0; q < 32; q++) {
            p2l[q] = -1;
            if (q < n && ((S >> q) & 1)) { ps->l2p[l] = (int8_t)q; p2l[q] = (int8_t)l; l++; }
        }
        ps->op_begin = start;
        ps->op_count = nord - start;
        for (int k = start; k < nord; k++) {
            const sgate_t* g = &p->gates[order[k]];
            qgt_dev_op_t* op = &p->ops_h[k];
            memset(op, 0, sizeof *op);
            op->q = (int8_t)g->q0;
            op->q2 = (int8_t)(g->q1 >= 0 ? g->q1 : 0);
            op->lb = p2l[g->q0];
            op->lb2 = g->q1 >= 0 ? p2l[g->q1] : -1;
            op->coef = g->coef;
            op->slot = g->slot;
            op->gen = QGEN_NONE;
            switch (g->type) {
            case QGT_GATE_RX: op->kind = QOP_1Q; op->gen = g->slot >= 0 ? QGEN_X : 0; break;
            case QGT_GATE_RY: op->kind = QOP_1Q; op->gen = g->slot >= 0 ? QGEN_Y : 0; break;
            case QGT_GATE_H: case QGT_GATE_X: case QGT_GATE_Y: op->kind = QOP_1Q; break;
            case QGT_GATE_RZ: op->kind = QOP_PHASE; op->gen = g->slot >= 0 ? QGEN_Z : 0; break;
            case QGT_GATE_Z: case QGT_GATE_S: case QGT_GATE_T: op->kind = QOP_PHASE; break;
            case QGT_GATE_CZ: op->kind = QOP_CZ; break;
            case QGT_GATE_CNOT:
                /* target in lb, control in lb2 / q2 */
                op->q = (int8_t)g->q1; op->lb = p2l[g->q1];
                op->q2 = (int8_t)g->q0; op->lb2 = p2l[g->q0];
                op->kind = QOP_CNOT;
                break;
            case QGT_GATE_SWAP: op->kind = QOP_SWAP; break;
            default: op->kind = QOP_PHASE; break; /* identity never reaches here */
            }
        }
    }
    p->npasses = np;
    p->nops = nord;
    free(placed);
    free(blocked);
    free(order);
    return 0;
}

/* entries: psi ping-pongs between row 0 and row `rows`, ending in row 0 */
static int build_entries(qgt_plan_t* p)
{
    int cap = 64, ne = 0;
    p->ents_h = (qgt_dev_entry_t*)malloc(sizeof(qgt_dev_entry_t) * (size_t)cap);
    if (!p->ents_h) return qgt_set_error(E_NOMEM, "entries: oom");
    char* live = (char*)calloc((size_t)p->nslots + 1, 1);
    if (!live) return qgt_set_error(E_NOMEM, "entries: oom");
    const int last = p->npasses - 1;
    const int split = p->opt.precision == QGT_PRECISION_MIXED_BF16X3;
    const int rmax = p->opt.precision == QGT_PRECISION_MIXED ? QENT_ROWMAX : 0;
    p->vector_passes = 0;
    p->gate_bytes = 0;
    const int64_t ab = p->fp64 ? 16 : 8; /* bytes per amplitude */
    for (int k = 0; k < p->npasses; k++) {
        spass_t* ps = &p->passes[k];
        ps->ent_begin = ne;
        int psi_dst = ((last - k) % 2 == 0) ? 0 : p->rows;
        int psi_src = (k == 0) ? -1 : (((last - (k - 1)) % 2 == 0) ? 0 : p->rows);
        int need = 1 + p->nslots;
        if (ne + need > cap) {
            while (ne + need > cap) cap *= 2;
            qgt_dev_entry_t* ne2 = (qgt_dev_entry_t*)realloc(p->ents_h, sizeof(qgt_dev_entry_t) * (size_t)cap);
            if (!ne2) { free(live); return qgt_set_error(E_NOMEM, "entries: oom"); }
            p->ents_h = ne2;
        }
        /* psi */
        qgt_dev_entry_t e;
        memset(&e, 0, sizeof e);
        e.src_row = psi_src < 0 ? 0 : psi_src;
        e.dst_row = psi_dst;
        e.spawn_op = -1;
        e.flags = QENT_STORE_V | (psi_src < 0 ? QENT_SRC_ZERO : 0) | ((k == last && split) ? QENT_STORE_SPLIT : 0) |
                  (k == last ? rmax : 0);
        e.split_row = 0;
        p->ents_h[ne++] = e;
        p->gate_bytes += ab * p->N * ((psi_src < 0 ? 0 : 1) + 1) + ((k == last && split) ? 8 * p->N : 0);
        /* transports of slots spawned in earlier passes */
        for (int s = 0; s < p->nslots; s++) {
            if (!live[s]) continue;
            memset(&e, 0, sizeof e);
            e.src_row = 2 + s;
            e.dst_row = 2 + s;
            e.spawn_op = -1;
            e.flags = ((k == last && split) ? QENT_STORE_SPLIT : QENT_STORE_V) | (k == last ? rmax : 0);
            e.split_row = 2 + s;
            p->ents_h[ne++] = e;
            p->gate_bytes += ab * p->N + ((k == last && split) ? 8 * p->N : ab * p->N);
        }
        /* spawns in this pass */
        for (int j = 0; j < ps->op_count; j++) {
            const qgt_dev_op_t* op = &p->ops_h[ps->op_begin + j];
            if (op->slot < 0) continue;
            memset(&e, 0, sizeof e);
            e.src_row = psi_src < 0 ? 0 : psi_src;
            e.dst_row = 2 + op->slot;
            e.spawn_op = j;
            e.flags = (psi_src < 0 ? QENT_SRC_ZERO : 0) | ((k == last && split) ? QENT_STORE_SPLIT : QENT_STORE_V) |
                      (k == last ? rmax : 0);
            e.split_row = 2 + op->slot;
            p->ents_h[ne++] = e;
            p->gate_bytes += ab * p->N * (psi_src < 0 ? 0 : 1) + ((k == last && split) ? 8 * p->N : ab * p->N);
        }
        for (int j = 0; j < ps->op_count; j++) {
            const qgt_dev_op_t* op = &p->ops_h[ps->op_begin + j];
            if (op->slot >= 0) live[op->slot] = 1;
        }
        ps->ent_count = ne - ps->ent_begin;
        if (ps->ent_count > 65535) { free(live); return qgt_set_error(E_INVAL, "pass has more than 65535 vectors"); }
        p->vector_passes += ps->ent_count;
    }
    p->nents = ne;
    free(live);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* plan lifecycle                                                            */
/* ------------------------------------------------------------------------ */

#define DALLOC(ptr, bytes)                                                        \
    do {                                                                          \
        size_t b_ = (size_t)(bytes);                                              \
        if ((rc = qgt_dev_malloc((void**)&(ptr), b_ ? b_ : 16)) != 0) goto fail;  \
        p->device_bytes += (int64_t)(b_ ? b_ : 16);                               \
    } while (0)

static int run_step(qgt_plan_t* p);

int qgt_plan_create(const qgt_circuit_desc_t* c, const qgt_plan_options_t* opt, qgt_plan_t** out)
{
    int rc = 0;
    if (!out) return qgt_set_error(E_INVAL, "qgt_plan_create: plan pointer is NULL");
    *out = NULL;
    if (!c || (c->num_gates > 0 && !c->gates)) return qgt_set_error(E_INVAL, "qgt_plan_create: circuit is NULL");
    if (c->num_qubits < 1 || c->num_qubits > QGT_MAX_QUBITS)
        return qgt_set_error(E_INVAL, "qgt_plan_create: num_qubits %d outside [1, %d]", c->num_qubits, QGT_MAX_QUBITS);
    if (c->num_gates < 0 || c->num_params < 0) return qgt_set_error(E_INVAL, "qgt_plan_create: negative sizes");
    qgt_plan_t* p = (qgt_plan_t*)calloc(1, sizeof(qgt_plan_t));
    if (!p) return qgt_set_error(E_NOMEM, "qgt_plan_create: out of memory");
    if (opt) p->opt = *opt; else qgt_plan_default_options(&p->opt);
    if (p->opt.precision < QGT_PRECISION_FP64 || p->opt.precision > QGT_PRECISION_MIXED_BF16X3) {
        int bad = (int)p->opt.precision;
        free(p);
        return qgt_set_error(E_INVAL, "qgt_plan_create: unknown precision %d", bad);
    }
    if (!(p->opt.lambda >= 0) || !isfinite(p->opt.lambda)) { free(p); return qgt_set_error(E_INVAL, "lambda must be >= 0"); }
    p->n = c->num_qubits;
    p->N = (int64_t)1 << p->n;
    p->P = c->num_params;
    p->fp64 = p->opt.precision == QGT_PRECISION_FP64;
    p->ngates = c->num_gates;
    p->gates = (sgate_t*)calloc((size_t)p->ngates + 1, sizeof(sgate_t));
    p->coef_h = (qgt_dev_coef_desc_t*)calloc((size_t)p->ngates + 1, sizeof(qgt_dev_coef_desc_t));
    if (!p->gates || !p->coef_h) { rc = qgt_set_error(E_NOMEM, "oom"); goto fail; }
    for (int g = 0; g < p->ngates; g++) {
        if ((rc = classify(&c->gates[g], p->n, p->P, &p->gates[g])) != 0) goto fail;
        sgate_t* sg = &p->gates[g];
        int rot = sg->type == QGT_GATE_RX || sg->type == QGT_GATE_RY || sg->type == QGT_GATE_RZ;
        if (rot && sg->param >= 0) sg->slot = p->nslots++;
        if (sg->type != QGT_GATE_CNOT && sg->type != QGT_GATE_CZ && sg->type != QGT_GATE_SWAP && sg->type != QGT_GATE_I) {
            sg->coef = p->ncoef;
            p->coef_h[p->ncoef].type = sg->type;
            p->coef_h[p->ncoef].param = sg->param;
            p->coef_h[p->ncoef].angle = sg->angle;
            p->ncoef++;
        }
    }
    p->rows = 2 + p->nslots;
    p->rows_pad = (p->rows + 127) / 128 * 128;
    p->split_ld = p->N < 32 ? 32 : p->N;
    /* slot -> param CSR */
    p->slot_param_h = (int32_t*)calloc((size_t)p->nslots + 1, sizeof(int32_t));
    p->param_ptr_h = (int32_t*)calloc((size_t)p->P + 2, sizeof(int32_t));
    p->param_slots_h = (int32_t*)calloc((size_t)p->nslots + 1, sizeof(int32_t));
    if (!p->slot_param_h || !p->param_ptr_h || !p->param_slots_h) { rc = qgt_set_error(E_NOMEM, "oom"); goto fail; }
    for (int g = 0; g < p->ngates; g++)
        if (p->gates[g].slot >= 0) { p->slot_param_h[p->gates[g].slot] = p->gates[g].param; p->param_ptr_h[p->gates[g].param + 1]++; }
    for (int q = 0; q < p->P; q++) p->param_ptr_h[q + 1] += p->param_ptr_h[q];
    {
        int32_t* fill = (int32_t*)calloc((size_t)p->P + 1, sizeof(int32_t));
        if (!fill) { rc = qgt_set_error(E_NOMEM, "oom"); goto fail; }
        for (int s = 0; s < p->nslots; s++) {
            int q = p->slot_param_h[s];
            p->param_slots_h[p->param_ptr_h[q] + fill[q]++] = s;
        }
        free(fill);
    }
    if ((rc = compile_schedule(p)) != 0) goto fail;
    if ((rc = build_entries(p)) != 0) goto fail;
    {
        int nb = p->n >= 3 ? p->n : p->n - 1;
        p->hscale = fabs(p->opt.tfim_J) * nb + fabs(p->opt.tfim_h) * p->n;
        if (p->hscale <= 0) p->hscale = 1.0;
    }
    p->split_scale = 16384.0f; /* 2^14: |amplitude| <= 1 stays below the FP16 maximum */

    /* ---- device resources ---- */
    if ((rc = qgt_dev_set_device(p->opt.device)) != 0) goto fail;
    if ((rc = qgt_dev_stream_create(&p->stream)) != 0) goto fail;
    {
        size_t ab = p->fp64 ? 16 : 8;
        DALLOC(p->V, (size_t)(p->rows + 1) * (size_t)p->N * ab);
        if ((rc = qgt_dev_memset(p->V, 0, (size_t)(p->rows + 1) * (size_t)p->N * ab, p->stream)) != 0) goto fail;
        if (p->opt.precision == QGT_PRECISION_MIXED_BF16X3) {
            size_t sb = (size_t)4 * p->rows_pad * (size_t)p->split_ld * 2;
            DALLOC(p->split, sb);
            if ((rc = qgt_dev_memset(p->split, 0, sb, p->stream)) != 0) goto fail;
        }
    }
    DALLOC(p->ops_d, sizeof(qgt_dev_op_t) * (size_t)(p->nops + 1));
    DALLOC(p->ents_d, sizeof(qgt_dev_entry_t) * (size_t)(p->nents + 1));
    DALLOC(p->coef_desc_d, sizeof(qgt_dev_coef_desc_t) * (size_t)(p->ncoef + 1));
    DALLOC(p->coef_d, sizeof(double) * 8 * (size_t)(p->ncoef + 1));
    DALLOC(p->theta_d, sizeof(double) * (size_t)(p->P + 1));
    DALLOC(p->HG_d, sizeof(double) * 2 * (size_t)p->rows * p->rows);
    DALLOC(p->Q_d, sizeof(double) * 2 * (size_t)p->P * p->P);
    DALLOC(p->grad_d, sizeof(double) * (size_t)(p->P + 1));
    DALLOC(p->energy_d, sizeof(double) * 2);
    DALLOC(p->natgrad_d, sizeof(double) * (size_t)(p->P + 1));
    DALLOC(p->chol_work_d, sizeof(double) * (size_t)p->P * p->P);
    DALLOC(p->status_d, sizeof(double) * 2);
    DALLOC(p->slot_param_d, sizeof(int32_t) * (size_t)(p->nslots + 1));
    DALLOC(p->param_ptr_d, sizeof(int32_t) * (size_t)(p->P + 2));
    DALLOC(p->param_slots_d, sizeof(int32_t) * (size_t)(p->nslots + 1));
    if (p->fp64) {
        int nt = (p->rows + 31) / 32, ntp = nt * (nt + 1) / 2;
        int ns = (int)(4 * 152 / ntp);
        if (ns < 1) ns = 1;
        int64_t maxs = p->N / 64;
        if (maxs < 1) maxs = 1;
        if (ns > maxs) ns = (int)maxs;
        p->part_nsplit = ns;
        DALLOC(p->part_d, sizeof(double) * 2 * 1024 * (size_t)ntp * ns);
    } else if (p->opt.precision == QGT_PRECISION_MIXED_BF16X3) {
        if ((rc = qgt_dev_tc_gram_create(p->split, p->split_ld, p->rows, p->rows_pad, 1, &p->tc)) != 0) goto fail;
        p->device_bytes += qgt_dev_tc_gram_scratch_bytes(p->tc);
    } else {
        if (p->n < 4) { rc = qgt_set_error(E_INVAL, "mixed precision needs at least 4 qubits (use FP64)"); goto fail; }
        DALLOC(p->rowmax_d, sizeof(uint32_t) * (size_t)p->rows);
        if ((rc = qgt_dev_dg_gram_create(p->V, p->N, p->rows, p->rowmax_d, &p->dg)) != 0) goto fail;
        p->device_bytes += qgt_dev_dg_gram_scratch_bytes(p->dg);
    }
    if ((rc = qgt_dev_memset(p->theta_d, 0, sizeof(double) * (size_t)(p->P + 1), p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_memcpy_h2d(p->ops_d, p->ops_h, sizeof(qgt_dev_op_t) * (size_t)p->nops, p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_memcpy_h2d(p->ents_d, p->ents_h, sizeof(qgt_dev_entry_t) * (size_t)p->nents, p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_memcpy_h2d(p->coef_desc_d, p->coef_h, sizeof(qgt_dev_coef_desc_t) * (size_t)p->ncoef, p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_memcpy_h2d(p->slot_param_d, p->slot_param_h, sizeof(int32_t) * (size_t)p->nslots, p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_memcpy_h2d(p->param_ptr_d, p->param_ptr_h, sizeof(int32_t) * (size_t)(p->P + 1), p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_memcpy_h2d(p->param_slots_d, p->param_slots_h, sizeof(int32_t) * (size_t)p->nslots, p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_host_alloc((void**)&p->theta_pin, sizeof(double) * (size_t)(p->P + 1))) != 0) goto fail;
    if ((rc = qgt_dev_host_alloc((void**)&p->Q_pin, sizeof(double) * 2 * (size_t)p->P * p->P + 16)) != 0) goto fail;
    if ((rc = qgt_dev_host_alloc((void**)&p->grad_pin, sizeof(double) * (size_t)(p->P + 1))) != 0) goto fail;
    if ((rc = qgt_dev_host_alloc((void**)&p->natgrad_pin, sizeof(double) * (size_t)(p->P + 1))) != 0) goto fail;
    if ((rc = qgt_dev_host_alloc((void**)&p->energy_pin, sizeof(double) * 2)) != 0) goto fail;
    if ((rc = qgt_dev_host_alloc((void**)&p->status_pin, sizeof(double) * 2)) != 0) goto fail;
    if ((rc = qgt_dev_stream_sync(p->stream)) != 0) goto fail;
    /* first step eagerly (sets kernel attributes, validates), then capture */
    if ((rc = run_step(p)) != 0) goto fail;
    if ((rc = qgt_dev_stream_sync(p->stream)) != 0) goto fail;
    if (p->opt.use_graph) {
        if ((rc = qgt_dev_graph_begin(p->stream)) != 0) goto fail;
        int rs = run_step(p);
        void* exec = NULL;
        int re = qgt_dev_graph_end(p->stream, &exec);
        if (rs) { rc = rs; goto fail; }
        if (re) { rc = re; goto fail; }
        p->graph = exec;
    }
    *out = p;
    return 0;
fail:
    qgt_plan_destroy(p);
    return rc ? rc : qgt_set_error(E_HW, "qgt_plan_create failed");
}

void qgt_plan_destroy(qgt_plan_t* p)
{
    if (!p) return;
    if (p->stream) qgt_dev_stream_sync(p->stream);
    qgt_dev_graph_destroy(p->graph);
    qgt_dev_tc_gram_destroy(p->tc);
    qgt_dev_dg_gram_destroy(p->dg);
    qgt_dev_free(p->rowmax_d);
    void* dev[] = {p->V, p->split, p->ops_d, p->ents_d, p->coef_desc_d, p->coef_d, p->theta_d, p->HG_d, p->part_d,
                   p->Q_d, p->grad_d, p->energy_d, p->natgrad_d, p->chol_work_d, p->status_d, p->slot_param_d,
                   p->param_ptr_d, p->param_slots_d};
    for (size_t i = 0; i < sizeof dev / sizeof dev[0]; i++) qgt_dev_free(dev[i]);
    void* pin[] = {p->theta_pin, p->Q_pin, p->grad_pin, p->natgrad_pin, p->energy_pin, p->status_pin};
    for (size_t i = 0; i < sizeof pin / sizeof pin[0]; i++) qgt_dev_host_free(pin[i]);
    qgt_dev_stream_destroy(p->stream);
    free(p->gates); free(p->passes); free(p->ops_h); free(p->ents_h); free(p->coef_h);
    free(p->slot_param_h); free(p->param_ptr_h); free(p->param_slots_h);
    free(p);
}

int qgt_plan_get_info(const qgt_plan_t* p, qgt_plan_info_t* info)
{
    if (!p || !info) return qgt_set_error(E_INVAL, "qgt_plan_get_info: NULL argument");
    memset(info, 0, sizeof *info);
    info->num_qubits = p->n;
    info->num_params = p->P;
    info->num_slots = p->nslots;
    info->num_rows = p->rows;
    info->num_passes = p->npasses;
    info->num_launches = p->launches;
    int tb = 0;
    for (int k = 0; k < p->npasses; k++) if (p->passes[k].tile_bits > tb) tb = p->passes[k].tile_bits;
    info->tile_bits = tb;
    info->vector_passes = p->vector_passes;
    info->gate_bytes = p->gate_bytes;
    info->gram_flops = (int64_t)4 * p->P * (p->P + 1) * p->N;
    info->device_bytes = p->device_bytes;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* execution                                                                 */
/* ------------------------------------------------------------------------ */

static int run_step(qgt_plan_t* p)
{
    int rc;
    int launches = 0;
    if ((rc = qgt_dev_prepare(p->coef_desc_d, p->ncoef, p->theta_d, p->coef_d, p->stream)) != 0) return rc;
    launches += p->ncoef > 0;
    if (p->dg && (rc = qgt_dev_memset(p->rowmax_d, 0, sizeof(uint32_t) * (size_t)p->rows, p->stream)) != 0) return rc;
    for (int k = 0; k < p->npasses; k++) {
        const spass_t* ps = &p->passes[k];
        qgt_dev_pass_args_t a;
        memset(&a, 0, sizeof a);
        a.V = p->V;
        a.N = p->N;
        a.ops = p->ops_d + ps->op_begin;
        a.nops = ps->op_count;
        a.entries = p->ents_d + ps->ent_begin;
        a.nentries = ps->ent_count;
        a.coef = p->coef_d;
        a.split = p->split;
        a.split_ld = p->split_ld;
        a.split_plane_stride = (int64_t)p->rows_pad * p->split_ld;
        a.split_scale = p->split_scale;
        a.split_bf16 = p->opt.precision == QGT_PRECISION_MIXED_BF16X3;
        a.n = p->n;
        a.tile_bits = ps->tile_bits;
        a.tile_mask = ps->tile_mask;
        memcpy(a.local_to_phys, ps->l2p, sizeof a.local_to_phys);
        a.rowmax = p->rowmax_d;
        if ((rc = qgt_dev_pass(&a, p->fp64, p->stream)) != 0) return rc;
        launches++;
    }
    if (p->npasses == 0) {
        /* no gates: psi = |0...0> written directly (row 0) */
        size_t ab = p->fp64 ? 16 : 8;
        double one[2] = {1.0, 0.0};
        float onef[2] = {1.0f, 0.0f};
        if ((rc = qgt_dev_memset(p->V, 0, (size_t)p->N * ab, p->stream)) != 0) return rc;
        if ((rc = qgt_dev_memcpy_h2d(p->V, p->fp64 ? (const void*)one : (const void*)onef, ab, p->stream)) != 0) return rc;
        if (!p->fp64) return qgt_set_error(E_INVAL, "mixed plan needs at least one gate");
    }
    const int has_h = p->opt.hamiltonian == QGT_HAMILTONIAN_TFIM;
    if (has_h) {
        size_t ab = p->fp64 ? 16 : 8;
        void* row1 = (char*)p->V + (size_t)p->N * ab;
        if ((rc = qgt_dev_tfim(p->V, row1, p->n, p->opt.tfim_J, p->opt.tfim_h, 1.0 / p->hscale, p->fp64,
                               p->split, p->split_ld, (int64_t)p->rows_pad * p->split_ld, 1, p->split_scale, 1,
                               p->rowmax_d ? p->rowmax_d + 1 : NULL, p->stream)) != 0)
            return rc;
        launches++;
    }
    if (p->fp64) {
        if ((rc = qgt_dev_gram_f64(p->V, p->N, p->rows, p->part_d, p->part_nsplit, p->HG_d, p->stream)) != 0) return rc;
    } else if (p->dg) {
        if ((rc = qgt_dev_dg_gram_run(p->dg, p->HG_d, p->stream)) != 0) return rc;
    } else {
        double s = (double)p->split_scale;
        if ((rc = qgt_dev_tc_gram_run(p->tc, 1.0 / (s * s), p->HG_d, p->stream)) != 0) return rc;
    }
    launches += 2;
    if (p->P > 0) {
        qgt_dev_post_args_t pa;
        memset(&pa, 0, sizeof pa);
        pa.HG = p->HG_d;
        pa.rows = p->rows;
        pa.P = p->P;
        pa.slot_param = p->slot_param_d;
        pa.param_ptr = p->param_ptr_d;
        pa.param_slots = p->param_slots_d;
        pa.hscale = p->hscale;
        pa.has_h = has_h;
        pa.Q = p->Q_d;
        pa.grad = p->grad_d;
        pa.energy = p->energy_d;
        if ((rc = qgt_dev_post(&pa, p->stream)) != 0) return rc;
        launches += 1 + has_h;
        if (has_h) {
            if ((rc = qgt_dev_cholesky(p->Q_d, 1, p->grad_d, p->P, p->opt.lambda, p->chol_work_d, p->natgrad_d,
                                       p->status_d, p->stream)) != 0)
                return rc;
            launches++;
        }
    }
    p->launches = launches;
    return 0;
}

static int launch_step(qgt_plan_t* p)
{
    int rc;
    if (p->graph) rc = qgt_dev_graph_launch(p->graph, p->stream);
    else rc = run_step(p);
    p->has_run = 1;
    return rc;
}

int qgt_plan_execute_device(qgt_plan_t* p, const double* theta_dev, double* Q_dev, double* grad_dev,
                            double* energy_dev, double* natgrad_dev)
{
    int rc;
    if (!p) return qgt_set_error(E_INVAL, "qgt_plan_execute_device: plan is NULL");
    if (p->P > 0 && theta_dev && theta_dev != p->theta_d)
        if ((rc = qgt_dev_memcpy_d2d(p->theta_d, theta_dev, sizeof(double) * (size_t)p->P, p->stream)) != 0) return rc;
    if ((rc = launch_step(p)) != 0) return rc;
    int has_h = p->opt.hamiltonian == QGT_HAMILTONIAN_TFIM;
    if (Q_dev && Q_dev != p->Q_d && (rc = qgt_dev_memcpy_d2d(Q_dev, p->Q_d, sizeof(double) * 2 * (size_t)p->P * p->P, p->stream)) != 0) return rc;
    if (has_h) {
        if (grad_dev && grad_dev != p->grad_d && (rc = qgt_dev_memcpy_d2d(grad_dev, p->grad_d, sizeof(double) * (size_t)p->P, p->stream)) != 0) return rc;
        if (energy_dev && energy_dev != p->energy_d && (rc = qgt_dev_memcpy_d2d(energy_dev, p->energy_d, sizeof(double), p->stream)) != 0) return rc;
        if (natgrad_dev && natgrad_dev != p->natgrad_d && (rc = qgt_dev_memcpy_d2d(natgrad_dev, p->natgrad_d, sizeof(double) * (size_t)p->P, p->stream)) != 0) return rc;
    }
    return 0;
}

int qgt_plan_execute_host(qgt_plan_t* p, const double* theta, double* Q, double* grad, double* energy, double* natgrad)
{
    int rc;
    if (!p) return qgt_set_error(E_INVAL, "qgt_plan_execute_host: plan is NULL");
    if (p->P > 0 && !theta) return qgt_set_error(E_INVAL, "qgt_plan_execute_host: theta is NULL");
    for (int k = 0; k < p->P; k++)
        if (!isfinite(theta[k])) return qgt_set_error(E_INVAL, "qgt_plan_execute_host: theta[%d] is not finite", k);
    int has_h = p->opt.hamiltonian == QGT_HAMILTONIAN_TFIM;
    if ((grad || energy || natgrad) && !has_h)
        return qgt_set_error(E_INVAL, "qgt_plan_execute_host: energy outputs need a Hamiltonian");
    if (p->P > 0) {
        memcpy(p->theta_pin, theta, sizeof(double) * (size_t)p->P);
        if ((rc = qgt_dev_memcpy_h2d(p->theta_d, p->theta_pin, sizeof(double) * (size_t)p->P, p->stream)) != 0) return rc;
    }
    if ((rc = launch_step(p)) != 0) return rc;
    if (Q && (rc = qgt_dev_memcpy_d2h(p->Q_pin, p->Q_d, sizeof(double) * 2 * (size_t)p->P * p->P, p->stream)) != 0) return rc;
    if (grad && (rc = qgt_dev_memcpy_d2h(p->grad_pin, p->grad_d, sizeof(double) * (size_t)p->P, p->stream)) != 0) return rc;
    if (energy && (rc = qgt_dev_memcpy_d2h(p->energy_pin, p->energy_d, sizeof(double), p->stream)) != 0) return rc;
    if (natgrad && (rc = qgt_dev_memcpy_d2h(p->natgrad_pin, p->natgrad_d, sizeof(double) * (size_t)p->P, p->stream)) != 0) return rc;
    if ((rc = qgt_dev_stream_sync(p->stream)) != 0) return rc;
    if (Q) memcpy(Q, p->Q_pin, sizeof(double) * 2 * (size_t)p->P * p->P);
    if (grad) memcpy(grad, p->grad_pin, sizeof(double) * (size_t)p->P);
    if (energy) *energy = p->energy_pin[0];
    if (natgrad) memcpy(natgrad, p->natgrad_pin, sizeof(double) * (size_t)p->P);
    if (p->tc || p->dg) {
        int st = p->tc ? qgt_dev_tc_gram_status(p->tc, p->stream) : qgt_dev_dg_gram_status(p->dg, p->stream);
        if (st) return qgt_set_error(st, "tensor-core Gram reported device status %d", st);
    }
    return 0;
}

int qgt_plan_synchronize(qgt_plan_t* p)
{
    if (!p) return qgt_set_error(E_INVAL, "qgt_plan_synchronize: plan is NULL");
    return qgt_dev_stream_sync(p->stream);
}

void* qgt_plan_stream(qgt_plan_t* p) { return p ? p->stream : NULL; }

int qgt_plan_get_state(qgt_plan_t* p, double* psi)
{
    if (!p || !psi) return qgt_set_error(E_INVAL, "qgt_plan_get_state: NULL argument");
    if (!p->has_run) return qgt_set_error(E_STATE, "qgt_plan_get_state: no step has run");
    int rc;
    if (p->fp64) {
        if ((rc = qgt_dev_memcpy_d2h(psi, p->V, sizeof(double) * 2 * (size_t)p->N, p->stream)) != 0) return rc;
        return qgt_dev_stream_sync(p->stream);
    }
    float* tmp = (float*)malloc(sizeof(float) * 2 * (size_t)p->N);
    if (!tmp) return qgt_set_error(E_NOMEM, "qgt_plan_get_state: oom");
    rc = qgt_dev_memcpy_d2h(tmp, p->V, sizeof(float) * 2 * (size_t)p->N, p->stream);
    if (!rc) rc = qgt_dev_stream_sync(p->stream);
    if (!rc) for (int64_t i = 0; i < 2 * p->N; i++) psi[i] = tmp[i];
    free(tmp);
    return rc;
}

/* row r of V (0 psi, 1 H psi / hscale, 2 + s slot s) as complex doubles; only
 * valid for FP64 plans and for slots of mixed plans before the last pass. */
int qgt_plan_get_row(qgt_plan_t* p, int row, double* out)
{
    if (!p || !out || row < 0 || row >= p->rows) return qgt_set_error(E_INVAL, "qgt_plan_get_row: bad argument");
    if (!p->fp64) return qgt_set_error(E_STATE, "qgt_plan_get_row: derivative rows are kept only by FP64 plans");
    int rc = qgt_dev_memcpy_d2h(out, (char*)p->V + (size_t)row * p->N * 16, sizeof(double) * 2 * (size_t)p->N, p->stream);
    if (!rc) rc = qgt_dev_stream_sync(p->stream);
    return rc;
}

int qgt_plan_device_status(qgt_plan_t* p, double* lambda_used)
{
    if (!p) return qgt_set_error(E_INVAL, "qgt_plan_device_status: plan is NULL");
    int rc = qgt_dev_memcpy_d2h(p->status_pin, p->status_d, sizeof(double) * 2, p->stream);
    if (!rc) rc = qgt_dev_stream_sync(p->stream);
    if (rc) return rc;
    if (lambda_used) *lambda_used = p->status_pin[1];
    int st = (int)p->status_pin[0];
    if (!st && p->tc) st = qgt_dev_tc_gram_status(p->tc, p->stream);
    if (!st && p->dg) st = qgt_dev_dg_gram_status(p->dg, p->stream);
    return st;
}

int qgt_compute_qgt_f64(const qgt_circuit_desc_t* c, const double* theta, double* Q, qgt_precision_t prec)
{
    qgt_plan_options_t o;
    qgt_plan_default_options(&o);
    o.precision = prec;
    o.hamiltonian = QGT_HAMILTONIAN_NONE;
    qgt_plan_t* p = NULL;
    int rc = qgt_plan_create(c, &o, &p);
    if (rc) return rc;
    rc = qgt_plan_execute_host(p, theta, Q, NULL, NULL, NULL);
    qgt_plan_destroy(p);
    return rc;
}

int qgt_natgrad_step_f64(const qgt_circuit_desc_t* c, const double* theta, const qgt_plan_options_t* opt, double* Q,
                         double* grad, double* energy, double* natgrad)
{
    qgt_plan_t* p = NULL;
    int rc = qgt_plan_create(c, opt, &p);
    if (rc) return rc;
    rc = qgt_plan_execute_host(p, theta, Q, grad, energy, natgrad);
    if (!rc) {
        double lam;
        int st = qgt_plan_device_status(p, &lam);
        if (st) rc = qgt_set_error(st, "natural-gradient solve failed (status %d, lambda %g)", st, lam);
    }
    qgt_plan_destroy(p);
    return rc;
}

int qgt_cholesky_solve_f64(const double* A, const double* g, double lambda, int32_t P, double* x, double* lambda_used)
{
    if (!A || !g || !x || P <= 0) return qgt_set_error(E_INVAL, "qgt_cholesky_solve_f64: bad argument");
    void* s = NULL;
    double *Ad = NULL, *gd = NULL, *xd = NULL, *wd = NULL, *sd = NULL;
    double st[2] = {0, 0};
    int rc = qgt_dev_stream_create(&s);
    if (!rc) rc = qgt_dev_malloc((void**)&Ad, sizeof(double) * (size_t)P * P);
    if (!rc) rc = qgt_dev_malloc((void**)&gd, sizeof(double) * (size_t)P);
    if (!rc) rc = qgt_dev_malloc((void**)&xd, sizeof(double) * (size_t)P);
    if (!rc) rc = qgt_dev_malloc((void**)&wd, sizeof(double) * (size_t)P * P);
    if (!rc) rc = qgt_dev_malloc((void**)&sd, sizeof(double) * 2);
    if (!rc) rc = qgt_dev_memcpy_h2d(Ad, A, sizeof(double) * (size_t)P * P, s);
    if (!rc) rc = qgt_dev_memcpy_h2d(gd, g, sizeof(double) * (size_t)P, s);
    if (!rc) rc = qgt_dev_cholesky(Ad, 0, gd, P, lambda, wd, xd, sd, s);
    if (!rc) rc = qgt_dev_memcpy_d2h(x, xd, sizeof(double) * (size_t)P, s);
    if (!rc) rc = qgt_dev_memcpy_d2h(st, sd, sizeof(double) * 2, s);
    if (!rc) rc = qgt_dev_stream_sync(s);
    qgt_dev_free(Ad); qgt_dev_free(gd); qgt_dev_free(xd); qgt_dev_free(wd); qgt_dev_free(sd);
    if (s) qgt_dev_stream_destroy(s);
    if (rc) return rc;
    if (lambda_used) *lambda_used = st[1];
    if ((int)st[0]) return qgt_set_error((int)st[0], "cholesky: matrix not positive definite after lambda retries");
    return 0;
}

/* out = sum_s c[s] d_s over the derivative slots of an FP64 plan (2^n complex, host) */
int qgt_plan_combine_slots(qgt_plan_t* p, const double* c, double* out)
{
    if (!p || !c || !out) return qgt_set_error(E_INVAL, "qgt_plan_combine_slots: bad argument");
    if (!p->fp64) return qgt_set_error(E_STATE, "qgt_plan_combine_slots: FP64 plans only");
    if (p->nslots == 0) { memset(out, 0, sizeof(double) * 2 * (size_t)p->N); return 0; }
    double *cd = NULL, *od = NULL;
    int rc = qgt_dev_malloc((void**)&cd, sizeof(double) * (size_t)p->nslots);
    if (!rc) rc = qgt_dev_malloc((void**)&od, sizeof(double) * 2 * (size_t)p->N);
    if (!rc) rc = qgt_dev_memcpy_h2d(cd, c, sizeof(double) * (size_t)p->nslots, p->stream);
    if (!rc) rc = qgt_dev_combine_rows(p->V, p->N, 2, cd, p->nslots, od, p->stream);
    if (!rc) rc = qgt_dev_memcpy_d2h(out, od, sizeof(double) * 2 * (size_t)p->N, p->stream);
    if (!rc) rc = qgt_dev_stream_sync(p->stream);
    qgt_dev_free(cd);
    qgt_dev_free(od);
    return rc;
}
