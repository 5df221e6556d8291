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
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../qgt_internal.h"
#include "qgt_gb300.h"

#define E_INVAL (-1)
#define E_NOMEM (-2)
#define E_STATE (-4)
#define E_HW (-6)

/* role encoding of register-resident programs (see qgt_dev_op2_t) */
#define QGT_CKPT_GROUPS 32
#define RL_REG_ 8
#define RL_WARP_ 16
#define RL_OUT_ 32

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
    int part;                     /* 0 forward (with first-half slots); meet in the middle: 1 psi forward, 2 backward */
    int op_begin, op_count;
    int ent_begin, ent_count;
    /* segment checkpoints (build_checkpoints): entry 0 writes them (launched first, alone); the
     * entries [grp_begin[g], + grp_count[g]) start at op grp_start[g] (a Q2_SEG) from checkpoint g */
    int ckpt_writer;
    int ngrp;
    int grp_begin[QGT_CKPT_GROUPS], grp_count[QGT_CKPT_GROUPS], grp_start[QGT_CKPT_GROUPS];
    int prog_begin, prog_count;   /* register-resident program (full tiles), 0 = v1 pass */
    int tile_bits;
    uint32_t tile_mask;
    int8_t l2p[16];
    qgt_jit_kernel_t* jit[2];     /* the pass program as straight-line kernels: [0] entries, [1] checkpoint writer */
} spass_t;

struct qgt_plan {
    qgt_plan_options_t opt;
    int n, P, nslots, rows, rows_pad;
    int B;                        /* parameter points per step (theta batch) */
    /* meet in the middle: gates [0, cut) forward with their slots, psi alone
     * through [cut, G), then [cut, G) backward (inverse gates) with the
     * second-half slots; part_begin[] delimits the three parts in `gates` */
    int mitm, cut, nparts, early_slots, row_T, orig_ngates;
    int* op_gate;                 /* gate (index into gates) of each op */
    /* combined phase entries of diagonal runs: entry ncoef + k = product of
     * comb_src[comb_ptr[k] .. comb_ptr[k+1]) (formed per step on the device) */
    int ncomb, comb_nsrc;
    int32_t *comb_ptr_h, *comb_src_h, *comb_ptr_d, *comb_src_d;
    int host_only;                /* schedule only (no device resources): qgt_plan_schedule_dump */
    int part_begin[4];
    /* amplitude-scale bookkeeping of meet in the middle (complex64 gates are
     * not exactly unitary): group m = the coefficient entries of psi-forward
     * pass m and of its mirror; rho[m] = product of their scales over groups
     * 0..m; a row carried through groups 0..m (row_group = m) is divided by it */
    int nscale_groups;
    int32_t *scale_ptr_h, *scale_src_h, *row_group_h;
    int32_t *scale_ptr_d, *scale_src_d, *row_group_d;
    /* pass renormalisation (complex64 programs): per pass its coefficient entries and the entry scaled by 1 / G */
    int32_t *ren_ptr_h, *ren_src_h, *ren_h;
    int32_t *ren_ptr_d, *ren_src_d, *ren_d;
    double* rho_d;
    int Pd;                       /* parameters [0, Pd) get derivative rows; Q is Pd x Pd */
    int64_t pstride;              /* amplitudes between points in V: (rows + 1) N */
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
    void* graph;                  /* the step up to Q, grad and energy (run_head) */
    void* graph_solve;            /* its natural-gradient solve (run_solve); NULL when there is none */
    /* passes with a checkpoint writer fork onto aux_stream (the writer, then the spawns that start
     * from its checkpoints) while the other entries run on stream; joined at the pass end */
    void* aux_stream;
    void* ev_fork;
    void* ev_join;
    /* host outputs: Q, grad and energy are final after the post kernels, before the solve;
     * qgt_plan_execute_host records ev_post between the two graphs and copies them on copy_stream
     * and into the caller's buffers while the solve still runs */
    void* copy_stream;
    void* ev_post;
    void* ev_copied;
    void* V;
    void* split;
    qgt_dev_op_t* ops_d;
    qgt_dev_entry_t* ents_d;
    qgt_dev_op2_t* prog_h;
    int nprog;
    int8_t* segs_h;
    int nsegs;
    qgt_dev_op2_t* prog_d;
    int8_t* segs_d;
    float* coef32_d;
    qgt_dev_coef_desc_t* coef_desc_d;
    double* coef_d;
    double* theta_d;
    double* HG_d;
    double* part_d;
    int part_nsplit;
    qgt_tc_gram_t* tc;            /* split-BF16 x3 Gram (operands written by the last pass) */
    qgt_dg_gram_t* dg;            /* integer-digit FP16 Gram (mixed default) */
    double* small_part_d;         /* partials of the small Gram (rows <= 8) */
    qgt_dev_pauli_term_t* pauli_h; /* Pauli-sum Hamiltonian terms (host / device) */
    qgt_dev_pauli_term_t* pauli_d;
    int npauli;
    int small_nsplit;
    uint32_t* rowmax_d;           /* per-row max |amplitude| (float bits) for the digit Gram */
    double *Q_d, *grad_d, *energy_d, *natgrad_d, *chol_work_d, *status_d;
    int32_t *slot_param_d, *param_ptr_d, *param_slots_d;
    /* pinned host staging */
    double *theta_pin, *Q_pin, *grad_pin, *energy_pin, *natgrad_pin, *status_pin;
    int* gerr_pin;                /* the tensor-core Gram's error flag, copied with the outputs */
    double hscale;
    float split_scale;
    int64_t device_bytes;
    int64_t vector_passes, gate_bytes;
    int wide;                     /* complex64 passes on 14-bit tiles (choose_tile) */
    int njit;                     /* passes running as compiled straight-line kernels */
    int launches;
    int has_run;
    void* prof_ev[7];             /* phase events of qgt_plan_profile_step (NULL otherwise) */
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

/* Backward part of meet in the middle: the psi-forward passes (part 1) in
 * reverse order, each with its ops reversed and every gate replaced by its
 * inverse (the coefficient entry of the matching part-2 gate, which also
 * carries the gate's derivative slot).  A pass and its mirror share the tile
 * set, so backward pass j starts exactly where forward pass nP-1-j ended and
 * can spawn from psi as the forward pass left it. */
static int mirror_backward_passes(qgt_plan_t* p)
{
    const int c = p->cut, G = p->orig_ngates, L2 = G - c;
    int nP = 0;
    for (int k = 0; k < p->npasses; k++) nP += p->passes[k].part == 1;
    spass_t* np2 = (spass_t*)realloc(p->passes, sizeof(spass_t) * (size_t)(p->npasses + nP + 1));
    if (!np2) return qgt_set_error(E_NOMEM, "schedule: oom");
    p->passes = np2;
    int extra = 0;
    for (int k = 0; k < p->npasses; k++) if (p->passes[k].part == 1) extra += p->passes[k].op_count;
    qgt_dev_op_t* nops = (qgt_dev_op_t*)realloc(p->ops_h, sizeof(qgt_dev_op_t) * (size_t)(p->nops + extra + 1));
    int* ng = (int*)realloc(p->op_gate, sizeof(int) * (size_t)(p->nops + extra + 1));
    if (nops) p->ops_h = nops;
    if (ng) p->op_gate = ng;
    if (!nops || !ng) return qgt_set_error(E_NOMEM, "schedule: oom");
    const int np = p->npasses;
    for (int k = np - 1; k >= 0; k--) {
        const spass_t* src = &p->passes[k];
        if (src->part != 1) continue;
        spass_t* ps = &p->passes[p->npasses++];
        *ps = *src;
        ps->part = 2;
        ps->op_begin = p->nops;
        for (int j = src->op_count - 1; j >= 0; j--) {
            const int si = src->op_begin + j;
            const int g = p->op_gate[si];                 /* forward copy of original gate g, c <= g < G */
            const int bg = c + L2 + (G - 1 - g);          /* its inverse in part 2 */
            const sgate_t* bgate = &p->gates[bg];
            qgt_dev_op_t op = p->ops_h[si];
            op.coef = bgate->coef;
            op.slot = bgate->slot;
            op.gen = QGEN_NONE;
            if (bgate->slot >= 0)
                op.gen = bgate->type == QGT_GATE_RX ? QGEN_X : (bgate->type == QGT_GATE_RY ? QGEN_Y : QGEN_Z);
            p->op_gate[p->nops] = bg;
            p->ops_h[p->nops++] = op;
        }
        ps->op_count = p->nops - ps->op_begin;
    }
    return 0;
}

/* width of a full register-resident tile: complex128 12 bits; complex64 13 bits, or 14 when
 * choose_tile found that they save vector passes */
static int full_tile_bits(const qgt_plan_t* p)
{
    if (p->fp64) return QGT_TILE_MAX_F64;
    if (p->n == QGT_TILE_MAX_F64) return QGT_TILE_MAX_F64;   /* 12 qubits: one 12-bit tile, 16 registers */
    return p->wide ? QGT_TILE_WIDE_F32 : QGT_TILE_MAX_F32;
}

/* register bits of the plan's register-resident tiles: 4 for complex128, for 12-bit complex64
 * tiles and for 13- / 14-bit tiles with thread_amps = 16 (compiled kernels only), 5 otherwise */
static int amps16(const qgt_plan_t* p)
{
    const int tb = full_tile_bits(p);
    return p->opt.precision == QGT_PRECISION_MIXED && p->opt.thread_amps == 16 &&
           (tb == QGT_TILE_MAX_F32 || tb == QGT_TILE_WIDE_F32);
}

static int reg_bits(const qgt_plan_t* p)
{
    if (amps16(p)) return 4;   /* 512 threads on 13-qubit tiles, 1024 on 14 */
    return (p->fp64 || full_tile_bits(p) == QGT_TILE_MAX_F64) ? 4 : 5;
}

static int compile_schedule(qgt_plan_t* p)
{
    const int n = p->n, G = p->ngates;
    const int tmax = n < full_tile_bits(p) ? n : full_tile_bits(p);
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
    int nord = 0, np = 0;
    /* with meet in the middle the backward part mirrors the psi-forward passes
     * (mirror_backward_passes), so only the first two parts are scheduled here */
    const int sched_parts = p->mitm ? 2 : p->nparts;
    free(p->op_gate);
    p->op_gate = (int*)calloc((size_t)G + 1, sizeof(int));
    if (!p->op_gate) { free(placed); free(blocked); free(order); return qgt_set_error(E_NOMEM, "schedule: oom"); }
    for (int part = 0; part < sched_parts; part++) {
    const int g0 = p->part_begin[part], g1 = p->part_begin[part + 1];
    int remaining = 0;
    for (int g = g0; g < g1; g++) {
        if (p->gates[g].type == QGT_GATE_I && p->gates[g].slot < 0) placed[g] = 1;
        else remaining++;
    }
    int first = g0;
    while (remaining > 0) {
        uint32_t S = (lane >= 32) ? 0xffffffffu : ((1u << lane) - 1u);
        int nb = 0, start = nord;
        while (first < g1 && placed[first]) first++;
        for (int g = first; g < g1; g++) {
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
        ps->part = part;
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
            p->op_gate[k] = order[k];
            memset(op, 0, sizeof *op);
            op->q = (int8_t)g->q0;
            op->q2 = (int8_t)(g->q1 >= 0 ? g->q1 : 0);
            op->lb = p2l[g->q0];
            op->lb2 = g->q1 >= 0 ? p2l[g->q1] : -1;
            op->coef = g->coef;
            op->slot = g->slot;
            op->pad = (int16_t)g->type;
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
    }
    p->npasses = np;
    p->nops = nord;
    free(placed);
    free(blocked);
    free(order);
    return p->mitm ? mirror_backward_passes(p) : 0;
}

static int build_entries(qgt_plan_t* p);
static int build_entries_mitm(qgt_plan_t* p);

static void free_schedule(qgt_plan_t* p)
{
    free(p->passes); free(p->ops_h); free(p->ents_h);
    free(p->scale_ptr_h); free(p->scale_src_h); free(p->row_group_h);
    p->passes = NULL; p->ops_h = NULL; p->ents_h = NULL;
    p->scale_ptr_h = NULL; p->scale_src_h = NULL; p->row_group_h = NULL;
}

/* complex64 plans of 14 or more qubits: 14-bit tiles (512-thread CTAs, one per SM) when their
 * schedule needs sufficiently fewer vector passes than 13-bit tiles (two 256-thread CTAs per SM).
 * A vector pass costs about 8 % more on the wide tile with the program interpreter and about
 * 55 % more with compiled kernels (20 qubits, 8 layers: 486 wide vector passes took 4.9 ms, 649
 * narrow ones 4.1 ms: two CTAs per SM overlap one tile's loads with the other's gates), so the wide
 * tile needs 8 % fewer vector passes with the interpreter and 36 % fewer with compiled kernels. */
static int jit_wanted(const qgt_plan_t* p);

static int choose_tile(qgt_plan_t* p)
{
    p->wide = 0;
    if (p->fp64 || p->n < QGT_TILE_WIDE_F32) return 0;
    if (p->opt.tile_bits == QGT_TILE_MAX_F32) return 0;
    if (p->opt.tile_bits == QGT_TILE_WIDE_F32) { p->wide = 1; return 0; }
    int64_t vp[2];
    for (int w = 1; w >= 0; w--) {
        p->wide = w;
        int rc = compile_schedule(p);
        if (!rc) rc = p->mitm ? build_entries_mitm(p) : build_entries(p);
        vp[w] = p->vector_passes;
        free_schedule(p);
        if (rc) return rc;
    }
    p->wide = 100 * vp[1] <= (jit_wanted(p) ? 64 : 92) * vp[0];
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
    const int rmax = (p->opt.precision == QGT_PRECISION_MIXED && !p->small_nsplit) ? QENT_ROWMAX : 0;
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

/* Transport choice.  Meet in the middle: with S slots numbered in gate
 * order, the cut is the gate of slot S/2.  The gate list becomes three parts:
 *   F  gates [0, cut) with slots 0 .. S/2-1 (carried forward to the cut),
 *   P  gates [cut, G) on psi alone (psi(G) for H psi),
 *   B  gates G-1 .. cut as inverses, slots S/2 .. S-1 spawned on the way
 *      (psi(k-) = U^dagger psi(G) before gate k; (-i/2) G_k psi(k-) carried
 *      backward to the cut), together with H psi carried backward.
 * Every Gram entry is then taken at the cut; <U a|U b> = <a|b> leaves Q,
 * the energy and the gradient unchanged. */
static int setup_transport(qgt_plan_t* p)
{
    p->nparts = 1;
    p->part_begin[0] = 0;
    p->part_begin[1] = p->ngates;
    p->orig_ngates = p->ngates;
    p->mitm = 0;
    const int want = p->opt.transport;
    if (want < QGT_TRANSPORT_AUTO || want > QGT_TRANSPORT_MEET)
        return qgt_set_error(E_INVAL, "qgt_plan_create: unknown transport %d", want);
    if (want == QGT_TRANSPORT_MEET && p->opt.precision == QGT_PRECISION_MIXED_BF16X3)
        return qgt_set_error(E_INVAL, "qgt_plan_create: meet-in-the-middle transport needs FP64 or MIXED precision");
    p->mitm = (want == QGT_TRANSPORT_MEET) ||
              (want == QGT_TRANSPORT_AUTO && p->opt.precision == QGT_PRECISION_MIXED && p->nslots >= 16);
    if (p->nslots < 2) p->mitm = 0;
    if (!p->mitm) return 0;
    const int G = p->ngates, half = p->nslots / 2;
    int c = -1;
    for (int g = 0; g < G && c < 0; g++)
        if (p->gates[g].slot == half) c = g;
    if (c <= 0) { p->mitm = 0; return 0; }
    const int L2 = G - c;
    sgate_t* ext = (sgate_t*)calloc((size_t)(c + 2 * L2) + 1, sizeof(sgate_t));
    qgt_dev_coef_desc_t* nc = (qgt_dev_coef_desc_t*)realloc(p->coef_h, sizeof(qgt_dev_coef_desc_t) * ((size_t)p->ncoef + L2 + 1));
    if (nc) p->coef_h = nc;
    if (!ext || !nc) { free(ext); return qgt_set_error(E_NOMEM, "transport: out of memory"); }
    int nl = 0;
    for (int g = 0; g < c; g++) ext[g] = p->gates[g];
    for (int g = c; g < G; g++) {
        ext[g] = p->gates[g];
        ext[g].slot = -1;
    }
    for (int k = 0; k < L2; k++) {
        sgate_t e = p->gates[G - 1 - k];
        if (e.coef >= 0) {
            const int ni = p->ncoef++;
            p->coef_h[ni] = p->coef_h[e.coef];
            p->coef_h[ni].type |= QGT_COEF_INVERSE;
            e.coef = ni;
        }
        ext[c + L2 + k] = e;
    }
    free(p->gates);
    p->gates = ext;
    p->ngates = c + 2 * L2;
    p->nparts = 3;
    p->part_begin[0] = 0;
    p->part_begin[1] = c;
    p->part_begin[2] = c + L2;
    p->part_begin[3] = c + 2 * L2;
    p->cut = c;
    p->early_slots = half;
    (void)nl;
    p->pstride = (int64_t)(p->rows + 2) * p->N;   /* final value set with the entries (psi checkpoints) */
    return 0;
}

static int add_entry(qgt_plan_t* p, int* cap, const qgt_dev_entry_t* e)
{
    if (p->nents >= *cap) {
        int nc = *cap * 2;
        qgt_dev_entry_t* ne = (qgt_dev_entry_t*)realloc(p->ents_h, sizeof(qgt_dev_entry_t) * (size_t)nc);
        if (!ne) return qgt_set_error(E_NOMEM, "entries: oom");
        p->ents_h = ne;
        *cap = nc;
    }
    p->ents_h[p->nents++] = *e;
    const int64_t ab = p->fp64 ? 16 : 8;
    p->gate_bytes += ab * p->N * ((e->flags & QENT_SRC_ZERO) ? 1 : 2);
    return 0;
}

/* entries of the three meet-in-the-middle parts (see setup_transport):
 * rows 0 psi(cut), 1 H psi carried to the cut, 2 + s slot s at the cut;
 * row `rows` is psi's second buffer in the forward part, rows + 1 + m holds
 * psi after psi-forward pass m (the start of its mirrored backward pass) */
static int build_entries_mitm(qgt_plan_t* p)
{
    int cap = 64, rc = 0;
    p->nents = 0;
    p->ents_h = (qgt_dev_entry_t*)malloc(sizeof(qgt_dev_entry_t) * (size_t)cap);
    char* live = (char*)calloc((size_t)p->nslots + 1, 1);
    if (!p->ents_h || !live) { free(live); return qgt_set_error(E_NOMEM, "entries: oom"); }
    const int rmax = (p->opt.precision == QGT_PRECISION_MIXED && !p->small_nsplit) ? QENT_ROWMAX : 0;
    const int has_h = p->opt.hamiltonian != QGT_HAMILTONIAN_NONE;
    const int RA = p->rows;
    int nf = 0, nP = 0, nb = 0;
    for (int k = 0; k < p->npasses; k++) {
        nf += p->passes[k].part == 0;
        nP += p->passes[k].part == 1;
        nb += p->passes[k].part == 2;
    }
    p->pstride = (int64_t)(p->rows + 1 + nP) * p->N;
    p->vector_passes = 0;
    p->gate_bytes = 0;
    int fi = 0, pi = 0, bi = 0;
    for (int k = 0; k < p->npasses && !rc; k++) {
        spass_t* ps = &p->passes[k];
        ps->ent_begin = p->nents;
        qgt_dev_entry_t e;
        if (ps->part == 0) {
            const int last = (fi == nf - 1);
            const int dst = ((nf - 1 - fi) % 2 == 0) ? 0 : RA;
            const int src = (fi == 0) ? -1 : (((nf - fi) % 2 == 0) ? 0 : RA);
            memset(&e, 0, sizeof e);
            e.src_row = src < 0 ? 0 : src;
            e.dst_row = dst;
            e.spawn_op = -1;
            e.flags = QENT_STORE_V | (src < 0 ? QENT_SRC_ZERO : 0) | (last ? rmax : 0);
            rc = add_entry(p, &cap, &e);
            for (int s = 0; s < p->nslots && !rc; s++) {
                if (!live[s]) continue;
                memset(&e, 0, sizeof e);
                e.src_row = e.dst_row = 2 + s;
                e.spawn_op = -1;
                e.flags = QENT_STORE_V | (last ? rmax : 0);
                rc = add_entry(p, &cap, &e);
            }
            for (int j = 0; j < ps->op_count && !rc; j++) {
                const qgt_dev_op_t* op = &p->ops_h[ps->op_begin + j];
                if (op->slot < 0) continue;
                memset(&e, 0, sizeof e);
                e.src_row = src < 0 ? 0 : src;
                e.dst_row = 2 + op->slot;
                e.spawn_op = j;
                e.flags = QENT_STORE_V | (src < 0 ? QENT_SRC_ZERO : 0) | (last ? rmax : 0);
                rc = add_entry(p, &cap, &e);
            }
            fi++;
        } else if (ps->part == 1) {
            memset(&e, 0, sizeof e);
            e.src_row = (pi == 0) ? 0 : p->rows + pi;
            e.dst_row = p->rows + 1 + pi;
            e.spawn_op = -1;
            e.flags = QENT_STORE_V;
            rc = add_entry(p, &cap, &e);
            p->row_T = e.dst_row;
            pi++;
        } else {
            const int last = (bi == nb - 1);
            const int src = p->rows + 1 + (nP - 1 - bi);   /* psi where the mirrored forward pass ended */
            if (has_h) {
                memset(&e, 0, sizeof e);
                e.src_row = e.dst_row = 1;
                e.spawn_op = -1;
                e.flags = QENT_STORE_V | (last ? rmax : 0);
                rc = add_entry(p, &cap, &e);
            }
            for (int s = p->early_slots; s < p->nslots && !rc; s++) {   /* first-half slots stay at the cut */
                if (!live[s]) continue;
                memset(&e, 0, sizeof e);
                e.src_row = e.dst_row = 2 + s;
                e.spawn_op = -1;
                e.flags = QENT_STORE_V | (last ? rmax : 0);
                rc = add_entry(p, &cap, &e);
            }
            for (int j = 0; j < ps->op_count && !rc; j++) {
                const qgt_dev_op_t* op = &p->ops_h[ps->op_begin + j];
                if (op->slot < 0) continue;
                memset(&e, 0, sizeof e);
                e.src_row = src;
                e.dst_row = 2 + op->slot;
                e.spawn_op = j;
                e.flags = QENT_STORE_V | (last ? rmax : 0);
                rc = add_entry(p, &cap, &e);
            }
            bi++;
        }
        for (int j = 0; j < ps->op_count; j++) {
            const qgt_dev_op_t* op = &p->ops_h[ps->op_begin + j];
            if (op->slot >= 0) live[op->slot] = 1;
        }
        ps->ent_count = p->nents - ps->ent_begin;
        if (!rc && ps->ent_count > 65535) rc = qgt_set_error(E_INVAL, "pass has more than 65535 vectors");
        p->vector_passes += ps->ent_count;
    }
    free(live);
    if (rc) return rc;
    /* scale groups: psi-forward pass m and backward pass nP-1-m (its mirror) */
    p->nscale_groups = nP;
    p->scale_ptr_h = (int32_t*)calloc((size_t)nP + 1, sizeof(int32_t));
    p->scale_src_h = (int32_t*)malloc(sizeof(int32_t) * ((size_t)p->nops + 1));
    p->row_group_h = (int32_t*)malloc(sizeof(int32_t) * ((size_t)p->rows + 1));
    if (!p->scale_ptr_h || !p->scale_src_h || !p->row_group_h) return qgt_set_error(E_NOMEM, "entries: oom");
    int ns = 0, m = 0, bj = 0;
    int* pk = (int*)malloc(sizeof(int) * ((size_t)nP + 1));
    int* bk = (int*)malloc(sizeof(int) * ((size_t)nP + 1));
    if (!pk || !bk) { free(pk); free(bk); return qgt_set_error(E_NOMEM, "entries: oom"); }
    for (int k = 0; k < p->npasses; k++) {
        if (p->passes[k].part == 1) pk[m++] = k;
        if (p->passes[k].part == 2) bk[bj++] = k;
    }
    for (m = 0; m < nP; m++) {
        const spass_t* a = &p->passes[pk[m]];
        const spass_t* bpass = &p->passes[bk[nP - 1 - m]];
        for (int j = 0; j < a->op_count; j++)
            if (p->ops_h[a->op_begin + j].coef >= 0) p->scale_src_h[ns++] = p->ops_h[a->op_begin + j].coef;
        for (int j = 0; j < bpass->op_count; j++)
            if (p->ops_h[bpass->op_begin + j].coef >= 0) p->scale_src_h[ns++] = p->ops_h[bpass->op_begin + j].coef;
        p->scale_ptr_h[m + 1] = ns;
    }
    /* rows: psi(cut) and first-half slots none; H psi all groups; a second-half
     * slot spawned in backward pass j crosses groups 0 .. nP-1-j */
    for (int r = 0; r < p->rows; r++) p->row_group_h[r] = -1;
    if (has_h) p->row_group_h[1] = nP - 1;
    for (int j = 0; j < nb; j++) {
        const spass_t* ps = &p->passes[bk[j]];
        for (int t = 0; t < ps->op_count; t++) {
            const int sl = p->ops_h[ps->op_begin + t].slot;
            if (sl >= 0) p->row_group_h[2 + sl] = nP - 1 - j;
        }
    }
    free(pk);
    free(bk);
    return 0;
}

/* Register-resident programs for passes whose tile has the full width
 * (13 or 14 bits complex64 / 12 bits complex128).  Lanes are local bits 0..4;
 * the other local bits are split into RB register bits and 3 (or 4) warp bits per
 * segment.  A gate whose target is a warp bit opens a new segment whose
 * register bits are the next distinct targets (looking ahead), so that the
 * shared-memory re-layouts are few.  SWAP becomes three CNOTs. */
static int build_programs(qgt_plan_t* p)
{
    const int tb = full_tile_bits(p);
    const int RB = reg_bits(p);
    int cap = 3 * p->nops + 2 * p->npasses + 16, scap = 2 * p->nops + p->npasses + 16;
    p->prog_h = (qgt_dev_op2_t*)calloc((size_t)cap, sizeof(qgt_dev_op2_t));
    p->segs_h = (int8_t*)calloc((size_t)scap * 16, 1);
    int* remap = (int*)malloc(sizeof(int) * ((size_t)p->nops + 1));
    if (!p->prog_h || !p->segs_h || !remap) { free(remap); return qgt_set_error(E_NOMEM, "programs: oom"); }
    p->nprog = 0;
    p->nsegs = 0;
    for (int k = 0; k < p->npasses; k++) {
        spass_t* ps = &p->passes[k];
        ps->prog_begin = p->nprog;
        ps->prog_count = 0;
        if (ps->tile_bits != tb || p->n < tb) continue;
        const qgt_dev_op_t* ops = p->ops_h + ps->op_begin;
        const int no = ps->op_count;
        /* expanded op list: SWAP -> 3 CNOTs (target local bit, control local bit) */
        int role[32];
        int regs[8];
        int nreg = 0;
        /* first layout: the first RB distinct non-lane targets */
        #define NEEDBIT(o) (((o)->kind == QOP_1Q || (o)->kind == QOP_CNOT) ? (o)->lb : ((o)->kind == QOP_SWAP ? (o)->lb : -1))
        int cur_op = 0;
        int first = 1;
        while (1) {
            /* choose the register bits for a segment starting at op cur_op */
            int chosen[8], nc = 0;
            for (int j = cur_op; j < no && nc < RB; j++) {
                int cands[2] = {NEEDBIT(&ops[j]), ops[j].kind == QOP_SWAP ? ops[j].lb2 : -1};
                for (int c = 0; c < 2; c++) {
                    int b = cands[c];
                    if (b < QGT_LANE_BITS || nc >= RB) continue;
                    int dup = 0;
                    for (int t = 0; t < nc; t++) dup |= chosen[t] == b;
                    if (!dup) chosen[nc++] = b;
                }
            }
            /* keep previous register bits to fill up, then the lowest free bits */
            for (int t = 0; t < nreg && nc < RB; t++) {
                int dup = 0;
                for (int u = 0; u < nc; u++) dup |= chosen[u] == regs[t];
                if (!dup) chosen[nc++] = regs[t];
            }
            for (int b = QGT_LANE_BITS; b < tb && nc < RB; b++) {
                int dup = 0;
                for (int u = 0; u < nc; u++) dup |= chosen[u] == b;
                if (!dup) chosen[nc++] = b;
            }
            nreg = nc;
            for (int t = 0; t < nc; t++) regs[t] = chosen[t];
            if (p->nsegs >= scap || p->nprog + 4 >= cap) { free(remap); return qgt_set_error(E_STATE, "programs: capacity"); }
            int8_t* L = p->segs_h + 16 * p->nsegs;
            for (int b = 0; b < 32; b++) role[b] = -1;
            for (int b = 0; b < QGT_LANE_BITS; b++) role[b] = b;
            for (int t = 0; t < RB; t++) { L[t] = (int8_t)regs[t]; role[regs[t]] = RL_REG_ + t; }
            int w = 0;
            for (int b = QGT_LANE_BITS; b < tb; b++)
                if (role[b] < 0) { L[8 + w] = (int8_t)b; role[b] = RL_WARP_ + w; w++; }
            qgt_dev_op2_t* so = &p->prog_h[p->nprog++];
            memset(so, 0, sizeof *so);
            so->kind = Q2_SEG;
            so->seg = (int16_t)p->nsegs++;
            first = 0;
            /* emit ops until one needs a warp bit */
            int j = cur_op;
            for (; j < no; j++) {
                const qgt_dev_op_t* o = &ops[j];
                int need1 = NEEDBIT(o), need2 = o->kind == QOP_SWAP ? o->lb2 : -1;
                if ((need1 >= 0 && role[need1] >= RL_WARP_) || (need2 >= 0 && role[need2] >= RL_WARP_)) break;
                if (p->nprog + 3 >= cap) { free(remap); return qgt_set_error(E_STATE, "programs: capacity"); }
                #define ROLE(lb, q) ((lb) >= 0 ? (uint8_t)role[(lb)] : (uint8_t)RL_OUT_)
                qgt_dev_op2_t x;
                memset(&x, 0, sizeof x);
                x.q = o->q;
                x.q2 = o->q2;
                x.coef = o->coef;
                x.slot = o->slot;
                x.gen = (uint8_t)o->gen;
                x.ra = ROLE(o->lb, o->q);
                x.rb = ROLE(o->lb2, o->q2);
                switch (o->kind) {
                case QOP_1Q:
                    x.kind = (o->pad == QGT_GATE_RY || o->pad == QGT_GATE_H || o->pad == QGT_GATE_X) ? Q2_UR : Q2_U;
                    break;
                case QOP_PHASE: x.kind = Q2_PHASE; break;
                case QOP_CZ: x.kind = Q2_CZ; break;
                case QOP_CNOT: x.kind = Q2_CNOT; break;
                case QOP_SWAP: {
                    /* SWAP(a, b) = CNOT(a->b) CNOT(b->a) CNOT(a->b): target first */
                    qgt_dev_op2_t c1 = x, c2 = x;
                    c1.kind = Q2_CNOT; c1.ra = ROLE(o->lb2, o->q2); c1.rb = ROLE(o->lb, o->q); c1.q = o->q2; c1.q2 = o->q;
                    c2.kind = Q2_CNOT; c2.ra = ROLE(o->lb, o->q); c2.rb = ROLE(o->lb2, o->q2);
                    c1.gen = 0; c2.gen = 0;
                    p->prog_h[p->nprog++] = c1;
                    p->prog_h[p->nprog++] = c2;
                    x = c1;
                    break;
                }
                default: x.kind = Q2_PHASE; break;
                }
                remap[j] = p->nprog;
                p->prog_h[p->nprog++] = x;
                #undef ROLE
            }
            cur_op = j;
            if (cur_op >= no) break;
        }
        (void)first;
        #undef NEEDBIT
        ps->prog_count = p->nprog - ps->prog_begin;
        /* spawn entries of this pass point into the program */
        for (int e = ps->ent_begin; e < ps->ent_begin + ps->ent_count; e++)
            if (p->ents_h[e].spawn_op >= 0) p->ents_h[e].spawn_op = remap[p->ents_h[e].spawn_op] - ps->prog_begin;
    }
    free(remap);
    return 0;
}

/* Runs of two or more consecutive diagonal ops (RZ / Z / S / T phases and
 * CZs) inside a segment get a Q2_DIAG header, so that the kernel multiplies
 * each amplitude once by the run's combined phase instead of once per gate.
 * Diagonal ops commute, so a derivative generator (-i/2) Z spawned inside the
 * run is applied after it. */
/* add a combined phase entry (product of the listed coefficient entries'
 * diagonals), or return the entry itself for a single factor */
static int comb_entry(qgt_plan_t* p, const int* list, int n)
{
    if (n == 1) return list[0];
    int32_t* ns = (int32_t*)realloc(p->comb_src_h, sizeof(int32_t) * ((size_t)p->comb_nsrc + n + 1));
    int32_t* np = (int32_t*)realloc(p->comb_ptr_h, sizeof(int32_t) * ((size_t)p->ncomb + 2));
    if (ns) p->comb_src_h = ns;
    if (np) p->comb_ptr_h = np;
    if (!ns || !np) return -1;
    if (p->ncomb == 0) p->comb_ptr_h[0] = 0;
    for (int i = 0; i < n; i++) p->comb_src_h[p->comb_nsrc++] = list[i];
    p->comb_ptr_h[p->ncomb + 1] = p->comb_nsrc;
    return p->ncoef + p->ncomb++;
}

/* One run of diagonal ops src[j, e) as a compact Q2_DIAG block (products of
 * the run's coefficients are formed once per step by the combine kernel):
 *   header   seg = sub-ops that follow, ra = thread phase entries, rb = CZT
 *            entries, slot = static sign mask over the register index
 *            (register-register CZs)
 *   RB register entries, bit i = 0 .. RB-1 in order: the bit's combined
 *            phase (coef -1: none) and in slot the physical qubits outside
 *            the register bits that share a CZ with it
 *   ra thread phase entries (lane, warp or outside qubit q)
 *   rb Q2_CZT entries: thread qubit q against the thread qubits in slot
 *   Q2_ZGEN markers, one per derivative spawned inside the run. */
static int emit_diag_run(qgt_plan_t* p, const qgt_dev_op2_t* src, int j, int e, qgt_dev_op2_t* out_ops, int* out,
                         int nb, int* remap)
{
    const int RB = reg_bits(p);
    int lists[40][64];
    int nl[40];
    int8_t role[40];
    memset(nl, 0, sizeof nl);
    memset(role, 0, sizeof role);
    uint32_t regmask = 0, czm[8] = {0}, czt[32] = {0};
    for (int t = j; t < e; t++) {
        const qgt_dev_op2_t* o = &src[t];
        const int ra_reg = o->ra >= RL_REG_ && o->ra < RL_WARP_;
        if (o->kind == Q2_PHASE) {
            /* slot index 0..7: register bits, 8 + q: thread qubit q */
            const int key = ra_reg ? (o->ra - RL_REG_) : 8 + o->q;
            if (key >= 40 || nl[key] >= 64) return qgt_set_error(E_STATE, "programs: diagonal run too long");
            role[key] = (int8_t)o->ra;
            lists[key][nl[key]++] = o->coef;
        } else {
            const int rb_reg = o->rb >= RL_REG_ && o->rb < RL_WARP_;
            if (ra_reg && rb_reg) {
                const int a = o->ra - RL_REG_, b = o->rb - RL_REG_;
                for (int r = 0; r < 32; r++)
                    if (((r >> a) & 1) && ((r >> b) & 1)) regmask ^= 1u << r;
            } else if (ra_reg || rb_reg) {
                const int i = (ra_reg ? o->ra : o->rb) - RL_REG_;
                const int q = ra_reg ? o->q2 : o->q;
                czm[i] ^= 1u << q;
            } else {
                const int a = o->q < o->q2 ? o->q : o->q2, b = o->q < o->q2 ? o->q2 : o->q;
                czt[a] ^= 1u << b;
            }
        }
    }
    int nt = 0, nz = 0, ng = 0;
    for (int k = 8; k < 40; k++) nt += nl[k] > 0;
    for (int a = 0; a < 32; a++) nz += czt[a] != 0;
    for (int t = j; t < e; t++) ng += src[t].slot >= 0;
    if (nt > 255 || nz > 255) return qgt_set_error(E_STATE, "programs: diagonal run too wide");
    qgt_dev_op2_t h;
    memset(&h, 0, sizeof h);
    h.kind = Q2_DIAG;
    h.seg = (int16_t)(RB + nt + nz + ng);
    h.ra = (uint8_t)nt;
    h.rb = (uint8_t)nz;
    h.coef = -1;
    h.slot = (int32_t)regmask;
    out_ops[(*out)++] = h;
    for (int i = 0; i < RB; i++) {
        qgt_dev_op2_t x;
        memset(&x, 0, sizeof x);
        x.kind = Q2_PHASE;
        x.ra = (uint8_t)(RL_REG_ + i);
        x.slot = (int32_t)czm[i];
        x.coef = nl[i] ? comb_entry(p, lists[i], nl[i]) : -1;
        if (nl[i] && x.coef < 0) return qgt_set_error(E_NOMEM, "programs: oom");
        out_ops[(*out)++] = x;
    }
    for (int k = 8; k < 40; k++) {
        if (!nl[k]) continue;
        qgt_dev_op2_t x;
        memset(&x, 0, sizeof x);
        x.kind = Q2_PHASE;
        x.ra = (uint8_t)role[k];
        x.q = (int8_t)(k - 8);
        x.slot = -1;
        x.coef = comb_entry(p, lists[k], nl[k]);
        if (x.coef < 0) return qgt_set_error(E_NOMEM, "programs: oom");
        out_ops[(*out)++] = x;
    }
    for (int a = 0; a < 32; a++) {
        if (!czt[a]) continue;
        qgt_dev_op2_t x;
        memset(&x, 0, sizeof x);
        x.kind = Q2_CZT;
        x.q = (int8_t)a;
        x.coef = -1;
        x.slot = (int32_t)czt[a];
        out_ops[(*out)++] = x;
    }
    for (int t = j; t < e; t++) {
        if (src[t].slot < 0) continue;
        qgt_dev_op2_t x = src[t];
        x.kind = Q2_ZGEN;
        x.coef = -1;
        remap[t] = *out - nb;
        out_ops[(*out)++] = x;
    }
    for (int t = j; t < e; t++)
        if (src[t].slot < 0) remap[t] = -1;   /* no entry spawns at a plain op */
    return 0;
}

/* Segment checkpoints.  Every vector of a pass runs the whole pass program, so
 * a derivative spawned in segment s first repeats the source vector's
 * evolution through segments 0 .. s-1.  For the largest group of spawns from
 * one source row, a writer entry (the source's own transport if the pass has
 * one, else an extra entry that stores nothing at the end) runs first and
 * stores its state at the start of every segment that a spawn begins in;
 * those spawns then start at their segment from the stored state (launched
 * after the writer).  The arithmetic of every vector is unchanged. */
static int build_checkpoints(qgt_plan_t* p)
{
    if (p->nprog == 0) return 0;
    for (int i = 0; i < p->nprog; i++)
        if (p->prog_h[i].kind == Q2_SEG) p->prog_h[i].slot = -1;
    int total = 0;
    for (int k = 0; k < p->npasses; k++) total += p->passes[k].ent_count + 1;
    qgt_dev_entry_t* ne = (qgt_dev_entry_t*)malloc(sizeof(qgt_dev_entry_t) * ((size_t)total + 1));
    int* segpos = (int*)malloc(sizeof(int) * ((size_t)p->nprog + 1));
    int* ckrow = (int*)malloc(sizeof(int) * ((size_t)p->nprog + 1));
    int* startof = (int*)malloc(sizeof(int) * ((size_t)total + 1));
    if (!ne || !segpos || !ckrow || !startof) {
        free(ne); free(segpos); free(ckrow); free(startof);
        return qgt_set_error(E_NOMEM, "checkpoints: oom");
    }
    const int base_row = (int)(p->pstride / p->N);
    int maxck = 0, out = 0;
    for (int k = 0; k < p->npasses; k++) {
        spass_t* ps = &p->passes[k];
        const qgt_dev_entry_t* src = p->ents_h + ps->ent_begin;
        const int nen = ps->ent_count, nb = out;
        ps->ckpt_writer = 0;
        ps->ngrp = 0;
        qgt_dev_op2_t* prog = p->prog_h + ps->prog_begin;
        int nseg = 0;
        for (int i = 0; i < ps->prog_count; i++)
            if (prog[i].kind == Q2_SEG) segpos[nseg++] = i;
        /* the segment (program index of its Q2_SEG) that a spawn from row r starts in */
#define SEG_OF(e) ({ int sp_ = 0; for (int t_ = 1; t_ < nseg; t_++) if (segpos[t_] <= (e)->spawn_op) sp_ = segpos[t_]; sp_; })
        /* the source row (with its zero-state flag) with the most spawns beyond the first segment */
        int best = -1, best_n = 0;
        for (int a = 0; a < nen && nseg > 1; a++) {
            if (src[a].spawn_op < 0) continue;
            int na = 0;
            for (int b = 0; b < nen; b++)
                if (src[b].spawn_op >= 0 && src[b].src_row == src[a].src_row &&
                    (src[b].flags & QENT_SRC_ZERO) == (src[a].flags & QENT_SRC_ZERO) && SEG_OF(&src[b]) > 0)
                    na++;
            if (na > best_n) { best_n = na; best = a; }
        }
        if (best_n < 2) {
            for (int a = 0; a < nen; a++) ne[out++] = src[a];
            ps->ent_begin = nb;
            ps->ent_count = out - nb;
            continue;
        }
        const int srow = src[best].src_row, szero = src[best].flags & QENT_SRC_ZERO;
        /* segments that spawns start in: a checkpoint row and a launch group each (at most
         * QGT_CKPT_GROUPS; spawns in further segments run the whole program as before) */
        for (int i = 0; i < ps->prog_count; i++) ckrow[i] = -1;
        int nck = 0;
        for (int a = 0; a < nen; a++) {
            const qgt_dev_entry_t* e = &src[a];
            startof[a] = 0;
            if (e->spawn_op < 0 || e->src_row != srow || (e->flags & QENT_SRC_ZERO) != szero) continue;
            const int sp = SEG_OF(e);
            if (sp == 0) continue;
            if (ckrow[sp] < 0) {
                if (nck >= QGT_CKPT_GROUPS) continue;
                ps->grp_start[nck] = sp;
                ckrow[sp] = nck++;
            }
            startof[a] = sp;
        }
#undef SEG_OF
        for (int i = 0; i < ps->prog_count; i++)
            if (ckrow[i] >= 0) prog[i].slot = base_row + ckrow[i];
        if (nck > maxck) maxck = nck;
        /* the writer: the source's transport, or an entry that keeps nothing */
        int wi = -1;
        for (int a = 0; a < nen; a++)
            if (src[a].spawn_op < 0 && src[a].src_row == srow && (src[a].flags & QENT_SRC_ZERO) == szero) { wi = a; break; }
        qgt_dev_entry_t w;
        if (wi >= 0) w = src[wi];
        else {
            memset(&w, 0, sizeof w);
            w.src_row = srow;
            w.dst_row = srow;
            w.spawn_op = -1;
            w.flags = szero;
            p->vector_passes++;
        }
        ne[out++] = w;
        ps->ckpt_writer = 1;
        /* entries that run the whole program, then one group per checkpoint */
        for (int a = 0; a < nen; a++)
            if (a != wi && startof[a] == 0) ne[out++] = src[a];
        ps->ngrp = nck;
        for (int g = 0; g < nck; g++) {
            const int sp = ps->grp_start[g];
            ps->grp_begin[g] = out - nb;
            for (int a = 0; a < nen; a++) {
                if (a == wi || startof[a] != sp) continue;
                qgt_dev_entry_t e = src[a];
                e.src_row = base_row + ckrow[sp];
                e.start_op = sp;
                e.flags &= ~QENT_SRC_ZERO;
                ne[out++] = e;
            }
            ps->grp_count[g] = out - nb - ps->grp_begin[g];
        }
        ps->ent_begin = nb;
        ps->ent_count = out - nb;
        if (ps->ent_count > 65535) {
            free(ne); free(segpos); free(ckrow); free(startof);
            return qgt_set_error(E_INVAL, "pass has more than 65535 vectors");
        }
    }
    free(p->ents_h);
    p->ents_h = ne;
    p->nents = out;
    p->pstride += (int64_t)maxck * p->N;
    free(segpos);
    free(ckrow);
    free(startof);
    return 0;
}

/* Pass renormalisation lists for complex64 register-resident programs: the
 * tangent-form RY coefficients scale vectors by up to sqrt 2 per gate, so
 * each pass's last single-qubit gate entry also divides by the product G of
 * the scales of all the pass's entries (formed on the device every step). */
static int build_renorm(qgt_plan_t* p)
{
    if (p->fp64 || p->nprog == 0 || p->npasses == 0) return 0;
    p->ren_ptr_h = (int32_t*)calloc((size_t)p->npasses + 1, sizeof(int32_t));
    p->ren_src_h = (int32_t*)malloc(sizeof(int32_t) * ((size_t)p->nops + 1));
    p->ren_h = (int32_t*)malloc(sizeof(int32_t) * (size_t)p->npasses);
    if (!p->ren_ptr_h || !p->ren_src_h || !p->ren_h) return qgt_set_error(E_NOMEM, "renormalisation: oom");
    int n = 0;
    for (int k = 0; k < p->npasses; k++) {
        const spass_t* ps = &p->passes[k];
        p->ren_h[k] = -1;
        for (int j = 0; j < ps->op_count; j++) {
            const qgt_dev_op_t* o = &p->ops_h[ps->op_begin + j];
            if (o->coef < 0) continue;
            p->ren_src_h[n++] = o->coef;
            if (o->kind == QOP_1Q && ps->prog_count > 0) p->ren_h[k] = o->coef;
        }
        p->ren_ptr_h[k + 1] = n;
    }
    return 0;
}

static int fold_diagonal_runs(qgt_plan_t* p)
{
    if (p->nprog == 0) return 0;
    int rc = 0;
    const int cap = 5 * p->nprog + 16;   /* a run of m ops emits at most 1 + RB + 2 m entries, a U block 1 + m */
    qgt_dev_op2_t* np2 = (qgt_dev_op2_t*)calloc((size_t)cap, sizeof(qgt_dev_op2_t));
    int* remap = (int*)malloc(sizeof(int) * ((size_t)p->nprog + 1));
    if (!np2 || !remap) { free(np2); free(remap); return qgt_set_error(E_NOMEM, "programs: oom"); }
    int out = 0;
    for (int k = 0; k < p->npasses; k++) {
        spass_t* ps = &p->passes[k];
        if (ps->prog_count == 0) { ps->prog_begin = out; continue; }
        const qgt_dev_op2_t* src = p->prog_h + ps->prog_begin;
        const int n = ps->prog_count, nb = out;
        for (int j = 0; j < n;) {
            int e = j;
            /* single-qubit gates on distinct lane / register bits commute: one Q2_UM block */
            uint32_t used = 0;
            while (e < n && (src[e].kind == Q2_U || src[e].kind == Q2_UR) && src[e].ra < RL_WARP_ &&
                   !((used >> src[e].ra) & 1u)) {
                used |= 1u << src[e].ra;
                e++;
            }
            if (e - j >= 2 && out + (e - j) + 2 < cap) {
                qgt_dev_op2_t h;
                memset(&h, 0, sizeof h);
                h.kind = Q2_UM;
                h.seg = (int16_t)(e - j);
                h.coef = -1;
                h.slot = -1;
                int nl = 0;
                for (int t = j; t < e; t++) nl += src[t].ra < RL_REG_;
                h.ra = (uint8_t)nl;
                h.rb = (uint8_t)((used >> RL_REG_) & 0xffu);
                np2[out++] = h;
                for (int t = j; t < e; t++)
                    if (src[t].ra < RL_REG_) { remap[t] = out - nb; np2[out++] = src[t]; }
                for (int b = RL_REG_; b < RL_WARP_; b++)
                    for (int t = j; t < e; t++)
                        if (src[t].ra == b) { remap[t] = out - nb; np2[out++] = src[t]; }
                j = e;
                continue;
            }
            e = j;
            while (e < n && (src[e].kind == Q2_PHASE || src[e].kind == Q2_CZ)) e++;
            if (e - j >= 2 && out + 2 * (e - j) + 8 < cap) {
                if ((rc = emit_diag_run(p, src, j, e, np2, &out, nb, remap)) != 0) { free(np2); free(remap); return rc; }
                j = e;
            } else {
                if (e == j) e = j + 1;
                for (int t = j; t < e; t++) { remap[t] = out - nb; np2[out++] = src[t]; }
                j = e;
            }
            if (out + 2 >= cap) { free(np2); free(remap); return qgt_set_error(E_STATE, "programs: capacity"); }
        }
        for (int en = ps->ent_begin; en < ps->ent_begin + ps->ent_count; en++)
            if (p->ents_h[en].spawn_op >= 0) p->ents_h[en].spawn_op = remap[p->ents_h[en].spawn_op];
        ps->prog_begin = nb;
        ps->prog_count = out - nb;
    }
    free(p->prog_h);
    p->prog_h = np2;
    p->nprog = out;
    free(remap);
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
static int run_head(qgt_plan_t* p, int* nl);
static int run_solve(qgt_plan_t* p, int* nl);

/* Straight-line pass kernels (qgt_jit.c): complex64 plans of MIXED precision
 * whose passes run on 13- or 14-qubit register tiles, from 13 qubits on (or
 * for every such plan with QGT_PASS_JIT=1; QGT_PASS_JIT=0 keeps the
 * interpreter).  The kernels of one plan compile in parallel. */
typedef struct {
    qgt_jit_pass_desc_t d;
    char* src;
    int32_t smem, device;
    qgt_jit_kernel_t* out;
    int rc;
    char err[256];
} jit_job_t;

static void* jit_worker(void* arg)
{
    jit_job_t* j = (jit_job_t*)arg;
    j->rc = qgt_dev_jit_compile(j->src, j->d.kname, j->smem, 32 << j->d.WB, j->device, &j->out);
    if (j->rc) snprintf(j->err, sizeof j->err, "%s", qgt_last_error());
    return NULL;
}

static int jit_wanted(const qgt_plan_t* p)
{
    const char* env = getenv("QGT_PASS_JIT");
    if (p->fp64 || p->opt.precision != QGT_PRECISION_MIXED) return 0;
    if (env && env[0] == '0') return 0;
    if (env && env[0] == '1') return 1;
    if (p->opt.pass_kernels == QGT_PASS_INTERPRET) return 0;
    if (p->opt.pass_kernels == QGT_PASS_COMPILED || p->opt.thread_amps == 16) return 1;
    return p->n >= 13;   /* every register-tile plan of 13 or more qubits */
}

/* the sources of every compiled pass kernel of the plan (host only) */
typedef struct {
    jit_job_t* jobs;
    int nj;
    int32_t* starts;
    int8_t* start_zero;
    char (*names)[48];
} jit_set_t;

static void jit_set_free(jit_set_t* js)
{
    for (int i = 0; i < js->nj; i++) free(js->jobs[i].src);
    free(js->jobs);
    free(js->starts);
    free(js->start_zero);
    free(js->names);
    memset(js, 0, sizeof *js);
}

static int jit_prepare(qgt_plan_t* p, jit_set_t* js)
{
    memset(js, 0, sizeof *js);
    js->jobs = (jit_job_t*)calloc((size_t)2 * p->npasses + 1, sizeof(jit_job_t));
    js->starts = (int32_t*)malloc(sizeof(int32_t) * ((size_t)p->nents + 2 * p->npasses + 1));
    js->start_zero = (int8_t*)calloc((size_t)p->nents + 2 * p->npasses + 1, 1);
    js->names = (char (*)[48])calloc((size_t)2 * p->npasses + 1, 48);
    if (!js->jobs || !js->starts || !js->start_zero || !js->names) { jit_set_free(js); return qgt_set_error(E_NOMEM, "jit: oom"); }
    int at = 0;
    for (int k = 0; k < p->npasses; k++) {
        spass_t* ps = &p->passes[k];
        if (ps->prog_count <= 0 || (ps->tile_bits != QGT_TILE_MAX_F32 && ps->tile_bits != QGT_TILE_WIDE_F32)) continue;
        for (int ck = 0; ck <= (ps->ckpt_writer ? 1 : 0); ck++) {
            /* the starts of the entries this kernel runs: all of the pass (ck = 0), the writer (ck = 1) */
            int32_t* st = js->starts + at;
            int8_t* sz = js->start_zero + at;
            int ns = 0;
            const int e0 = ps->ent_begin, e1 = ck ? ps->ent_begin + 1 : ps->ent_begin + ps->ent_count;
            for (int i = e0; i < e1; i++) {
                int t = 0;
                while (t < ns && st[t] != p->ents_h[i].start_op) t++;
                if (t == ns) { st[ns] = p->ents_h[i].start_op; sz[ns] = 0; ns++; }
                if (p->ents_h[i].flags & QENT_SRC_ZERO) sz[t] = 1;
            }
            at += ns;
            jit_job_t* j = &js->jobs[js->nj];
            snprintf(js->names[js->nj], 48, "qgt_pass%d_%s", k, ck ? "ckpt" : "run");
            j->d.prog = p->prog_h + ps->prog_begin;
            j->d.nops = ps->prog_count;
            j->d.segs = p->segs_h;
            j->d.l2p = ps->l2p;
            j->d.n = p->n;
            j->d.tile_bits = ps->tile_bits;
            j->d.RB = reg_bits(p);
            j->d.WB = ps->tile_bits - 5 - j->d.RB;
            j->d.tile_mask = ps->tile_mask;
            j->d.ckpt = ck;
            j->d.starts = st;
            j->d.start_zero = sz;
            j->d.nstarts = ns;
            j->d.kname = js->names[js->nj];
            j->smem = (int32_t)(8 << ps->tile_bits);
            j->device = p->opt.device;
            j->src = qgt_jit_pass_source(&j->d);
            if (!j->src) { int rc = qgt_last_error()[0] ? -1 : E_NOMEM; jit_set_free(js); return rc; }
            js->nj++;
        }
    }
    return 0;
}

static int build_jit(qgt_plan_t* p)
{
    p->njit = 0;
    if (!jit_wanted(p)) return 0;
    jit_set_t js;
    int rc = jit_prepare(p, &js);
    if (rc) return rc;
    jit_job_t* jobs = js.jobs;
    const int nj = js.nj;
    if (nj) {
        pthread_t* th = (pthread_t*)calloc((size_t)nj, sizeof(pthread_t));
        int* started = (int*)calloc((size_t)nj, sizeof(int));
        if (!th || !started) rc = qgt_set_error(E_NOMEM, "jit: oom");
        for (int i = 0; !rc && i < nj; i++) started[i] = pthread_create(&th[i], NULL, jit_worker, &jobs[i]) == 0;
        for (int i = 0; !rc && i < nj; i++) {
            if (started[i]) pthread_join(th[i], NULL);
            else jit_worker(&jobs[i]);
        }
        free(th);
        free(started);
        for (int i = 0; !rc && i < nj; i++)
            if (jobs[i].rc) rc = qgt_set_error(jobs[i].rc, "%s", jobs[i].err);
    }
    if (!rc) {
        int i = 0;
        for (int k = 0; k < p->npasses && i < nj; k++) {
            spass_t* ps = &p->passes[k];
            if (jobs[i].d.prog != p->prog_h + ps->prog_begin) continue;
            ps->jit[0] = jobs[i++].out;
            if (ps->ckpt_writer && i < nj) ps->jit[1] = jobs[i++].out;
            p->njit++;
        }
    }
    jit_set_free(&js);
    /* the interpreter has no 16-amplitude 13- / 14-qubit tile: every such pass must have its kernels */
    for (int k = 0; !rc && k < p->npasses; k++) {
        const spass_t* ps = &p->passes[k];
        if (ps->prog_count > 0 && amps16(p) && (!ps->jit[0] || (ps->ckpt_writer && !ps->jit[1])))
            rc = qgt_set_error(E_STATE, "jit: pass %d of a 16-amplitude tile has no compiled kernel", k);
    }
    if (rc) { for (int k = 0; k < p->npasses; k++) p->passes[k].jit[0] = p->passes[k].jit[1] = NULL; p->njit = 0; }
    return rc;
}

static int plan_create(const qgt_circuit_desc_t* c, const qgt_plan_options_t* opt, qgt_plan_t** out, int host_only);

int qgt_plan_create(const qgt_circuit_desc_t* c, const qgt_plan_options_t* opt, qgt_plan_t** out)
{
    return plan_create(c, opt, out, 0);
}

/* host_only: 0 a full plan; 1 the schedule without checkpoints (qgt_plan_schedule_dump); 2 the
 * schedule with checkpoints (qgt_plan_jit_check, qgt_plan_schedule_dump_ckpt); 1 and 2 hold no device
 * resources */
static int plan_create(const qgt_circuit_desc_t* c, const qgt_plan_options_t* opt, qgt_plan_t** out, int host_only)
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
    if ((p->opt.tile_bits != 0 && p->opt.tile_bits != QGT_TILE_MAX_F32 && p->opt.tile_bits != QGT_TILE_WIDE_F32) ||
        p->opt.pass_kernels < QGT_PASS_AUTO || p->opt.pass_kernels > QGT_PASS_COMPILED) {
        int tb = p->opt.tile_bits, pk = p->opt.pass_kernels;
        free(p);
        return qgt_set_error(E_INVAL, "qgt_plan_create: tile_bits %d (0, 13, 14) / pass_kernels %d (0 .. 2)", tb, pk);
    }
    if (p->opt.thread_amps != 0 && p->opt.thread_amps != 16 && p->opt.thread_amps != 32) {
        int bad = p->opt.thread_amps;
        free(p);
        return qgt_set_error(E_INVAL, "qgt_plan_create: thread_amps %d (0, 16 or 32)", bad);
    }
    if (p->opt.hamiltonian < QGT_HAMILTONIAN_NONE || p->opt.hamiltonian > QGT_HAMILTONIAN_PAULI) {
        int bad = (int)p->opt.hamiltonian;
        free(p);
        return qgt_set_error(E_INVAL, "qgt_plan_create: unknown Hamiltonian %d", bad);
    }
    p->n = c->num_qubits;
    p->N = (int64_t)1 << p->n;
    if (p->opt.thread_amps == 16 && p->opt.precision == QGT_PRECISION_MIXED && !jit_wanted(p)) {
        free(p);
        return qgt_set_error(E_INVAL, "qgt_plan_create: thread_amps 16 needs compiled pass kernels (pass_kernels, QGT_PASS_JIT)");
    }
    p->P = c->num_params;
    p->B = p->opt.batch > 0 ? p->opt.batch : 1;
    p->Pd = p->opt.num_deriv_params > 0 ? p->opt.num_deriv_params : p->P;
    if (p->B > 65535 || p->Pd > p->P || p->opt.batch < 0 || p->opt.num_deriv_params < 0) {
        int b = p->opt.batch, d = p->opt.num_deriv_params;
        free(p);
        return qgt_set_error(E_INVAL, "qgt_plan_create: batch %d (max 65535) / num_deriv_params %d (max num_params)", b, d);
    }
    if (p->B > 1 && p->opt.precision == QGT_PRECISION_MIXED_BF16X3) {
        free(p);
        return qgt_set_error(E_INVAL, "qgt_plan_create: batched plans support FP64 and MIXED precision");
    }
    p->fp64 = p->opt.precision == QGT_PRECISION_FP64;
    p->ngates = c->num_gates;
    p->gates = (sgate_t*)calloc((size_t)p->ngates + 1, sizeof(sgate_t));
    p->coef_h = (qgt_dev_coef_desc_t*)calloc((size_t)p->ngates + 1, sizeof(qgt_dev_coef_desc_t));
    if (!p->gates || !p->coef_h) { rc = qgt_set_error(E_NOMEM, "oom"); goto fail; }
    for (int g = 0; g < p->ngates; g++) {
        if ((rc = classify(&c->gates[g], p->n, p->P, &p->gates[g])) != 0) goto fail;
        sgate_t* sg = &p->gates[g];
        int rot = sg->type == QGT_GATE_RX || sg->type == QGT_GATE_RY || sg->type == QGT_GATE_RZ;
        if (rot && sg->param >= 0 && sg->param < p->Pd) sg->slot = p->nslots++;
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
    p->pstride = (int64_t)(p->rows + 1) * p->N;
    p->small_nsplit = p->rows <= 8 ? 1 : 0;   /* few rows: memory-bound FP64 small Gram */
    p->split_ld = p->N < 32 ? 32 : p->N;
    /* slot -> param CSR */
    p->slot_param_h = (int32_t*)calloc((size_t)p->nslots + 1, sizeof(int32_t));
    p->param_ptr_h = (int32_t*)calloc((size_t)p->Pd + 2, sizeof(int32_t));
    p->param_slots_h = (int32_t*)calloc((size_t)p->nslots + 1, sizeof(int32_t));
    if (!p->slot_param_h || !p->param_ptr_h || !p->param_slots_h) { rc = qgt_set_error(E_NOMEM, "oom"); goto fail; }
    for (int g = 0; g < p->ngates; g++)
        if (p->gates[g].slot >= 0) { p->slot_param_h[p->gates[g].slot] = p->gates[g].param; p->param_ptr_h[p->gates[g].param + 1]++; }
    for (int q = 0; q < p->Pd; q++) p->param_ptr_h[q + 1] += p->param_ptr_h[q];
    {
        int32_t* fill = (int32_t*)calloc((size_t)p->Pd + 1, sizeof(int32_t));
        if (!fill) { rc = qgt_set_error(E_NOMEM, "oom"); goto fail; }
        for (int s = 0; s < p->nslots; s++) {
            int q = p->slot_param_h[s];
            p->param_slots_h[p->param_ptr_h[q] + fill[q]++] = s;
        }
        free(fill);
    }
    if ((rc = setup_transport(p)) != 0) goto fail;
    if ((rc = choose_tile(p)) != 0) goto fail;
    if ((rc = compile_schedule(p)) != 0) goto fail;
    if ((rc = (p->mitm ? build_entries_mitm(p) : build_entries(p))) != 0) goto fail;
    if ((rc = build_programs(p)) != 0) goto fail;
    if ((rc = fold_diagonal_runs(p)) != 0) goto fail;
    if ((rc = build_renorm(p)) != 0) goto fail;
    if (host_only != 1 && (rc = build_checkpoints(p)) != 0) goto fail;
    if (p->opt.hamiltonian == QGT_HAMILTONIAN_PAULI) {
        /* parse the strings: character [n-1-q] acts on qubit q */
        const int T = p->opt.num_pauli_terms;
        if (T < 1 || T > 2048 || !p->opt.pauli_strings || !p->opt.pauli_coeffs) {
            rc = qgt_set_error(E_INVAL, "Pauli Hamiltonian: 1..2048 terms with strings and coefficients required");
            goto fail;
        }
        p->pauli_h = (qgt_dev_pauli_term_t*)calloc((size_t)T, sizeof(qgt_dev_pauli_term_t));
        if (!p->pauli_h) { rc = qgt_set_error(E_NOMEM, "oom"); goto fail; }
        p->hscale = 0;
        for (int k = 0; k < T; k++) {
            const char* str = p->opt.pauli_strings + (size_t)k * p->n;
            qgt_dev_pauli_term_t* t = &p->pauli_h[k];
            t->c = p->opt.pauli_coeffs[k];
            if (!isfinite(t->c)) { rc = qgt_set_error(E_INVAL, "Pauli coefficient %d is not finite", k); goto fail; }
            for (int q = 0; q < p->n; q++) {
                const char ch = str[p->n - 1 - q];
                if (ch == 'X' || ch == 'x') t->x |= 1u << q;
                else if (ch == 'Y' || ch == 'y') { t->x |= 1u << q; t->z |= 1u << q; t->ny++; }
                else if (ch == 'Z' || ch == 'z') t->z |= 1u << q;
            }
            p->hscale += fabs(t->c);
        }
        p->npauli = T;
        p->opt.pauli_strings = NULL;   /* copied; the caller's buffers need not outlive the call */
        p->opt.pauli_coeffs = NULL;
        if (p->hscale <= 0) p->hscale = 1.0;
    } else {
        int nb = p->n >= 3 ? p->n : p->n - 1;
        p->hscale = fabs(p->opt.tfim_J) * nb + fabs(p->opt.tfim_h) * p->n;
        if (p->hscale <= 0) p->hscale = 1.0;
    }
    p->split_scale = 16384.0f; /* 2^14: |amplitude| <= 1 stays below the FP16 maximum */

    /* ---- device resources ---- */
    p->host_only = host_only;
    if (host_only) { *out = p; return 0; }
    if ((rc = qgt_dev_set_device(p->opt.device)) != 0) goto fail;
    if ((rc = qgt_dev_stream_create(&p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_stream_create(&p->copy_stream)) != 0) goto fail;
    if ((rc = qgt_dev_event_create(&p->ev_post)) != 0) goto fail;
    if ((rc = qgt_dev_event_create(&p->ev_copied)) != 0) goto fail;
    for (int k = 0; k < p->npasses; k++)
        if (p->passes[k].ckpt_writer && !p->aux_stream) {
            if ((rc = qgt_dev_stream_create(&p->aux_stream)) != 0) goto fail;
            if ((rc = qgt_dev_event_create(&p->ev_fork)) != 0) goto fail;
            if ((rc = qgt_dev_event_create(&p->ev_join)) != 0) goto fail;
        }
    {
        size_t ab = p->fp64 ? 16 : 8;
        DALLOC(p->V, (size_t)p->B * (size_t)p->pstride * ab);
        if ((rc = qgt_dev_memset(p->V, 0, (size_t)p->B * (size_t)p->pstride * ab, p->stream)) != 0) goto fail;
        if (p->opt.precision == QGT_PRECISION_MIXED_BF16X3) {
            size_t sb = (size_t)4 * p->rows_pad * (size_t)p->split_ld * 2;
            DALLOC(p->split, sb);
            if ((rc = qgt_dev_memset(p->split, 0, sb, p->stream)) != 0) goto fail;
        }
    }
    DALLOC(p->ops_d, sizeof(qgt_dev_op_t) * (size_t)(p->nops + 1));
    DALLOC(p->ents_d, sizeof(qgt_dev_entry_t) * (size_t)(p->nents + 1));
    DALLOC(p->coef_desc_d, sizeof(qgt_dev_coef_desc_t) * (size_t)(p->ncoef + 1));
    DALLOC(p->coef_d, sizeof(double) * 8 * (size_t)p->B * (size_t)(p->ncoef + p->ncomb + 1));
    DALLOC(p->coef32_d, sizeof(float) * 8 * (size_t)p->B * (size_t)(p->ncoef + p->ncomb + 1));
    if (p->ncomb) {
        DALLOC(p->comb_ptr_d, sizeof(int32_t) * (size_t)(p->ncomb + 1));
        DALLOC(p->comb_src_d, sizeof(int32_t) * (size_t)(p->comb_nsrc + 1));
        if ((rc = qgt_dev_memcpy_h2d(p->comb_ptr_d, p->comb_ptr_h, sizeof(int32_t) * (size_t)(p->ncomb + 1), p->stream)) != 0)
            goto fail;
        if ((rc = qgt_dev_memcpy_h2d(p->comb_src_d, p->comb_src_h, sizeof(int32_t) * (size_t)p->comb_nsrc, p->stream)) != 0)
            goto fail;
    }
    DALLOC(p->prog_d, sizeof(qgt_dev_op2_t) * (size_t)(p->nprog + 1));
    DALLOC(p->segs_d, (size_t)16 * (p->nsegs + 1));
    {
        const size_t B = (size_t)p->B, Pd = (size_t)p->Pd;
        DALLOC(p->theta_d, sizeof(double) * (B * (size_t)p->P + 1));
        DALLOC(p->HG_d, sizeof(double) * 2 * B * (size_t)p->rows * p->rows);
        DALLOC(p->Q_d, sizeof(double) * 2 * B * Pd * Pd);
        DALLOC(p->grad_d, sizeof(double) * (B * Pd + 1));
        DALLOC(p->energy_d, sizeof(double) * (B + 1));
        DALLOC(p->natgrad_d, sizeof(double) * (B * Pd + 1));
        /* single points of complex64 plans solve with the refined FP32 factorisation */
        size_t cw = B * Pd * Pd;
        if (!p->fp64 && B == 1 && Pd > 0 && Pd <= 2048 && (size_t)qgt_dev_cholesky_refined_work((int32_t)Pd) > cw)
            cw = (size_t)qgt_dev_cholesky_refined_work((int32_t)Pd);
        DALLOC(p->chol_work_d, sizeof(double) * (cw + 1));
        DALLOC(p->status_d, sizeof(double) * 2 * B);
    }
    if (p->npauli) {
        DALLOC(p->pauli_d, sizeof(qgt_dev_pauli_term_t) * (size_t)p->npauli);
        if ((rc = qgt_dev_memcpy_h2d(p->pauli_d, p->pauli_h, sizeof(qgt_dev_pauli_term_t) * (size_t)p->npauli,
                                     p->stream)) != 0)
            goto fail;
    }
    if (p->mitm && !p->fp64 && p->nprog > 0) {
        const int ng = p->nscale_groups;
        DALLOC(p->scale_ptr_d, sizeof(int32_t) * (size_t)(ng + 1));
        DALLOC(p->scale_src_d, sizeof(int32_t) * (size_t)(p->scale_ptr_h[ng] + 1));
        DALLOC(p->row_group_d, sizeof(int32_t) * (size_t)p->rows);
        DALLOC(p->rho_d, sizeof(double) * (size_t)p->B * ng);
        if ((rc = qgt_dev_memcpy_h2d(p->scale_ptr_d, p->scale_ptr_h, sizeof(int32_t) * (size_t)(ng + 1), p->stream)) != 0)
            goto fail;
        if ((rc = qgt_dev_memcpy_h2d(p->row_group_d, p->row_group_h, sizeof(int32_t) * (size_t)p->rows, p->stream)) != 0)
            goto fail;
        if (p->scale_ptr_h[ng] && (rc = qgt_dev_memcpy_h2d(p->scale_src_d, p->scale_src_h, sizeof(int32_t) * (size_t)p->scale_ptr_h[ng],
                                                      p->stream)) != 0)
            goto fail;
    }
    if (p->ren_h) {
        const int np = p->npasses;
        DALLOC(p->ren_ptr_d, sizeof(int32_t) * (size_t)(np + 1));
        DALLOC(p->ren_src_d, sizeof(int32_t) * (size_t)(p->ren_ptr_h[np] + 1));
        DALLOC(p->ren_d, sizeof(int32_t) * (size_t)np);
        if ((rc = qgt_dev_memcpy_h2d(p->ren_ptr_d, p->ren_ptr_h, sizeof(int32_t) * (size_t)(np + 1), p->stream)) != 0) goto fail;
        if ((rc = qgt_dev_memcpy_h2d(p->ren_d, p->ren_h, sizeof(int32_t) * (size_t)np, p->stream)) != 0) goto fail;
        if (p->ren_ptr_h[np] &&
            (rc = qgt_dev_memcpy_h2d(p->ren_src_d, p->ren_src_h, sizeof(int32_t) * (size_t)p->ren_ptr_h[np], p->stream)) != 0)
            goto fail;
    }
    DALLOC(p->slot_param_d, sizeof(int32_t) * (size_t)(p->nslots + 1));
    DALLOC(p->param_ptr_d, sizeof(int32_t) * (size_t)(p->Pd + 2));
    DALLOC(p->param_slots_d, sizeof(int32_t) * (size_t)(p->nslots + 1));
    if (p->small_nsplit) {
        /* rows <= 8: about 4 CTAs per SM over all points, >= 1024 amplitudes per CTA */
        int64_t ns = (4 * 152 + p->B - 1) / p->B;
        int64_t maxs = p->N / 1024;
        if (ns > maxs) ns = maxs;
        if (ns < 1) ns = 1;
        p->small_nsplit = (int)ns;
        DALLOC(p->small_part_d, sizeof(double) * 2 * 36 * (size_t)p->B * (size_t)ns);
    } else if (p->fp64) {
        int nt = (p->rows + 31) / 32, ntp = nt * (nt + 1) / 2;
        int ns = (int)(4 * 152 / ((int64_t)ntp * p->B));
        if (ns < 1) ns = 1;
        int64_t maxs = p->N / 64;
        if (maxs < 1) maxs = 1;
        if (ns > maxs) ns = (int)maxs;
        p->part_nsplit = ns;
        DALLOC(p->part_d, sizeof(double) * 2 * 1024 * (size_t)ntp * ns * (size_t)p->B);
    } else if (p->opt.precision == QGT_PRECISION_MIXED_BF16X3) {
        if ((rc = qgt_dev_tc_gram_create(p->split, p->split_ld, p->rows, p->rows_pad, 1, &p->tc)) != 0) goto fail;
        p->device_bytes += qgt_dev_tc_gram_scratch_bytes(p->tc);
    } else {
        if (p->n < 4) { rc = qgt_set_error(E_INVAL, "mixed precision needs at least 4 qubits (use FP64)"); goto fail; }
        DALLOC(p->rowmax_d, sizeof(uint32_t) * (size_t)p->rows * p->B);
        if ((rc = qgt_dev_dg_gram_create(p->V, p->N, p->rows, p->rowmax_d, p->B, (int32_t)(p->pstride / p->N), &p->dg)) != 0) goto fail;
        p->device_bytes += qgt_dev_dg_gram_scratch_bytes(p->dg);
    }
    if ((rc = qgt_dev_memset(p->theta_d, 0, sizeof(double) * ((size_t)p->B * p->P + 1), p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_memcpy_h2d(p->ops_d, p->ops_h, sizeof(qgt_dev_op_t) * (size_t)p->nops, p->stream)) != 0) goto fail;
    for (int k = 0; k < p->npasses; k++) {   /* initial layouts of the register-resident entries */
        const spass_t* ps = &p->passes[k];
        if (ps->prog_count <= 0) continue;
        for (int i = ps->ent_begin; i < ps->ent_begin + ps->ent_count; i++) {
            qgt_dev_entry_t* e = &p->ents_h[i];
            const int8_t* L = p->segs_h + 16 * p->prog_h[ps->prog_begin + e->start_op].seg;
            for (int b = 0; b < 16; b++) {
                e->lay[b] = L[b];
                e->lay[16 + b] = (L[b] >= 0 && L[b] < 16) ? ps->l2p[L[b]] : (int8_t)0;
            }
        }
    }
    if ((rc = qgt_dev_memcpy_h2d(p->ents_d, p->ents_h, sizeof(qgt_dev_entry_t) * (size_t)p->nents, p->stream)) != 0) goto fail;
    if (p->nprog && (rc = qgt_dev_memcpy_h2d(p->prog_d, p->prog_h, sizeof(qgt_dev_op2_t) * (size_t)p->nprog, p->stream)) != 0) goto fail;
    if (p->nsegs && (rc = qgt_dev_memcpy_h2d(p->segs_d, p->segs_h, (size_t)16 * p->nsegs, p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_memcpy_h2d(p->coef_desc_d, p->coef_h, sizeof(qgt_dev_coef_desc_t) * (size_t)p->ncoef, p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_memcpy_h2d(p->slot_param_d, p->slot_param_h, sizeof(int32_t) * (size_t)p->nslots, p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_memcpy_h2d(p->param_ptr_d, p->param_ptr_h, sizeof(int32_t) * (size_t)(p->Pd + 1), p->stream)) != 0) goto fail;
    if ((rc = qgt_dev_memcpy_h2d(p->param_slots_d, p->param_slots_h, sizeof(int32_t) * (size_t)p->nslots, p->stream)) != 0) goto fail;
    {
        const size_t B = (size_t)p->B, Pd = (size_t)p->Pd;
        if ((rc = qgt_dev_host_alloc((void**)&p->theta_pin, sizeof(double) * (B * p->P + 1))) != 0) goto fail;
        if ((rc = qgt_dev_host_alloc((void**)&p->Q_pin, sizeof(double) * 2 * B * Pd * Pd + 16)) != 0) goto fail;
        if ((rc = qgt_dev_host_alloc((void**)&p->grad_pin, sizeof(double) * (B * Pd + 1))) != 0) goto fail;
        if ((rc = qgt_dev_host_alloc((void**)&p->natgrad_pin, sizeof(double) * (B * Pd + 1))) != 0) goto fail;
        if ((rc = qgt_dev_host_alloc((void**)&p->energy_pin, sizeof(double) * (B + 1))) != 0) goto fail;
        if ((rc = qgt_dev_host_alloc((void**)&p->status_pin, sizeof(double) * 2 * B)) != 0) goto fail;
        if ((rc = qgt_dev_host_alloc((void**)&p->gerr_pin, sizeof(int) * 4)) != 0) goto fail;
    }
    if ((rc = qgt_dev_stream_sync(p->stream)) != 0) goto fail;
    if ((rc = build_jit(p)) != 0) goto fail;
    /* first step eagerly (sets kernel attributes, validates), then capture */
    if ((rc = run_step(p)) != 0) goto fail;
    if ((rc = qgt_dev_stream_sync(p->stream)) != 0) goto fail;
    if (p->opt.use_graph) {
        /* two graphs: the step up to Q / grad / energy, then the solve (so that host outputs can
         * leave while the solve runs) */
        int nl = 0;
        for (int part = 0; part < 2; part++) {
            if (part == 1 && !(p->Pd > 0 && p->opt.hamiltonian != QGT_HAMILTONIAN_NONE)) break;
            if ((rc = qgt_dev_graph_begin(p->stream)) != 0) goto fail;
            int rs = part == 0 ? run_head(p, &nl) : run_solve(p, &nl);
            void* exec = NULL;
            int re = qgt_dev_graph_end(p->stream, &exec);
            if (rs) { qgt_dev_graph_destroy(exec); rc = rs; goto fail; }
            if (re) { rc = re; goto fail; }
            if (part == 0) p->graph = exec;
            else p->graph_solve = exec;
        }
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
    if (p->host_only) {
        free(p->gates); free(p->passes); free(p->ops_h); free(p->ents_h); free(p->coef_h); free(p->prog_h);
        free(p->segs_h); free(p->slot_param_h); free(p->param_ptr_h); free(p->param_slots_h); free(p->pauli_h);
        free(p->scale_ptr_h); free(p->scale_src_h); free(p->row_group_h);
        free(p->ren_ptr_h); free(p->ren_src_h); free(p->ren_h);
        free(p->op_gate);
        free(p->comb_ptr_h);
        free(p->comb_src_h);
        free(p);
        return;
    }
    if (p->stream) qgt_dev_stream_sync(p->stream);
    qgt_dev_graph_destroy(p->graph);
    qgt_dev_graph_destroy(p->graph_solve);
    if (p->aux_stream) {
        qgt_dev_stream_sync(p->aux_stream);
        qgt_dev_stream_destroy(p->aux_stream);
    }
    qgt_dev_event_destroy(p->ev_fork);
    qgt_dev_event_destroy(p->ev_join);
    if (p->copy_stream) {
        qgt_dev_stream_sync(p->copy_stream);
        qgt_dev_stream_destroy(p->copy_stream);
    }
    qgt_dev_event_destroy(p->ev_post);
    qgt_dev_event_destroy(p->ev_copied);
    qgt_dev_tc_gram_destroy(p->tc);
    qgt_dev_dg_gram_destroy(p->dg);
    qgt_dev_free(p->rowmax_d);
    free(p->pauli_h);
    free(p->scale_ptr_h); free(p->scale_src_h); free(p->row_group_h);
    free(p->ren_ptr_h); free(p->ren_src_h); free(p->ren_h);
    free(p->op_gate);
    free(p->comb_ptr_h);
    free(p->comb_src_h);
    void* dev[] = {p->V, p->split, p->small_part_d, p->pauli_d, p->scale_ptr_d, p->scale_src_d, p->row_group_d,
                   p->rho_d, p->comb_ptr_d, p->comb_src_d, p->ren_ptr_d, p->ren_src_d, p->ren_d,
                   p->ops_d, p->ents_d, p->prog_d, p->segs_d, p->coef32_d, p->coef_desc_d, p->coef_d, p->theta_d, p->HG_d, p->part_d,
                   p->Q_d, p->grad_d, p->energy_d, p->natgrad_d, p->chol_work_d, p->status_d, p->slot_param_d,
                   p->param_ptr_d, p->param_slots_d};
    for (size_t i = 0; i < sizeof dev / sizeof dev[0]; i++) qgt_dev_free(dev[i]);
    void* pin[] = {p->theta_pin, p->Q_pin, p->grad_pin, p->natgrad_pin, p->energy_pin, p->status_pin, p->gerr_pin};
    for (size_t i = 0; i < sizeof pin / sizeof pin[0]; i++) qgt_dev_host_free(pin[i]);
    qgt_dev_stream_destroy(p->stream);
    free(p->gates); free(p->passes); free(p->ops_h); free(p->ents_h); free(p->coef_h); free(p->prog_h); free(p->segs_h);
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
    info->vector_passes = p->vector_passes * p->B;
    info->gate_bytes = p->gate_bytes * p->B;
    info->gram_flops = (int64_t)4 * p->Pd * (p->Pd + 1) * p->N * p->B;
    info->batch = p->B;
    info->num_deriv_params = p->Pd;
    info->meet_in_middle = p->mitm;
    info->cut_gate = p->mitm ? p->cut : -1;
    info->jit_passes = p->njit;
    info->thread_amps = p->nprog > 0 ? 1 << reg_bits(p) : 0;
    info->device_bytes = p->device_bytes;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* execution                                                                 */
/* ------------------------------------------------------------------------ */

#define MARK(i) do { if (p->prof_ev[i] && (rc = qgt_dev_event_record(p->prof_ev[i], p->stream)) != 0) return rc; } while (0)

/* row 1 = H psi / hscale; psi is row 0, or psi(G) in a spare row with
 * meet-in-the-middle transport (whose last backward pass records row 1's
 * maximum instead, after carrying it to the cut) */
static int apply_hamiltonian(qgt_plan_t* p, int* launches)
{
    int rc = 0;
    const size_t ab = p->fp64 ? 16 : 8;
    const void* psi = (const char*)p->V + (size_t)(p->mitm ? p->row_T : 0) * p->N * ab;
    void* row1 = (char*)p->V + (size_t)p->N * ab;
    uint32_t* rmax = (p->rowmax_d && !p->mitm) ? p->rowmax_d + 1 : NULL;
    if (p->opt.hamiltonian == QGT_HAMILTONIAN_PAULI) {
        if ((rc = qgt_dev_pauli(psi, row1, p->n, p->pauli_d, p->npauli, 1.0 / p->hscale, p->fp64, rmax, p->B,
                                p->pstride, p->rows, p->stream)) != 0)
            return rc;
        (*launches)++;
    } else if (p->opt.hamiltonian == QGT_HAMILTONIAN_TFIM) {
        if ((rc = qgt_dev_tfim(psi, row1, p->n, p->opt.tfim_J, p->opt.tfim_h, 1.0 / p->hscale, p->fp64, p->split,
                               p->split_ld, (int64_t)p->rows_pad * p->split_ld, 1, p->split_scale, 1, rmax, p->B,
                               p->pstride, p->rows, p->stream)) != 0)
            return rc;
        (*launches)++;
    }
    return 0;
}

/* one register-resident launch: the pass's compiled kernel when it has one, else the interpreter */
static int pass2_launch(const spass_t* ps, const qgt_dev_pass2_args_t* b, int fp64, void* stream)
{
    const qgt_jit_kernel_t* k = ps->jit[b->ckpt ? 1 : 0];
    if (k) return qgt_dev_jit_launch(k, b, stream);
    return qgt_dev_pass2(b, fp64, stream);
}

static int run_head(qgt_plan_t* p, int* nl)
{
    int rc;
    int launches = 0;
    MARK(0);
    const int cstride = p->ncoef + p->ncomb;
    if ((rc = qgt_dev_prepare(p->coef_desc_d, p->ncoef, p->theta_d, p->coef_d, p->B, p->P, cstride, p->stream)) != 0)
        return rc;
    launches += p->ncoef > 0;
    if (!p->fp64 && p->nprog > 0) {
        if ((rc = qgt_dev_prepare32(p->coef_desc_d, p->ncoef, p->theta_d, p->coef32_d, p->B, p->P, cstride, p->stream)) != 0)
            return rc;
        launches += p->ncoef > 0;
        if (p->ren_d) {
            if ((rc = qgt_dev_renorm_passes(p->coef32_d, cstride, p->ren_ptr_d, p->ren_src_d, p->ren_d, p->npasses, p->B,
                                            p->stream)) != 0)
                return rc;
            launches++;
        }
        if (p->rho_d) {
            if ((rc = qgt_dev_scale_product(p->coef32_d, cstride, p->scale_ptr_d, p->scale_src_d, p->nscale_groups,
                                            p->rho_d, p->B, p->stream)) != 0)
                return rc;
            launches++;
        }
    }
    if (p->ncomb) {
        if ((rc = qgt_dev_combine_diag(p->fp64 ? p->coef_d : NULL, p->fp64 ? NULL : p->coef32_d, cstride, p->ncoef,
                                       p->comb_ptr_d, p->comb_src_d, p->ncomb, p->B, p->stream)) != 0)
            return rc;
        launches++;
    }
    if (p->dg && (rc = qgt_dev_memset(p->rowmax_d, 0, sizeof(uint32_t) * (size_t)p->rows * p->B, p->stream)) != 0)
        return rc;
    MARK(1);
    int h_done = 0;
    for (int k = 0; k < p->npasses; k++) {
        const spass_t* ps = &p->passes[k];
        if (ps->part == 2 && !h_done) {
            if ((rc = apply_hamiltonian(p, &launches)) != 0) return rc;
            h_done = 1;
        }
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
        a.npoints = p->B;
        a.coef_stride = p->ncoef + p->ncomb;
        a.point_stride = p->pstride;
        a.rowmax_stride = p->rows;
        if (ps->prog_count > 0) {
            qgt_dev_pass2_args_t b;
            memset(&b, 0, sizeof b);
            b.V = p->V;
            b.N = p->N;
            b.ops = p->prog_d + ps->prog_begin;
            b.nops = ps->prog_count;
            b.segs = p->segs_d;
            b.entries = a.entries;
            b.nentries = a.nentries;
            b.coef = p->coef_d;
            b.coef32 = p->coef32_d;
            b.split = a.split;
            b.split_ld = a.split_ld;
            b.split_plane_stride = a.split_plane_stride;
            b.split_scale = a.split_scale;
            b.n = a.n;
            b.tile_bits = a.tile_bits;
            b.tile_mask = a.tile_mask;
            memcpy(b.local_to_phys, a.local_to_phys, sizeof b.local_to_phys);
            b.rowmax = a.rowmax;
            b.npoints = a.npoints;
            b.coef_stride = a.coef_stride;
            b.point_stride = a.point_stride;
            b.rowmax_stride = a.rowmax_stride;
            if (ps->ckpt_writer) {
                /* fork: the checkpoint writer and then the spawns that start from its checkpoints
                 * (each from its own segment of the program) on the auxiliary stream, the entries
                 * that need no checkpoint on the main stream; join */
                const int nall = b.nentries;
                const int c0 = ps->ngrp > 0 ? ps->grp_begin[0] : nall;
                if ((rc = qgt_dev_event_record(p->ev_fork, p->stream)) != 0) return rc;
                if ((rc = qgt_dev_stream_wait_event(p->aux_stream, p->ev_fork)) != 0) return rc;
                b.nentries = 1;
                b.ckpt = 1;
                if ((rc = pass2_launch(ps, &b, p->fp64, p->aux_stream)) != 0) return rc;
                b.ckpt = 0;
                if (c0 < nall) {
                    b.entries = a.entries + c0;
                    b.nentries = nall - c0;
                    if ((rc = pass2_launch(ps, &b, p->fp64, p->aux_stream)) != 0) return rc;
                    launches++;
                }
                if (c0 > 1) {
                    b.entries = a.entries + 1;
                    b.nentries = c0 - 1;
                    if ((rc = pass2_launch(ps, &b, p->fp64, p->stream)) != 0) return rc;
                    launches++;
                }
                if ((rc = qgt_dev_event_record(p->ev_join, p->aux_stream)) != 0) return rc;
                if ((rc = qgt_dev_stream_wait_event(p->stream, p->ev_join)) != 0) return rc;
            } else if ((rc = pass2_launch(ps, &b, p->fp64, p->stream)) != 0) {
                return rc;
            }
        } else if ((rc = qgt_dev_pass(&a, p->fp64, p->stream)) != 0) {
            return rc;
        }
        launches++;
    }
    if (p->npasses == 0) {
        /* no gates: psi = |0...0> written directly (row 0) */
        size_t ab = p->fp64 ? 16 : 8;
        double one[2] = {1.0, 0.0};
        float onef[2] = {1.0f, 0.0f};
        if (!p->fp64) return qgt_set_error(E_INVAL, "mixed plan needs at least one gate");
        for (int b = 0; b < p->B; b++) {
            char* row0 = (char*)p->V + (size_t)b * p->pstride * ab;
            if ((rc = qgt_dev_memset(row0, 0, (size_t)p->N * ab, p->stream)) != 0) return rc;
            if ((rc = qgt_dev_memcpy_h2d(row0, one, ab, p->stream)) != 0) return rc;
        }
        (void)onef;
    }
    MARK(2);
    const int has_h = p->opt.hamiltonian != QGT_HAMILTONIAN_NONE;
    if (!h_done && (rc = apply_hamiltonian(p, &launches)) != 0) return rc;
    MARK(3);
    if (p->small_nsplit) {
        if ((rc = qgt_dev_gram_small(p->V, p->N, p->rows, !has_h, p->fp64, p->small_part_d, p->small_nsplit, p->HG_d,
                                     p->B, p->pstride, p->stream)) != 0)
            return rc;
    } else if (p->fp64) {
        if ((rc = qgt_dev_gram_f64(p->V, p->N, p->rows, p->part_d, p->part_nsplit, p->HG_d, p->B, p->pstride,
                                   p->stream)) != 0)
            return rc;
    } else if (p->dg) {
        if ((rc = qgt_dev_dg_gram_run(p->dg, p->HG_d, p->stream)) != 0) return rc;
    } else {
        double s = (double)p->split_scale;
        if ((rc = qgt_dev_tc_gram_run(p->tc, 1.0 / (s * s), p->HG_d, p->stream)) != 0) return rc;
    }
    launches += 2;
    MARK(4);
    if (p->Pd > 0) {
        qgt_dev_post_args_t pa;
        memset(&pa, 0, sizeof pa);
        pa.HG = p->HG_d;
        pa.rows = p->rows;
        pa.P = p->Pd;
        pa.npoints = p->B;
        pa.slot_param = p->slot_param_d;
        pa.param_ptr = p->param_ptr_d;
        pa.param_slots = p->param_slots_d;
        pa.hscale = p->hscale;
        pa.has_h = has_h;
        pa.Q = p->Q_d;
        pa.grad = p->grad_d;
        pa.energy = p->energy_d;
        pa.rho = p->rho_d;
        pa.row_group = p->row_group_d;
        pa.ngroups = p->nscale_groups;
        if ((rc = qgt_dev_post(&pa, p->stream)) != 0) return rc;
        launches += 1 + has_h;
    }
    MARK(5);
    *nl += launches;
    return 0;
}

/* the natural-gradient solve of a step (after run_head) */
static int run_solve(qgt_plan_t* p, int* nl)
{
    int rc;
    int launches = 0;
    const int has_h = p->opt.hamiltonian != QGT_HAMILTONIAN_NONE;
    if (p->Pd > 0) {
        if (has_h) {
            if (p->B > 1) {
                /* one CTA per point, lambda x10 retries inside */
                if ((rc = qgt_dev_cholesky_batch(p->Q_d, 1, p->grad_d, p->Pd, p->opt.lambda, p->chol_work_d,
                                                 p->natgrad_d, p->status_d, p->B, p->stream)) != 0)
                    return rc;
                launches++;
            } else if (p->Pd <= 2048 && !p->fp64) {
                if ((rc = qgt_dev_cholesky_refined(p->Q_d, 1, p->grad_d, p->Pd, p->opt.lambda, p->chol_work_d,
                                                   p->natgrad_d, p->status_d, p->stream)) != 0)
                    return rc;
                launches += qgt_dev_cholesky_refined_launches(p->Pd);
            } else if (p->Pd <= 2048) {
                if ((rc = qgt_dev_cholesky_blocked(p->Q_d, 1, p->grad_d, p->Pd, p->opt.lambda, p->chol_work_d,
                                                   p->natgrad_d, p->status_d, p->stream)) != 0)
                    return rc;
                launches += qgt_dev_cholesky_launches(p->Pd);
            } else {
                if ((rc = qgt_dev_cholesky(p->Q_d, 1, p->grad_d, p->Pd, p->opt.lambda, p->chol_work_d, p->natgrad_d,
                                           p->status_d, p->stream)) != 0)
                    return rc;
                launches++;
            }
        }
    }
    MARK(6);
    *nl += launches;
    return 0;
}

static int run_step(qgt_plan_t* p)
{
    int launches = 0;
    int rc = run_head(p, &launches);
    if (!rc) rc = run_solve(p, &launches);
    if (!rc) p->launches = launches;
    return rc;
}

int qgt_plan_profile_step(qgt_plan_t* p, qgt_step_profile_t* pr)
{
    if (!p || !pr) return qgt_set_error(E_INVAL, "qgt_plan_profile_step: NULL argument");
    int rc = 0;
    for (int i = 0; i < 7 && !rc; i++) rc = qgt_dev_event_create(&p->prof_ev[i]);
    if (!rc) rc = run_step(p);
    float t[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 6 && !rc; i++) rc = qgt_dev_event_elapsed(p->prof_ev[i], p->prof_ev[i + 1], &t[i]);
    for (int i = 0; i < 7; i++) { qgt_dev_event_destroy(p->prof_ev[i]); p->prof_ev[i] = NULL; }
    if (rc) return rc;
    p->has_run = 1;
    pr->prepare_ms = t[0];
    pr->passes_ms = t[1];
    pr->hamiltonian_ms = t[2];
    pr->gram_ms = t[3];
    pr->post_ms = t[4];
    pr->solve_ms = t[5];
    pr->total_ms = t[0] + t[1] + t[2] + t[3] + t[4] + t[5];
    return 0;
}

/* one step; post_event: recorded on the stream once Q, grad and energy are final (NULL: none) */
static int launch_step_ev(qgt_plan_t* p, void* post_event)
{
    int rc, nl = 0;
    if (p->graph) rc = qgt_dev_graph_launch(p->graph, p->stream);
    else rc = run_head(p, &nl);
    if (!rc && post_event) rc = qgt_dev_event_record(post_event, p->stream);
    if (!rc) {
        if (p->graph) rc = p->graph_solve ? qgt_dev_graph_launch(p->graph_solve, p->stream) : 0;
        else rc = run_solve(p, &nl);
    }
    p->has_run = 1;
    return rc;
}

static int launch_step(qgt_plan_t* p) { return launch_step_ev(p, NULL); }

int qgt_plan_execute_device(qgt_plan_t* p, const double* theta_dev, double* Q_dev, double* grad_dev,
                            double* energy_dev, double* natgrad_dev)
{
    int rc;
    if (!p) return qgt_set_error(E_INVAL, "qgt_plan_execute_device: plan is NULL");
    const size_t B = (size_t)p->B, Pd = (size_t)p->Pd;
    if (p->P > 0 && theta_dev && theta_dev != p->theta_d)
        if ((rc = qgt_dev_memcpy_d2d(p->theta_d, theta_dev, sizeof(double) * B * (size_t)p->P, p->stream)) != 0) return rc;
    if ((rc = launch_step(p)) != 0) return rc;
    int has_h = p->opt.hamiltonian != QGT_HAMILTONIAN_NONE;
    if (Q_dev && Q_dev != p->Q_d && (rc = qgt_dev_memcpy_d2d(Q_dev, p->Q_d, sizeof(double) * 2 * B * Pd * Pd, p->stream)) != 0) return rc;
    if (has_h) {
        if (grad_dev && grad_dev != p->grad_d && (rc = qgt_dev_memcpy_d2d(grad_dev, p->grad_d, sizeof(double) * B * Pd, p->stream)) != 0) return rc;
        if (energy_dev && energy_dev != p->energy_d && (rc = qgt_dev_memcpy_d2d(energy_dev, p->energy_d, sizeof(double) * B, p->stream)) != 0) return rc;
        if (natgrad_dev && natgrad_dev != p->natgrad_d && (rc = qgt_dev_memcpy_d2d(natgrad_dev, p->natgrad_d, sizeof(double) * B * Pd, p->stream)) != 0) return rc;
    }
    return 0;
}

int qgt_plan_execute_host(qgt_plan_t* p, const double* theta, double* Q, double* grad, double* energy, double* natgrad)
{
    int rc;
    if (!p) return qgt_set_error(E_INVAL, "qgt_plan_execute_host: plan is NULL");
    if (p->P > 0 && !theta) return qgt_set_error(E_INVAL, "qgt_plan_execute_host: theta is NULL");
    const size_t B = (size_t)p->B, Pd = (size_t)p->Pd, nth = B * (size_t)p->P;
    for (size_t k = 0; k < nth; k++)
        if (!isfinite(theta[k])) return qgt_set_error(E_INVAL, "qgt_plan_execute_host: theta[%zu] is not finite", k);
    int has_h = p->opt.hamiltonian != QGT_HAMILTONIAN_NONE;
    if ((grad || energy || natgrad) && !has_h)
        return qgt_set_error(E_INVAL, "qgt_plan_execute_host: energy outputs need a Hamiltonian");
    if (p->P > 0) {
        memcpy(p->theta_pin, theta, sizeof(double) * nth);
        if ((rc = qgt_dev_memcpy_h2d(p->theta_d, p->theta_pin, sizeof(double) * nth, p->stream)) != 0) return rc;
    }
    const int early = p->Pd > 0;
    if ((rc = launch_step_ev(p, early ? p->ev_post : NULL)) != 0) return rc;
    const int need_status = has_h && p->Pd > 0;
    const int* gerr = p->tc ? qgt_dev_tc_gram_err(p->tc) : (p->dg ? qgt_dev_dg_gram_err(p->dg) : NULL);
    /* Q, grad, energy and the Gram's status are final when the post kernels end (ev_post): they
     * travel on copy_stream and into the caller's buffers while the solve runs; the solve's
     * status and natgrad follow on the step's stream (one more synchronisation) */
    void* cs = early ? p->copy_stream : p->stream;
    if (early && (rc = qgt_dev_stream_wait_event(cs, p->ev_post)) != 0) return rc;
    if (gerr && (rc = qgt_dev_memcpy_d2h(p->gerr_pin, gerr, sizeof(int), cs)) != 0) return rc;
    if (Q && (rc = qgt_dev_memcpy_d2h(p->Q_pin, p->Q_d, sizeof(double) * 2 * B * Pd * Pd, cs)) != 0) return rc;
    if (grad && (rc = qgt_dev_memcpy_d2h(p->grad_pin, p->grad_d, sizeof(double) * B * Pd, cs)) != 0) return rc;
    if (energy && (rc = qgt_dev_memcpy_d2h(p->energy_pin, p->energy_d, sizeof(double) * B, cs)) != 0) return rc;
    if (early && (rc = qgt_dev_event_record(p->ev_copied, cs)) != 0) return rc;
    if (need_status && (rc = qgt_dev_memcpy_d2h(p->status_pin, p->status_d, sizeof(double) * 2 * B, p->stream)) != 0) return rc;
    if (natgrad && (rc = qgt_dev_memcpy_d2h(p->natgrad_pin, p->natgrad_d, sizeof(double) * B * Pd, p->stream)) != 0) return rc;
    if (early && (rc = qgt_dev_event_sync(p->ev_copied)) != 0) return rc;
    /* a failed Gram invalidates everything after it: report it first */
    if (gerr && p->gerr_pin[0]) {
        qgt_dev_stream_sync(p->stream);
        return qgt_set_error(p->gerr_pin[0], "tensor-core Gram reported device status %d", p->gerr_pin[0]);
    }
    if (Q) memcpy(Q, p->Q_pin, sizeof(double) * 2 * B * Pd * Pd);
    if (grad) memcpy(grad, p->grad_pin, sizeof(double) * B * Pd);
    if (energy) memcpy(energy, p->energy_pin, sizeof(double) * B);
    if ((rc = qgt_dev_stream_sync(p->stream)) != 0) return rc;
    if (need_status) {
        if (B == 1) {
            /* the graph's blocked solve has no retries: on a non-positive pivot
             * rerun the solve with lambda x 10 retries (outside the graph).  The
             * refined solve of complex64 plans also stops when its FP32 factor
             * loses a pivot or the refinement does not converge; the FP64
             * solver then starts from lambda itself */
            const double lam0 = p->fp64 || p->Pd > 2048 ? p->opt.lambda * 10.0 : p->opt.lambda;
            if ((int)p->status_pin[0] != 0) {
                if ((rc = qgt_dev_cholesky(p->Q_d, 1, p->grad_d, p->Pd, lam0, p->chol_work_d, p->natgrad_d,
                                           p->status_d, p->stream)) != 0)
                    return rc;
                if (natgrad &&
                    (rc = qgt_dev_memcpy_d2h(p->natgrad_pin, p->natgrad_d, sizeof(double) * B * Pd, p->stream)) != 0)
                    return rc;
                if ((rc = qgt_dev_memcpy_d2h(p->status_pin, p->status_d, sizeof(double) * 2, p->stream)) != 0)
                    return rc;
                if ((rc = qgt_dev_stream_sync(p->stream)) != 0) return rc;
                if ((int)p->status_pin[0] != 0)
                    return qgt_set_error((int)p->status_pin[0],
                                         "cholesky: not positive definite after lambda retries (last lambda %g)",
                                         p->status_pin[1]);
            }
        } else {
            for (size_t b = 0; b < B; b++)
                if ((int)p->status_pin[2 * b] != 0)
                    return qgt_set_error((int)p->status_pin[2 * b], "cholesky: point %zu not positive definite after lambda retries", b);
        }
    }
    if (natgrad) memcpy(natgrad, p->natgrad_pin, sizeof(double) * B * Pd);
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
    const size_t row = p->mitm ? (size_t)p->row_T : 0;   /* psi after the last gate */
    if (p->fp64) {
        if ((rc = qgt_dev_memcpy_d2h(psi, (const char*)p->V + row * p->N * 16, sizeof(double) * 2 * (size_t)p->N,
                                     p->stream)) != 0)
            return rc;
        return qgt_dev_stream_sync(p->stream);
    }
    float* tmp = (float*)malloc(sizeof(float) * 2 * (size_t)p->N);
    if (!tmp) return qgt_set_error(E_NOMEM, "qgt_plan_get_state: oom");
    rc = qgt_dev_memcpy_d2h(tmp, (const char*)p->V + row * p->N * 8, sizeof(float) * 2 * (size_t)p->N, p->stream);
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
    if (!p->has_run) return qgt_set_error(E_STATE, "qgt_plan_get_row: no step has run");
    if (p->fp64) {
        int rc = qgt_dev_memcpy_d2h(out, (char*)p->V + (size_t)row * p->N * 16, sizeof(double) * 2 * (size_t)p->N, p->stream);
        if (!rc) rc = qgt_dev_stream_sync(p->stream);
        return rc;
    }
    if (p->opt.precision != QGT_PRECISION_MIXED) return qgt_set_error(E_STATE, "qgt_plan_get_row: not kept by BF16x3 plans");
    float* tmp = (float*)malloc(sizeof(float) * 2 * (size_t)p->N);
    if (!tmp) return qgt_set_error(E_NOMEM, "qgt_plan_get_row: oom");
    int rc = qgt_dev_memcpy_d2h(tmp, (char*)p->V + (size_t)row * p->N * 8, sizeof(float) * 2 * (size_t)p->N, p->stream);
    if (!rc) rc = qgt_dev_stream_sync(p->stream);
    if (!rc) for (int64_t i = 0; i < 2 * p->N; i++) out[i] = tmp[i];
    free(tmp);
    return rc;
}

int qgt_plan_device_status(qgt_plan_t* p, double* lambda_used)
{
    if (!p) return qgt_set_error(E_INVAL, "qgt_plan_device_status: plan is NULL");
    int rc = qgt_dev_memcpy_d2h(p->status_pin, p->status_d, sizeof(double) * 2 * (size_t)p->B, p->stream);
    if (!rc) rc = qgt_dev_stream_sync(p->stream);
    if (rc) return rc;
    if (lambda_used) *lambda_used = p->status_pin[1];
    /* the Gram's status first: a failed Gram makes the solve's status meaningless */
    int st = 0;
    if (p->tc) st = qgt_dev_tc_gram_status(p->tc, p->stream);
    if (!st && p->dg) st = qgt_dev_dg_gram_status(p->dg, p->stream);
    for (int b = 0; b < p->B && !st; b++) st = (int)p->status_pin[2 * b];
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

int qgt_plan_test_gram_stall(qgt_plan_t* p, int stall, int64_t timeout_ns)
{
    if (!p) return qgt_set_error(E_INVAL, "qgt_plan_test_gram_stall: plan is NULL");
    if (!p->dg) return qgt_set_error(E_STATE, "qgt_plan_test_gram_stall: the plan has no integer-digit Gram");
    if ((stall && timeout_ns <= 0) || timeout_ns > 4000000000LL)
        return qgt_set_error(E_INVAL, "qgt_plan_test_gram_stall: timeout %lld ns out of range (a stall needs (0, 4 s])",
                             (long long)timeout_ns);
    int rc = qgt_dev_stream_sync(p->stream);
    if (!rc) rc = qgt_dev_dg_gram_set_stall(p->dg, stall, timeout_ns, p->stream);
    return rc;
}

/* The compiled pass kernels of a plan without a device: the schedule (with
 * checkpoints), every pass's generated source (written to dump_dir when given)
 * and, with compile = 1, each source through the compiler (no load).  Returns
 * the number of kernels (or a negative error); *seconds = compile time. */
int qgt_plan_jit_check(const void* circuit, const void* options, const char* dump_dir, int compile, double* seconds)
{
    qgt_plan_t* p = NULL;
    int rc = plan_create((const qgt_circuit_desc_t*)circuit, (const qgt_plan_options_t*)options, &p, 2);
    if (rc) return rc;
    jit_set_t js;
    if ((rc = jit_prepare(p, &js)) != 0) { qgt_plan_destroy(p); return rc; }
    double tot = 0;
    for (int i = 0; i < js.nj && !rc; i++) {
        if (dump_dir) {
            char path[1024];
            snprintf(path, sizeof path, "%s/%s.cu", dump_dir, js.jobs[i].d.kname);
            FILE* f = fopen(path, "w");
            if (!f) { rc = qgt_set_error(E_INVAL, "qgt_plan_jit_check: cannot write %s", path); break; }
            fputs(js.jobs[i].src, f);
            fclose(f);
        }
        if (compile) {
            double t = 0;
            rc = qgt_jit_nvrtc_check(js.jobs[i].src, &t);
            tot += t;
        }
    }
    const int n = js.nj;
    jit_set_free(&js);
    qgt_plan_destroy(p);
    if (seconds) *seconds = tot;
    return rc ? rc : n;
}

int qgt_plan_enqueue_step(qgt_plan_t* p, void* stream)
{
    void* own = p->stream;
    p->stream = stream;
    int rc = run_step(p);
    p->stream = own;
    p->has_run = 1;
    return rc;
}

double* qgt_plan_dev_theta(qgt_plan_t* p) { return p->theta_d; }
double* qgt_plan_dev_Q(qgt_plan_t* p) { return p->Q_d; }
int qgt_plan_launches(const qgt_plan_t* p) { return p->launches; }
const void* qgt_plan_dev_V(qgt_plan_t* p, int64_t* point_stride, int32_t* fp64)
{
    if (point_stride) *point_stride = p->pstride;
    if (fp64) *fp64 = p->fp64;
    return p->V;
}
double* qgt_plan_dev_grad(qgt_plan_t* p) { return p->grad_d; }
double* qgt_plan_dev_energy(qgt_plan_t* p) { return p->energy_d; }
double* qgt_plan_dev_natgrad(qgt_plan_t* p) { return p->natgrad_d; }

/* out = sum_s c[s] d_s over the derivative slots of an FP64 plan (2^n complex, host) */
int qgt_plan_combine_slots(qgt_plan_t* p, const double* c, double* out)
{
    if (!p || !c || !out) return qgt_set_error(E_INVAL, "qgt_plan_combine_slots: bad argument");
    if (!p->fp64 || p->B != 1 || p->mitm)
        return qgt_set_error(E_STATE, "qgt_plan_combine_slots: unbatched FP64 plans with forward transport only");
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

/* The compiled schedule as JSON (no device needed): passes with their gate
 * ops and vector entries, coefficient sources and the row layout.  Used by
 * the CPU tests, which replay it against the FP64 oracle. */
static int schedule_dump(const void* circuit, const void* options, const char* path, int host_only);

int qgt_plan_schedule_dump(const void* circuit, const void* options, const char* path)
{
    return schedule_dump(circuit, options, path, 1);
}

int qgt_plan_schedule_dump_ckpt(const void* circuit, const void* options, const char* path)
{
    return schedule_dump(circuit, options, path, 2);
}

static int schedule_dump(const void* circuit, const void* options, const char* path, int host_only)
{
    const qgt_circuit_desc_t* c = (const qgt_circuit_desc_t*)circuit;
    const qgt_plan_options_t* opt = (const qgt_plan_options_t*)options;
    qgt_plan_t* p = NULL;
    int rc = plan_create(c, opt, &p, host_only);
    if (rc) return rc;
    FILE* f = fopen(path, "w");
    if (!f) { qgt_plan_destroy(p); return qgt_set_error(E_INVAL, "qgt_plan_schedule_dump: cannot write %s", path); }
    fprintf(f, "{\"n\": %d, \"rows\": %d, \"nslots\": %d, \"mitm\": %d, \"cut\": %d, \"early_slots\": %d, "
               "\"row_T\": %d, \"hscale\": %.17g,\n", p->n, p->rows, p->nslots, p->mitm, p->cut, p->early_slots,
            p->row_T, p->hscale);
    fprintf(f, "\"coefs\": [");
    for (int i = 0; i < p->ncoef; i++)
        fprintf(f, "%s[%d, %d, %.17g]", i ? ", " : "", p->coef_h[i].type, p->coef_h[i].param, p->coef_h[i].angle);
    fprintf(f, "],\n\"slot_param\": [");
    for (int i = 0; i < p->nslots; i++) fprintf(f, "%s%d", i ? ", " : "", p->slot_param_h[i]);
    fprintf(f, "],\n\"passes\": [");
    for (int k = 0; k < p->npasses; k++) {
        const spass_t* ps = &p->passes[k];
        fprintf(f, "%s{\"part\": %d, \"tile_mask\": %u, \"ops\": [", k ? ",\n" : "", ps->part, ps->tile_mask);
        for (int j = 0; j < ps->op_count; j++) {
            const qgt_dev_op_t* o = &p->ops_h[ps->op_begin + j];
            fprintf(f, "%s[%d, %d, %d, %d, %d, %d]", j ? ", " : "", (int)o->pad, (int)o->q, (int)o->q2, o->coef, o->slot,
                    (int)o->kind);
        }
        if (p->ren_h) {
            fprintf(f, "], \"ren\": %d, \"ren_src\": [", p->ren_h[k]);
            for (int j = p->ren_ptr_h[k]; j < p->ren_ptr_h[k + 1]; j++)
                fprintf(f, "%s%d", j > p->ren_ptr_h[k] ? ", " : "", p->ren_src_h[j]);
        }
        fprintf(f, "], \"prog\": [");
        for (int j = 0; j < ps->prog_count; j++) {
            const qgt_dev_op2_t* o = &p->prog_h[ps->prog_begin + j];
            fprintf(f, "%s[%d, %d, %d, %d, %d]", j ? ", " : "", (int)o->kind, (int)o->ra, (int)o->rb, (int)o->seg, o->slot);
        }
        fprintf(f, "], \"entries\": [");
        for (int e = 0; e < ps->ent_count; e++) {
            const qgt_dev_entry_t* en = &p->ents_h[ps->ent_begin + e];
            fprintf(f, "%s[%d, %d, %d, %d]", e ? ", " : "", en->src_row, en->dst_row, en->spawn_op, en->flags);
        }
        /* the register programs in full (kind, ra, rb, seg, slot, coef, q, q2, gen), the pass's tile
         * (local bit -> physical qubit) and the start op of each entry */
        fprintf(f, "], \"ckpt_writer\": %d, \"tile_bits\": %d, \"l2p\": [", ps->ckpt_writer, ps->tile_bits);
        for (int b = 0; b < 16; b++) fprintf(f, "%s%d", b ? ", " : "", (int)ps->l2p[b]);
        fprintf(f, "], \"prog2\": [");
        for (int j = 0; j < ps->prog_count; j++) {
            const qgt_dev_op2_t* o = &p->prog_h[ps->prog_begin + j];
            fprintf(f, "%s[%d, %d, %d, %d, %d, %d, %d, %d, %d]", j ? ", " : "", (int)o->kind, (int)o->ra, (int)o->rb,
                    (int)o->seg, o->slot, o->coef, (int)o->q, (int)o->q2, (int)o->gen);
        }
        fprintf(f, "], \"starts\": [");
        for (int e = 0; e < ps->ent_count; e++)
            fprintf(f, "%s%d", e ? ", " : "", p->ents_h[ps->ent_begin + e].start_op);
        fprintf(f, "]}");
    }
    fprintf(f, "],\n\"reg_bits\": %d, \"ncoef\": %d, \"segs\": [", p->nprog ? reg_bits(p) : 0, p->ncoef);
    for (int g = 0; g < p->nsegs; g++) {
        fprintf(f, "%s[", g ? ", " : "");
        for (int b = 0; b < 16; b++) fprintf(f, "%s%d", b ? ", " : "", (int)p->segs_h[16 * g + b]);
        fprintf(f, "]");
    }
    fprintf(f, "], \"comb\": [");
    for (int k = 0; k < p->ncomb; k++) {
        fprintf(f, "%s[", k ? ", " : "");
        for (int i = p->comb_ptr_h[k]; i < p->comb_ptr_h[k + 1]; i++)
            fprintf(f, "%s%d", i > p->comb_ptr_h[k] ? ", " : "", p->comb_src_h[i]);
        fprintf(f, "]");
    }
    fprintf(f, "]}\n");
    fclose(f);
    qgt_plan_destroy(p);
    return 0;
}
