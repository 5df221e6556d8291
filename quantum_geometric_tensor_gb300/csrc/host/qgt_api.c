/*
 * qgt_api.c -- the reference library's C entry points on this path, served by
 * GPU plans.
 *
 * Reference behaviour kept: prototypes, struct layouts, return conventions
 * (geometric_* return qgt_error_t, QGTN / gradient functions return bool and
 * set a last-error string), parameter order (k-th parameterised gate in
 * layer -> gate order, src/quantum_geometric/core/quantum_parameter_shift.c:
 * 278-337), output layouts (row-major P x P ComplexFloat; metric imag = 0;
 * curvature +Im Q in .real with Omega_nm = -Omega_mn,
 * src/quantum_geometric/core/quantum_geometric_curvature.c:201-320).
 *
 * Deviations (all corrections of reference defects on this path):
 *   - derivative states are exact (generator insertion); the reference's
 *     (psi(t+pi/16) - psi(t+pi/4))/2 (quantum_geometric_gradient.c:2356-2365)
 *     is not a derivative;
 *   - metric / curvature dimensions are not capped at 16;
 *   - compute_quantum_natural_gradient solves in parameter space and returns
 *     the state-space natural-gradient direction sum_k [(G + lambda I)^-1]_ik
 *     d_k psi (the reference mixes state and parameter indices,
 *     quantum_geometric_gradient.c:1649-1673);
 *   - the last error is thread-local.
 */
#include <math.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../qgt_internal.h"
#include "qgt_gb300.h"
#include "quantum_geometric/core/quantum_gate_operations.h"
#include "quantum_geometric/core/quantum_geometric_curvature.h"
#include "quantum_geometric/core/quantum_geometric_gradient.h"
#include "quantum_geometric/core/quantum_geometric_metric.h"
#include "quantum_geometric/core/quantum_geometric_tensor.h"
#include "quantum_geometric/core/quantum_geometric_tensor_network.h"
#include "quantum_geometric/hybrid/classical_optimization_engine.h"

static _Thread_local const char* g_qgtn_error;
static void set_qgtn_error(const char* e) { g_qgtn_error = e; }
const char* get_quantum_geometric_tensor_network_error(void) { return g_qgtn_error ? g_qgtn_error : "No error"; }

/* ------------------------------------------------------------------------ */
/* gates (quantum_gate_operations.c:10-440)                                  */
/* ------------------------------------------------------------------------ */

static void rotation_matrix(gate_type_t t, double a, ComplexFloat* m)
{
    double c = cos(a / 2.0), s = sin(a / 2.0);
    if (t == GATE_TYPE_RX) { m[0] = (ComplexFloat){(float)c, 0}; m[1] = (ComplexFloat){0, (float)-s}; m[2] = (ComplexFloat){0, (float)-s}; m[3] = (ComplexFloat){(float)c, 0}; }
    else if (t == GATE_TYPE_RY) { m[0] = (ComplexFloat){(float)c, 0}; m[1] = (ComplexFloat){(float)-s, 0}; m[2] = (ComplexFloat){(float)s, 0}; m[3] = (ComplexFloat){(float)c, 0}; }
    else { m[0] = (ComplexFloat){(float)c, (float)-s}; m[1] = (ComplexFloat){0, 0}; m[2] = (ComplexFloat){0, 0}; m[3] = (ComplexFloat){(float)c, (float)s}; }
}

static void fixed_matrix(gate_type_t t, ComplexFloat* m, size_t nq)
{
    size_t d = (size_t)1 << nq;
    for (size_t i = 0; i < d * d; i++) m[i] = (ComplexFloat){0, 0};
    const float r = (float)(1.0 / sqrt(2.0));
    switch (t) {
    case GATE_TYPE_X: m[1].real = 1; m[2].real = 1; break;
    case GATE_TYPE_Y: m[1].imag = -1; m[2].imag = 1; break;
    case GATE_TYPE_Z: m[0].real = 1; m[3].real = -1; break;
    case GATE_TYPE_H: m[0].real = r; m[1].real = r; m[2].real = r; m[3].real = -r; break;
    case GATE_TYPE_S: m[0].real = 1; m[3].imag = 1; break;
    case GATE_TYPE_T: m[0].real = 1; m[3] = (ComplexFloat){r, r}; break;
    case GATE_TYPE_CNOT: m[0].real = 1; m[5].real = 1; m[11].real = 1; m[14].real = 1; break;
    case GATE_TYPE_CZ: m[0].real = 1; m[5].real = 1; m[10].real = 1; m[15].real = -1; break;
    case GATE_TYPE_SWAP: m[0].real = 1; m[6].real = 1; m[9].real = 1; m[15].real = 1; break;
    default: for (size_t i = 0; i < d; i++) m[i * d + i].real = 1; break;
    }
}

quantum_gate_t* create_quantum_gate(gate_type_t type, const size_t* qubits, size_t num_qubits,
                                    const double* parameters, size_t num_parameters)
{
    if (!qubits || num_qubits == 0 || num_qubits > 2 || (parameters == NULL && num_parameters > 0)) return NULL;
    int rot = type == GATE_TYPE_RX || type == GATE_TYPE_RY || type == GATE_TYPE_RZ;
    int two = type == GATE_TYPE_CNOT || type == GATE_TYPE_CZ || type == GATE_TYPE_SWAP;
    if (rot && (num_parameters != 1 || num_qubits != 1)) return NULL;
    if (two && num_qubits != 2) return NULL;
    quantum_gate_t* g = (quantum_gate_t*)calloc(1, sizeof(quantum_gate_t));
    if (!g) return NULL;
    g->type = type;
    g->num_qubits = num_qubits;
    g->target_qubits = (size_t*)malloc(num_qubits * sizeof(size_t));
    g->matrix = (ComplexFloat*)malloc(((size_t)1 << (2 * num_qubits)) * sizeof(ComplexFloat));
    if (!g->target_qubits || !g->matrix) { destroy_quantum_gate(g); return NULL; }
    memcpy(g->target_qubits, qubits, num_qubits * sizeof(size_t));
    g->is_controlled = (type == GATE_TYPE_CNOT || type == GATE_TYPE_CZ);
    if (rot) {
        g->is_parameterized = true;
        g->parameters = (double*)malloc(sizeof(double));
        if (!g->parameters) { destroy_quantum_gate(g); return NULL; }
        g->parameters[0] = parameters[0];
        g->num_parameters = 1;
        rotation_matrix(type, parameters[0], g->matrix);
    } else {
        fixed_matrix(type, g->matrix, num_qubits);
    }
    return g;
}

quantum_gate_t* copy_quantum_gate(const quantum_gate_t* gate)
{
    if (!gate) return NULL;
    quantum_gate_t* g = (quantum_gate_t*)calloc(1, sizeof(quantum_gate_t));
    if (!g) return NULL;
    *g = *gate;
    g->target_qubits = NULL; g->control_qubits = NULL; g->qubits = NULL; g->parameters = NULL; g->matrix = NULL;
    g->custom_data = NULL;
    size_t ms = (size_t)1 << (2 * (gate->num_qubits ? gate->num_qubits : 1));
    g->target_qubits = (size_t*)malloc(sizeof(size_t) * (gate->num_qubits ? gate->num_qubits : 1));
    g->matrix = (ComplexFloat*)calloc(ms, sizeof(ComplexFloat));
    if (!g->target_qubits || !g->matrix) { destroy_quantum_gate(g); return NULL; }
    if (gate->target_qubits) memcpy(g->target_qubits, gate->target_qubits, sizeof(size_t) * gate->num_qubits);
    if (gate->matrix) memcpy(g->matrix, gate->matrix, ms * sizeof(ComplexFloat));
    if (gate->num_controls && gate->control_qubits) {
        g->control_qubits = (size_t*)malloc(sizeof(size_t) * gate->num_controls);
        if (!g->control_qubits) { destroy_quantum_gate(g); return NULL; }
        memcpy(g->control_qubits, gate->control_qubits, sizeof(size_t) * gate->num_controls);
    }
    if (gate->qubits && gate->num_qubits) {
        g->qubits = (size_t*)malloc(sizeof(size_t) * gate->num_qubits);
        if (!g->qubits) { destroy_quantum_gate(g); return NULL; }
        memcpy(g->qubits, gate->qubits, sizeof(size_t) * gate->num_qubits);
    }
    if (gate->num_parameters && gate->parameters) {
        g->parameters = (double*)malloc(sizeof(double) * gate->num_parameters);
        if (!g->parameters) { destroy_quantum_gate(g); return NULL; }
        memcpy(g->parameters, gate->parameters, sizeof(double) * gate->num_parameters);
    }
    return g;
}

void destroy_quantum_gate(quantum_gate_t* g)
{
    if (!g) return;
    free(g->matrix); free(g->target_qubits); free(g->control_qubits); free(g->qubits); free(g->parameters);
    free(g);
}

bool update_gate_parameters(quantum_gate_t* g, const double* p, size_t np)
{
    if (!g || !p || !g->is_parameterized || np != g->num_parameters || !g->parameters) return false;
    memcpy(g->parameters, p, np * sizeof(double));
    if (g->matrix) rotation_matrix(g->type, p[0], g->matrix);
    return true;
}

bool shift_gate_parameters(quantum_gate_t* g, size_t idx, double shift)
{
    if (!g || !g->parameters || idx >= g->num_parameters) return false;
    double v = g->parameters[idx] + shift;
    return update_gate_parameters(g, &v, 1);
}

#define ONEQ(name, T) quantum_gate_t* name(size_t q) { size_t qs[1] = {q}; return create_quantum_gate(T, qs, 1, NULL, 0); }
#define ROTQ(name, T) quantum_gate_t* name(size_t q, double a) { size_t qs[1] = {q}; return create_quantum_gate(T, qs, 1, &a, 1); }
ROTQ(create_rx_gate, GATE_TYPE_RX)
ROTQ(create_ry_gate, GATE_TYPE_RY)
ROTQ(create_rz_gate, GATE_TYPE_RZ)
ONEQ(create_h_gate, GATE_TYPE_H)
ONEQ(create_x_gate, GATE_TYPE_X)
ONEQ(create_y_gate, GATE_TYPE_Y)
ONEQ(create_z_gate, GATE_TYPE_Z)
quantum_gate_t* create_cnot_gate(size_t c, size_t t) { size_t qs[2] = {c, t}; return create_quantum_gate(GATE_TYPE_CNOT, qs, 2, NULL, 0); }
quantum_gate_t* create_cz_gate(size_t c, size_t t) { size_t qs[2] = {c, t}; return create_quantum_gate(GATE_TYPE_CZ, qs, 2, NULL, 0); }

/* ------------------------------------------------------------------------ */
/* QGTN object                                                               */
/* ------------------------------------------------------------------------ */

typedef struct {
    int precision;
    uint64_t version;            /* bumped on every circuit change */
    /* GPU plan for the QGT (selected precision) and an FP64 plan for states */
    qgt_plan_t* plan;
    uint64_t plan_version;
    qgt_plan_t* plan64;
    uint64_t plan64_version;
    int have_q;
    double* theta_q;             /* theta of the cached Q */
    double* Q;                   /* P x P complex of the cached step */
    int have_run64;
    double* theta64;
    int P;
} qgtn_backend_t;

static qgtn_backend_t* backend(const quantum_geometric_tensor_network_t* q)
{
    return (qgtn_backend_t*)q->backend_state;
}

static void backend_free(qgtn_backend_t* b)
{
    if (!b) return;
    qgt_plan_destroy(b->plan);
    qgt_plan_destroy(b->plan64);
    free(b->theta_q); free(b->Q); free(b->theta64);
    free(b);
}

static circuit_layer_t* new_layer(void)
{
    circuit_layer_t* l = (circuit_layer_t*)calloc(1, sizeof(circuit_layer_t));
    if (!l) return NULL;
    l->gates = (quantum_gate_t**)calloc(16, sizeof(quantum_gate_t*));
    if (!l->gates) { free(l); return NULL; }
    return l;
}

quantum_geometric_tensor_network_t* create_quantum_geometric_tensor_network(size_t num_qubits, size_t num_layers,
                                                                           bool is_distributed, bool use_hw)
{
    if (num_qubits == 0 || num_qubits > QGT_MAX_QUBITS) { set_qgtn_error("num_qubits must be in [1, 30]"); return NULL; }
    quantum_geometric_tensor_network_t* q = (quantum_geometric_tensor_network_t*)calloc(1, sizeof(*q));
    qgtn_backend_t* b = (qgtn_backend_t*)calloc(1, sizeof(qgtn_backend_t));
    quantum_circuit_t* c = (quantum_circuit_t*)calloc(1, sizeof(quantum_circuit_t));
    size_t nl = num_layers > 0 ? num_layers : 1;
    if (q && c) c->layers = (circuit_layer_t**)calloc(nl, sizeof(circuit_layer_t*));
    if (!q || !b || !c || !c->layers) {
        free(q); free(b); if (c) free(c->layers); free(c);
        set_qgtn_error("Failed to allocate quantum geometric tensor network");
        return NULL;
    }
    c->num_qubits = num_qubits;
    c->num_layers = nl;
    c->layers_capacity = nl;
    for (size_t l = 0; l < nl; l++) {
        c->layers[l] = new_layer();
        if (!c->layers[l]) {
            for (size_t k = 0; k < l; k++) { free(c->layers[k]->gates); free(c->layers[k]); }
            free(c->layers); free(c); free(q); free(b);
            set_qgtn_error("Failed to allocate circuit layer");
            return NULL;
        }
    }
    q->circuit = c;
    q->num_qubits = num_qubits;
    q->num_layers = nl;
    q->is_distributed = is_distributed;
    q->use_hardware_acceleration = true;
    (void)use_hw;
    q->hardware_config.type = QGTN_BACKEND_SIMULATOR;
    q->hardware_config.supports_gradients = true;
    q->hardware_config.supports_hybrid = true;
    b->precision = QGT_PRECISION_FP64;
    q->backend_state = b;
    return q;
}

void destroy_quantum_geometric_tensor_network(quantum_geometric_tensor_network_t* q)
{
    if (!q) return;
    if (q->circuit) {
        for (size_t l = 0; l < q->circuit->num_layers; l++) {
            circuit_layer_t* L = q->circuit->layers[l];
            if (!L) continue;
            for (size_t g = 0; g < L->num_gates; g++) destroy_quantum_gate(L->gates[g]);
            free(L->gates);
            free(L);
        }
        free(q->circuit->layers);
        free(q->circuit);
    }
    backend_free(backend(q));
    free(q);
}

static bool layer_append(circuit_layer_t* L, quantum_gate_t* g)
{
    if (L->num_gates >= 16 && (L->num_gates & (L->num_gates - 1)) == 0) {
        quantum_gate_t** ng = (quantum_gate_t**)realloc(L->gates, sizeof(quantum_gate_t*) * L->num_gates * 2);
        if (!ng) return false;
        L->gates = ng;
    }
    L->gates[L->num_gates++] = g;
    if (g->is_parameterized) L->is_parameterized = true;
    return true;
}

quantum_geometric_tensor_network_t* copy_quantum_geometric_tensor_network(const quantum_geometric_tensor_network_t* q)
{
    if (!q || !q->circuit) { set_qgtn_error("Invalid network to copy"); return NULL; }
    quantum_geometric_tensor_network_t* r =
        create_quantum_geometric_tensor_network(q->num_qubits, q->num_layers, q->is_distributed, true);
    if (!r) return NULL;
    backend(r)->precision = backend(q)->precision;
    for (size_t l = 0; l < q->circuit->num_layers; l++) {
        circuit_layer_t* L = q->circuit->layers[l];
        if (!L) continue;
        for (size_t g = 0; g < L->num_gates; g++) {
            quantum_gate_t* cg = copy_quantum_gate(L->gates[g]);
            if (!cg || !layer_append(r->circuit->layers[l], cg)) {
                destroy_quantum_gate(cg);
                destroy_quantum_geometric_tensor_network(r);
                set_qgtn_error("Failed to copy gate");
                return NULL;
            }
        }
    }
    r->circuit->is_parameterized = q->circuit->is_parameterized;
    return r;
}

bool apply_quantum_gate(quantum_geometric_tensor_network_t* q, const quantum_gate_t* gate, const size_t* qubits,
                        size_t nq)
{
    if (!q || !gate || !qubits || nq == 0) { set_qgtn_error("Invalid arguments to apply_quantum_gate"); return false; }
    if (!q->circuit || !q->circuit->layers) { set_qgtn_error("Circuit not initialized"); return false; }
    for (size_t i = 0; i < nq; i++)
        if (qubits[i] >= q->num_qubits) { set_qgtn_error("Qubit index out of range"); return false; }
    if ((gate->type == GATE_TYPE_RX || gate->type == GATE_TYPE_RY || gate->type == GATE_TYPE_RZ)) {
        if (!gate->is_parameterized || !gate->parameters) { set_qgtn_error("Invalid rotation gate parameters"); return false; }
        if (!isfinite(gate->parameters[0])) { set_qgtn_error("Invalid rotation matrix values"); return false; }
    }
    size_t layer = q->num_layers > 0 ? q->num_layers - 1 : 0;
    quantum_gate_t* cg = copy_quantum_gate(gate);
    if (!cg) { set_qgtn_error("Failed to copy quantum gate"); return false; }
    free(cg->qubits);
    cg->qubits = (size_t*)malloc(sizeof(size_t) * nq);
    if (!cg->qubits) { destroy_quantum_gate(cg); set_qgtn_error("Failed to copy quantum gate"); return false; }
    memcpy(cg->qubits, qubits, sizeof(size_t) * nq);
    if (!layer_append(q->circuit->layers[layer], cg)) {
        destroy_quantum_gate(cg);
        set_qgtn_error("Failed to resize gates array");
        return false;
    }
    if (cg->is_parameterized) q->circuit->is_parameterized = true;
    backend(q)->version++;
    return true;
}

bool apply_quantum_circuit(quantum_geometric_tensor_network_t* q, const quantum_circuit_t* circuit)
{
    if (!q || !circuit) { set_qgtn_error("Invalid arguments to apply_quantum_circuit"); return false; }
    for (size_t l = 0; l < circuit->num_layers; l++) {
        circuit_layer_t* L = circuit->layers ? circuit->layers[l] : NULL;
        if (!L) continue;
        for (size_t g = 0; g < L->num_gates; g++) {
            const quantum_gate_t* gt = L->gates[g];
            if (!gt) continue;
            const size_t* qs = gt->qubits ? gt->qubits : gt->target_qubits;
            if (!apply_quantum_gate(q, gt, qs, gt->num_qubits)) return false;
        }
    }
    for (size_t g = 0; g < circuit->num_gates; g++) {
        const quantum_gate_t* gt = circuit->gates ? circuit->gates[g] : NULL;
        if (!gt) continue;
        const size_t* qs = gt->qubits ? gt->qubits : gt->target_qubits;
        if (!apply_quantum_gate(q, gt, qs, gt->num_qubits)) return false;
    }
    return true;
}

size_t count_trainable_parameters(const quantum_geometric_tensor_network_t* q)
{
    if (!q || !q->circuit) return 0;
    size_t c = 0;
    for (size_t l = 0; l < q->num_layers; l++) {
        circuit_layer_t* L = q->circuit->layers ? q->circuit->layers[l] : NULL;
        if (!L) continue;
        for (size_t g = 0; g < L->num_gates; g++)
            if (L->gates[g] && L->gates[g]->is_parameterized && L->gates[g]->parameters) c += L->gates[g]->num_parameters;
    }
    return c;
}

/* circuit -> (gate descriptors, theta) in layer -> gate order */
static int extract(const quantum_geometric_tensor_network_t* q, qgt_gate_desc_t** gates, int* ng, double** theta, int* P)
{
    size_t total = 0;
    for (size_t l = 0; l < q->num_layers; l++) if (q->circuit->layers[l]) total += q->circuit->layers[l]->num_gates;
    qgt_gate_desc_t* gd = (qgt_gate_desc_t*)calloc(total + 1, sizeof(qgt_gate_desc_t));
    double* th = (double*)calloc(total + 1, sizeof(double));
    if (!gd || !th) { free(gd); free(th); return -2; }
    int k = 0, p = 0;
    for (size_t l = 0; l < q->num_layers; l++) {
        circuit_layer_t* L = q->circuit->layers[l];
        if (!L) continue;
        for (size_t g = 0; g < L->num_gates; g++) {
            const quantum_gate_t* gt = L->gates[g];
            if (!gt) continue;
            const size_t* qs = gt->qubits ? gt->qubits : gt->target_qubits;
            qgt_gate_desc_t* d = &gd[k];
            d->type = (int32_t)gt->type;
            d->param = -1;
            d->qubits[1] = -1;
            if (gt->type == GATE_TYPE_CNOT || gt->type == GATE_TYPE_CZ || gt->type == GATE_TYPE_SWAP) {
                if (gt->num_controls > 0 && gt->control_qubits && gt->num_qubits == 1) {
                    d->qubits[0] = (int32_t)gt->control_qubits[0];
                    d->qubits[1] = (int32_t)qs[0];
                } else if (gt->num_qubits >= 2) {
                    d->qubits[0] = (int32_t)qs[0];
                    d->qubits[1] = (int32_t)qs[1];
                } else { free(gd); free(th); return -1; }
            } else {
                d->qubits[0] = (int32_t)qs[0];
            }
            if (gt->is_parameterized && gt->parameters &&
                (gt->type == GATE_TYPE_RX || gt->type == GATE_TYPE_RY || gt->type == GATE_TYPE_RZ)) {
                d->param = p;
                th[p++] = gt->parameters[0];
            }
            k++;
        }
    }
    *gates = gd; *ng = k; *theta = th; *P = p;
    return 0;
}

/* build / refresh the plan(s) and run one step when the circuit or theta changed */
static bool ensure_step(const quantum_geometric_tensor_network_t* q, int want64)
{
    qgtn_backend_t* b = backend(q);
    if (!b || !q->circuit) { set_qgtn_error("Network not initialized"); return false; }
    qgt_gate_desc_t* gd = NULL;
    double* th = NULL;
    int ng = 0, P = 0;
    if (extract(q, &gd, &ng, &th, &P) != 0) { set_qgtn_error("Unsupported gate in circuit"); return false; }
    qgt_circuit_desc_t cd = {(int32_t)q->num_qubits, ng, gd, P};
    qgt_plan_options_t o;
    qgt_plan_default_options(&o);
    o.hamiltonian = QGT_HAMILTONIAN_NONE;
    bool ok = true;
    qgt_plan_t** pp = want64 ? &b->plan64 : &b->plan;
    uint64_t* pv = want64 ? &b->plan64_version : &b->plan_version;
    o.precision = want64 ? QGT_PRECISION_FP64 : (qgt_precision_t)b->precision;
    /* the integer-digit Gram walks amplitudes 16 at a time: registers below
       4 qubits (fewer than 16 amplitudes) run the FP64 plan instead */
    if (o.precision == QGT_PRECISION_MIXED && q->num_qubits < 4) o.precision = QGT_PRECISION_FP64;
    if (!*pp || *pv != b->version + 1) {
        qgt_plan_destroy(*pp);
        *pp = NULL;
        if (qgt_plan_create(&cd, &o, pp) != 0) { set_qgtn_error(qgt_last_error()); ok = false; }
        *pv = b->version + 1;
        if (want64) b->have_run64 = 0; else b->have_q = 0;
    }
    if (ok && P != b->P) {
        free(b->theta_q); free(b->Q); free(b->theta64);
        b->theta_q = (double*)calloc((size_t)P + 1, sizeof(double));
        b->theta64 = (double*)calloc((size_t)P + 1, sizeof(double));
        b->Q = (double*)calloc(2 * (size_t)P * P + 2, sizeof(double));
        b->P = P;
        b->have_q = 0;
        b->have_run64 = 0;
        if (!b->theta_q || !b->Q || !b->theta64) { set_qgtn_error("Out of memory"); ok = false; }
    }
    if (ok) {
        if (want64) {
            if (!b->have_run64 || memcmp(b->theta64, th, sizeof(double) * (size_t)P) != 0) {
                if (qgt_plan_execute_host(*pp, th, NULL, NULL, NULL, NULL) != 0) { set_qgtn_error(qgt_last_error()); ok = false; }
                else { memcpy(b->theta64, th, sizeof(double) * (size_t)P); b->have_run64 = 1; }
            }
        } else if (!b->have_q || memcmp(b->theta_q, th, sizeof(double) * (size_t)P) != 0) {
            if (qgt_plan_execute_host(*pp, th, b->Q, NULL, NULL, NULL) != 0) { set_qgtn_error(qgt_last_error()); ok = false; }
            else { memcpy(b->theta_q, th, sizeof(double) * (size_t)P); b->have_q = 1; }
        }
    }
    free(gd);
    free(th);
    return ok;
}

bool qgtn_set_precision(quantum_geometric_tensor_network_t* q, int precision)
{
    if (!q || precision < 0 || precision > 2) return false;
    backend(q)->precision = precision;
    backend(q)->version++;
    return true;
}

bool get_quantum_state(const quantum_geometric_tensor_network_t* q, ComplexFloat** sv, size_t* dim)
{
    if (!q || !sv || !dim) { set_qgtn_error("Invalid arguments to get_quantum_state"); return false; }
    if (!ensure_step(q, 1)) return false;
    size_t N = (size_t)1 << q->num_qubits;
    double* psi = (double*)malloc(sizeof(double) * 2 * N);
    ComplexFloat* out = (ComplexFloat*)malloc(sizeof(ComplexFloat) * N);
    if (!psi || !out || qgt_plan_get_state(backend(q)->plan64, psi) != 0) {
        free(psi); free(out);
        set_qgtn_error("Failed to read the state");
        return false;
    }
    for (size_t i = 0; i < N; i++) out[i] = (ComplexFloat){(float)psi[2 * i], (float)psi[2 * i + 1]};
    free(psi);
    *sv = out;
    *dim = N;
    return true;
}

bool qgtn_measure_qubit(const quantum_geometric_tensor_network_t* q, size_t qubit, double* p0, double* p1)
{
    if (!q || !p0 || !p1 || qubit >= q->num_qubits) { set_qgtn_error("Invalid arguments to qgtn_measure_qubit"); return false; }
    if (!ensure_step(q, 1)) return false;
    size_t N = (size_t)1 << q->num_qubits;
    double* psi = (double*)malloc(sizeof(double) * 2 * N);
    if (!psi || qgt_plan_get_state(backend(q)->plan64, psi) != 0) { free(psi); set_qgtn_error("Failed to read the state"); return false; }
    double a = 0, c = 0;
    for (size_t i = 0; i < N; i++) {
        double w = psi[2 * i] * psi[2 * i] + psi[2 * i + 1] * psi[2 * i + 1];
        if ((i >> qubit) & 1) c += w; else a += w;
    }
    free(psi);
    double t = a + c;
    *p0 = t > 0 ? a / t : 0;
    *p1 = t > 0 ? c / t : 0;
    return true;
}

bool compute_quantum_geometric_tensor(const quantum_geometric_tensor_network_t* q, size_t i, size_t j, ComplexFloat* r)
{
    if (!q || !r) { set_qgtn_error("Invalid arguments to compute_quantum_geometric_tensor"); return false; }
    if (!ensure_step(q, 0)) return false;
    qgtn_backend_t* b = backend(q);
    if (i >= (size_t)b->P || j >= (size_t)b->P) { set_qgtn_error("Parameter index out of range"); return false; }
    size_t at = 2 * (i * (size_t)b->P + j);
    r->real = (float)b->Q[at];
    r->imag = (float)b->Q[at + 1];
    return true;
}

static bool q_element(const quantum_geometric_tensor_network_t* q, size_t i, size_t j, double* re, double* im)
{
    if (!ensure_step(q, 0)) return false;
    qgtn_backend_t* b = backend(q);
    if (i >= (size_t)b->P || j >= (size_t)b->P) { set_qgtn_error("Parameter index out of range"); return false; }
    size_t at = 2 * (i * (size_t)b->P + j);
    if (re) *re = b->Q[at];
    if (im) *im = b->Q[at + 1];
    return true;
}

bool compute_quantum_metric(const quantum_geometric_tensor_network_t* q, size_t i, size_t j, double* r)
{
    if (!q || !r) { set_qgtn_error("Invalid arguments to compute_quantum_metric"); return false; }
    return q_element(q, i, j, r, NULL);
}

bool compute_berry_curvature(const quantum_geometric_tensor_network_t* q, size_t i, size_t j, double* r)
{
    if (!q || !r) { set_qgtn_error("Invalid arguments to compute_berry_curvature"); return false; }
    return q_element(q, i, j, NULL, r);
}

bool distribute_computation(quantum_geometric_tensor_network_t* q, const size_t* ids, size_t n)
{
    /* one GPU per process: a network runs on one device */
    if (!q || !ids || n == 0) { set_qgtn_error("Invalid arguments to distribute_computation"); return false; }
    q->is_distributed = false;
    return true;
}

bool synchronize_distributed_state(quantum_geometric_tensor_network_t* q) { return q != NULL; }

bool enable_hardware_acceleration(quantum_geometric_tensor_network_t* q, HardwareType t)
{
    if (!q) return false;
    (void)t;
    q->use_hardware_acceleration = true;
    return true;
}

bool disable_hardware_acceleration(quantum_geometric_tensor_network_t* q)
{
    /* there is no CPU path: the GPU stays the only backend */
    if (!q) return false;
    set_qgtn_error("This library has no CPU backend; hardware acceleration stays on");
    return false;
}

/* ------------------------------------------------------------------------ */
/* metric / curvature / tensor objects                                       */
/* ------------------------------------------------------------------------ */

#define CHECK_NULL(p) do { if (!(p)) return QGT_ERROR_INVALID_ARGUMENT; } while (0)

qgt_error_t geometric_create_metric(quantum_geometric_metric_t** m, geometric_metric_type_t type, size_t dim)
{
    CHECK_NULL(m);
    if (dim == 0 || dim > QGT_MAX_PARAMETERS) return QGT_ERROR_INVALID_ARGUMENT;
    if (type != GEOMETRIC_METRIC_EUCLIDEAN && type != GEOMETRIC_METRIC_MINKOWSKI && type != GEOMETRIC_METRIC_FUBINI_STUDY)
        return QGT_ERROR_INVALID_ARGUMENT;
    quantum_geometric_metric_t* r = (quantum_geometric_metric_t*)calloc(1, sizeof(*r));
    if (!r) return QGT_ERROR_ALLOCATION_FAILED;
    r->components = (ComplexFloat*)calloc(dim * dim, sizeof(ComplexFloat));
    if (!r->components) { free(r); return QGT_ERROR_ALLOCATION_FAILED; }
    r->type = type;
    r->dimension = dim;
    r->is_symmetric = true;
    r->hardware = HARDWARE_TYPE_GPU;
    for (size_t i = 0; i < dim; i++)
        r->components[i * dim + i].real = (type == GEOMETRIC_METRIC_MINKOWSKI && i == 0) ? -1.0f : 1.0f;
    *m = r;
    return QGT_SUCCESS;
}

void geometric_destroy_metric(quantum_geometric_metric_t* m)
{
    if (!m) return;
    free(m->components);
    free(m);
}

qgt_error_t geometric_clone_metric(quantum_geometric_metric_t** d, const quantum_geometric_metric_t* s)
{
    CHECK_NULL(d); CHECK_NULL(s);
    qgt_error_t e = geometric_create_metric(d, s->type, s->dimension);
    if (e) return e;
    memcpy((*d)->components, s->components, sizeof(ComplexFloat) * s->dimension * s->dimension);
    (*d)->is_symmetric = s->is_symmetric;
    return QGT_SUCCESS;
}

/* The state-space metric of geometric_compute_metric
 * (src/quantum_geometric/core/quantum_geometric_metric.c:85-189): Euclidean
 * leaves the components as they are; Fubini-Study writes
 * M_ij = delta_ij - conj(psi_i) psi_j for the state's amplitudes (computed
 * on the GPU); other types are not implemented, as in the reference. */
qgt_error_t geometric_compute_metric(quantum_geometric_metric_t* m, const quantum_state_t* state)
{
    CHECK_NULL(m); CHECK_NULL(state);
    if (m->dimension != state->dimension) return QGT_ERROR_INVALID_ARGUMENT;
    switch (m->type) {
    case GEOMETRIC_METRIC_EUCLIDEAN:
        return QGT_SUCCESS;
    case GEOMETRIC_METRIC_FUBINI_STUDY:
        CHECK_NULL(state->coordinates);
        CHECK_NULL(m->components);
        if (qgt_dev_fs_metric((const float*)state->coordinates, (int64_t)m->dimension, (float*)m->components) != 0)
            return QGT_ERROR_COMPUTATION_FAILED;
        return QGT_SUCCESS;
    default:
        return QGT_ERROR_NOT_IMPLEMENTED;
    }
}

static qgt_error_t full_q(const quantum_geometric_tensor_network_t* q, size_t P, const double** Q)
{
    if (!ensure_step(q, 0)) return QGT_ERROR_COMPUTATION_FAILED;
    if ((size_t)backend(q)->P != P) return QGT_ERROR_DIMENSION_MISMATCH;
    *Q = backend(q)->Q;
    return QGT_SUCCESS;
}

qgt_error_t geometric_compute_fubini_study_metric(quantum_geometric_metric_t* m,
                                                  const quantum_geometric_tensor_network_t* q, size_t P)
{
    CHECK_NULL(m); CHECK_NULL(q);
    if (P == 0) return QGT_ERROR_INVALID_ARGUMENT;
    if (m->type != GEOMETRIC_METRIC_FUBINI_STUDY) return QGT_ERROR_INVALID_ARGUMENT;
    if (m->dimension != P) return QGT_ERROR_DIMENSION_MISMATCH;
    const double* Q;
    qgt_error_t e = full_q(q, P, &Q);
    if (e) return e;
    for (size_t i = 0; i < P; i++)
        for (size_t j = 0; j < P; j++) {
            /* symmetric by construction: average the two mirrored entries */
            double g = 0.5 * (Q[2 * (i * P + j)] + Q[2 * (j * P + i)]);
            m->components[i * P + j] = (ComplexFloat){(float)g, 0.0f};
        }
    m->is_symmetric = true;
    return QGT_SUCCESS;
}

qgt_error_t geometric_compute_fubini_study_element(const quantum_geometric_tensor_network_t* q, size_t mu, size_t nu,
                                                   float* r)
{
    CHECK_NULL(q); CHECK_NULL(r);
    double v;
    if (!compute_quantum_metric(q, mu, nu, &v)) return QGT_ERROR_COMPUTATION_FAILED;
    *r = (float)v;
    return QGT_SUCCESS;
}

qgt_error_t geometric_create_curvature(quantum_geometric_curvature_t** c, geometric_curvature_type_t type, size_t dim)
{
    CHECK_NULL(c);
    if (dim == 0 || dim > QGT_MAX_PARAMETERS) return QGT_ERROR_INVALID_ARGUMENT;
    size_t n = type == GEOMETRIC_CURVATURE_BERRY ? dim * dim : dim * dim * dim * dim;
    if (type != GEOMETRIC_CURVATURE_BERRY && dim > 256) return QGT_ERROR_INVALID_ARGUMENT;
    quantum_geometric_curvature_t* r = (quantum_geometric_curvature_t*)calloc(1, sizeof(*r));
    if (!r) return QGT_ERROR_ALLOCATION_FAILED;
    r->components = (ComplexFloat*)calloc(n, sizeof(ComplexFloat));
    if (!r->components) { free(r); return QGT_ERROR_ALLOCATION_FAILED; }
    r->type = type;
    r->dimension = dim;
    r->is_flat = true;
    r->hardware = HARDWARE_TYPE_GPU;
    *c = r;
    return QGT_SUCCESS;
}

void geometric_destroy_curvature(quantum_geometric_curvature_t* c)
{
    if (!c) return;
    free(c->components);
    free(c);
}

qgt_error_t geometric_clone_curvature(quantum_geometric_curvature_t** d, const quantum_geometric_curvature_t* s)
{
    CHECK_NULL(d); CHECK_NULL(s);
    qgt_error_t e = geometric_create_curvature(d, s->type, s->dimension);
    if (e) return e;
    size_t n = s->type == GEOMETRIC_CURVATURE_BERRY ? s->dimension * s->dimension
                                                    : s->dimension * s->dimension * s->dimension * s->dimension;
    memcpy((*d)->components, s->components, sizeof(ComplexFloat) * n);
    (*d)->is_flat = s->is_flat;
    return QGT_SUCCESS;
}

qgt_error_t geometric_compute_berry_curvature(quantum_geometric_curvature_t* c,
                                              const quantum_geometric_tensor_network_t* q, size_t P)
{
    CHECK_NULL(c); CHECK_NULL(q);
    if (P == 0) return QGT_ERROR_INVALID_ARGUMENT;
    if (c->type != GEOMETRIC_CURVATURE_BERRY) return QGT_ERROR_INVALID_ARGUMENT;
    if (c->dimension != P) return QGT_ERROR_DIMENSION_MISMATCH;
    const double* Q;
    qgt_error_t e = full_q(q, P, &Q);
    if (e) return e;
    for (size_t i = 0; i < P; i++) {
        c->components[i * P + i] = (ComplexFloat){0, 0};
        for (size_t j = i + 1; j < P; j++) {
            double w = 0.5 * (Q[2 * (i * P + j) + 1] - Q[2 * (j * P + i) + 1]);
            c->components[i * P + j] = (ComplexFloat){(float)w, 0};
            c->components[j * P + i] = (ComplexFloat){(float)-w, 0};
        }
    }
    c->is_flat = false;
    return QGT_SUCCESS;
}

qgt_error_t geometric_compute_berry_curvature_element(const quantum_geometric_tensor_network_t* q, size_t mu,
                                                      size_t nu, float* r)
{
    CHECK_NULL(q); CHECK_NULL(r);
    double v;
    if (!compute_berry_curvature(q, mu, nu, &v)) return QGT_ERROR_COMPUTATION_FAILED;
    *r = (float)v;
    return QGT_SUCCESS;
}

qgt_error_t geometric_compose_qgt(ComplexFloat* qgt, const quantum_geometric_metric_t* m,
                                  const quantum_geometric_curvature_t* c, size_t dim)
{
    CHECK_NULL(qgt); CHECK_NULL(m); CHECK_NULL(c);
    if (m->dimension != dim || c->dimension != dim) return QGT_ERROR_DIMENSION_MISMATCH;
    if (m->type != GEOMETRIC_METRIC_FUBINI_STUDY || c->type != GEOMETRIC_CURVATURE_BERRY) return QGT_ERROR_INVALID_ARGUMENT;
    for (size_t i = 0; i < dim * dim; i++) qgt[i] = (ComplexFloat){m->components[i].real, c->components[i].real};
    return QGT_SUCCESS;
}

qgt_error_t geometric_compute_full_qgt(ComplexFloat* qgt, const quantum_geometric_tensor_network_t* q, size_t P)
{
    CHECK_NULL(qgt); CHECK_NULL(q);
    if (P == 0) return QGT_ERROR_INVALID_ARGUMENT;
    const double* Q;
    qgt_error_t e = full_q(q, P, &Q);
    if (e) return e;
    for (size_t i = 0; i < P; i++)
        for (size_t j = i; j < P; j++) {
            double re = 0.5 * (Q[2 * (i * P + j)] + Q[2 * (j * P + i)]);
            double im = 0.5 * (Q[2 * (i * P + j) + 1] - Q[2 * (j * P + i) + 1]);
            qgt[i * P + j] = (ComplexFloat){(float)re, (float)(i == j ? 0.0 : im)};
            if (j != i) qgt[j * P + i] = (ComplexFloat){(float)re, (float)-im};
        }
    return QGT_SUCCESS;
}

static qgt_error_t validate_dims(const size_t* d, size_t rank, size_t* total)
{
    if (!d || rank == 0) return QGT_ERROR_INVALID_PARAMETER;
    size_t t = 1;
    for (size_t i = 0; i < rank; i++) {
        if (d[i] == 0) return QGT_ERROR_INVALID_PARAMETER;
        if (t > SIZE_MAX / d[i]) return QGT_ERROR_INVALID_PARAMETER;
        t *= d[i];
    }
    *total = t;
    return QGT_SUCCESS;
}

qgt_error_t geometric_tensor_create(quantum_geometric_tensor_t** t, geometric_tensor_type_t type, const size_t* dims,
                                    size_t rank)
{
    if (!t) return QGT_ERROR_INVALID_PARAMETER;
    size_t total;
    qgt_error_t e = validate_dims(dims, rank, &total);
    if (e) return e;
    size_t aligned = (total + 7) & ~(size_t)7;
    quantum_geometric_tensor_t* r = (quantum_geometric_tensor_t*)calloc(1, sizeof(*r));
    if (!r) return QGT_ERROR_MEMORY_ALLOCATION;
    r->dimensions = (size_t*)malloc(rank * sizeof(size_t));
    r->components = (ComplexFloat*)aligned_alloc(64, aligned * sizeof(ComplexFloat));
    if (!r->dimensions || !r->components) { free(r->dimensions); free(r->components); free(r); return QGT_ERROR_MEMORY_ALLOCATION; }
    memset(r->components, 0, aligned * sizeof(ComplexFloat));
    memcpy(r->dimensions, dims, rank * sizeof(size_t));
    r->rank = rank;
    r->dimension = dims[0];
    r->total_elements = total;
    r->aligned_elements = aligned;
    r->type = type;
    r->hardware = HARDWARE_TYPE_SIMULATOR;
    switch (type) {
    case GEOMETRIC_TENSOR_SYMMETRIC: case GEOMETRIC_TENSOR_SCALAR: r->is_symmetric = true; r->is_hermitian = true; break;
    case GEOMETRIC_TENSOR_UNITARY: r->is_unitary = true; break;
    case GEOMETRIC_TENSOR_HERMITIAN: r->is_hermitian = true; break;
    case GEOMETRIC_TENSOR_BIVECTOR: case GEOMETRIC_TENSOR_TRIVECTOR: r->is_symmetric = true; break;
    default: break;
    }
    *t = r;
    return QGT_SUCCESS;
}

void geometric_tensor_destroy(quantum_geometric_tensor_t* t)
{
    if (!t) return;
    free(t->dimensions);
    free(t->components);
    free(t->auxiliary_data);
    free(t);
}

qgt_error_t geometric_tensor_clone(quantum_geometric_tensor_t** d, const quantum_geometric_tensor_t* s)
{
    if (!d || !s) return QGT_ERROR_INVALID_PARAMETER;
    qgt_error_t e = geometric_tensor_create(d, s->type, s->dimensions, s->rank);
    if (e) return e;
    memcpy((*d)->components, s->components, s->total_elements * sizeof(ComplexFloat));
    (*d)->is_symmetric = s->is_symmetric;
    (*d)->is_unitary = s->is_unitary;
    (*d)->is_hermitian = s->is_hermitian;
    return QGT_SUCCESS;
}

qgt_error_t geometric_tensor_initialize(quantum_geometric_tensor_t* t, const ComplexFloat* data)
{
    if (!t || !data || !t->components) return QGT_ERROR_INVALID_PARAMETER;
    memcpy(t->components, data, t->total_elements * sizeof(ComplexFloat));
    return QGT_SUCCESS;
}

qgt_error_t geometric_tensor_initialize_zero(quantum_geometric_tensor_t* t)
{
    if (!t || !t->components) return QGT_ERROR_INVALID_PARAMETER;
    memset(t->components, 0, t->aligned_elements * sizeof(ComplexFloat));
    return QGT_SUCCESS;
}

/* uniform double in [0, 1) from a splitmix64 stream (53 random bits) */
static double tensor_uniform(uint64_t* state)
{
    uint64_t z = (*state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

/* The reference fills from its entropy-seeded QRNG
 * (src/quantum_geometric/core/quantum_geometric_tensor.c:257-340): every
 * element (re, im) uniform in [min, max) scaled to unit modulus; a rank-2
 * Hermitian tensor gets a real uniform diagonal and unit-modulus upper
 * entries mirrored as conjugates.  Here the stream is splitmix64, seeded
 * differently on every call (clock and a per-process counter), so the values
 * are as unrepeatable as the reference's. */
qgt_error_t geometric_tensor_initialize_random(quantum_geometric_tensor_t* t, float min_val, float max_val)
{
    if (!t || !t->components) return QGT_ERROR_INVALID_ARGUMENT;
    if (!(min_val < max_val)) return QGT_ERROR_INVALID_ARGUMENT;
    static uint64_t calls = 0;
    struct timespec ts;
    clock_gettime(CLOCK_REALTIME, &ts);
    uint64_t st = ((uint64_t)ts.tv_sec * 1000000007ULL) ^ (uint64_t)ts.tv_nsec ^
                  (__atomic_add_fetch(&calls, 1, __ATOMIC_RELAXED) * 0xD1B54A32D192ED03ULL) ^ (uint64_t)(uintptr_t)t;
    const float range = max_val - min_val;
    ComplexFloat* d = t->components;
    if (t->type == GEOMETRIC_TENSOR_HERMITIAN && t->rank == 2) {
        const size_t n = t->dimensions[0];
        for (size_t i = 0; i < n; i++)
            for (size_t j = i; j < n; j++) {
                float re = min_val + (float)tensor_uniform(&st) * range;
                if (i == j) { d[i * n + i] = (ComplexFloat){re, 0.0f}; continue; }
                float im = min_val + (float)tensor_uniform(&st) * range;
                const float m = sqrtf(re * re + im * im);
                if (m > 0) { re /= m; im /= m; }
                d[i * n + j] = (ComplexFloat){re, im};
                d[j * n + i] = (ComplexFloat){re, -im};
            }
    } else {
        for (size_t i = 0; i < t->total_elements; i++) {
            float re = min_val + (float)tensor_uniform(&st) * range;
            float im = min_val + (float)tensor_uniform(&st) * range;
            const float m = sqrtf(re * re + im * im);
            if (m > 0) { re /= m; im /= m; }
            d[i] = (ComplexFloat){re, im};
        }
    }
    return QGT_SUCCESS;
}

/* src/quantum_geometric/core/quantum_geometric_tensor_cpu.c:837-863: square rank-2 tensors only */
qgt_error_t geometric_tensor_initialize_identity(quantum_geometric_tensor_t* t)
{
    if (!t || !t->components || !t->dimensions) return QGT_ERROR_INVALID_ARGUMENT;
    if (t->rank != 2 || t->dimensions[0] != t->dimensions[1]) return QGT_ERROR_INVALID_DIMENSION;
    const size_t n = t->dimensions[0];
    memset(t->components, 0, t->total_elements * sizeof(ComplexFloat));
    for (size_t i = 0; i < n; i++) t->components[i * n + i] = (ComplexFloat){1.0f, 0.0f};
    return QGT_SUCCESS;
}

/* ------------------------------------------------------------------------ */
/* gradients and natural gradients (quantum_geometric_gradient.c)            */
/* ------------------------------------------------------------------------ */

static gradient_options_t g_opts = {1.5707963267948966, false, false, 2, false, NULL};

bool set_gradient_options(const gradient_options_t* o)
{
    if (!o) return false;
    g_opts = *o;
    return true;
}

bool get_gradient_options(gradient_options_t* o)
{
    if (!o) return false;
    *o = g_opts;
    return true;
}

bool compute_quantum_gradient(const quantum_geometric_tensor_network_t* q, size_t idx, ComplexFloat** grad, size_t* dim)
{
    if (!q || !grad || !dim) { set_qgtn_error("Invalid arguments to compute_quantum_gradient"); return false; }
    if (!ensure_step(q, 1)) return false;
    if (idx >= (size_t)backend(q)->P) { set_qgtn_error("Parameter index out of range"); return false; }
    size_t N = (size_t)1 << q->num_qubits;
    double* row = (double*)malloc(sizeof(double) * 2 * N);
    ComplexFloat* out = (ComplexFloat*)malloc(sizeof(ComplexFloat) * N);
    if (!row || !out || qgt_plan_get_row(backend(q)->plan64, 2 + (int)idx, row) != 0) {
        free(row); free(out);
        set_qgtn_error("Failed to read the derivative state");
        return false;
    }
    for (size_t i = 0; i < N; i++) out[i] = (ComplexFloat){(float)row[2 * i], (float)row[2 * i + 1]};
    free(row);
    *grad = out;
    *dim = N;
    return true;
}

bool compute_quantum_natural_gradient(const quantum_geometric_tensor_network_t* q, size_t idx, ComplexFloat** ng,
                                      size_t* dim)
{
    if (!q || !ng || !dim) { set_qgtn_error("Invalid arguments to compute_quantum_natural_gradient"); return false; }
    if (!ensure_step(q, 1) || !ensure_step(q, 0)) return false;
    qgtn_backend_t* b = backend(q);
    int P = b->P;
    if (idx >= (size_t)P) { set_qgtn_error("Parameter index out of range"); return false; }
    natural_gradient_config_t cfg = get_default_natural_gradient_config();
    double* A = (double*)malloc(sizeof(double) * (size_t)P * P);
    double* e = (double*)calloc((size_t)P, sizeof(double));
    double* c = (double*)malloc(sizeof(double) * (size_t)P);
    size_t N = (size_t)1 << q->num_qubits;
    double* out = (double*)malloc(sizeof(double) * 2 * N);
    ComplexFloat* r = (ComplexFloat*)malloc(sizeof(ComplexFloat) * N);
    bool ok = A && e && c && out && r;
    if (ok) {
        for (int i = 0; i < P * P; i++) A[i] = b->Q[2 * i];
        e[idx] = 1.0;
        /* row idx of (G + lambda I)^{-1} = (G + lambda I)^{-1} e_idx (symmetric) */
        ok = qgt_cholesky_solve_f64(A, e, cfg.regularization_param, P, c, NULL) == 0 &&
             qgt_plan_combine_slots(b->plan64, c, out) == 0;
    }
    if (ok) for (size_t i = 0; i < N; i++) r[i] = (ComplexFloat){(float)out[2 * i], (float)out[2 * i + 1]};
    free(A); free(e); free(c); free(out);
    if (!ok) { free(r); set_qgtn_error("Natural-gradient solve failed"); return false; }
    *ng = r;
    *dim = N;
    return true;
}

natural_gradient_config_t get_default_natural_gradient_config(void)
{
    /* quantum_geometric_gradient.c:2721-2730 */
    natural_gradient_config_t c = {1e-4f, 1e8f, true, true, 1e-10f};
    return c;
}

/* Singular values and the pseudo-inverse come from a one-sided Jacobi SVD of
 * the general complex matrix on the GPU (qgt_linalg.cu), where the reference
 * calls LAPACK cgesvd (quantum_geometric_gradient.c:2733-2884); the
 * regularised step solves (G + lambda I) x = g by LU with partial pivoting on
 * the GPU with the singularity rule of the reference's matrix_inverse
 * (matrix_operations.c:55-217).  All three work on G as given (Hermitian or
 * not), in FP64, and return ComplexFloat as the reference does. */
#define NG_MAX_SWEEPS 60

bool compute_complex_matrix_condition_number(const ComplexFloat* m, size_t P, float* kappa)
{
    if (!m || !kappa || P == 0 || P > 8192) return false;
    double* s = (double*)malloc(sizeof(double) * P);
    if (!s) return false;
    int32_t sweeps = 0;
    bool ok = qgt_dev_svd_pinv((const float*)m, (int32_t)P, s, NULL, 0.0, NULL, NG_MAX_SWEEPS, &sweeps) == 0;
    if (ok) {
        /* sigma_max over sigma_min among the positive values (quantum_geometric_gradient.c:2762-2773) */
        double mx = s[0], mn = s[0];
        for (size_t i = 1; i < P; i++) {
            if (s[i] > mx) mx = s[i];
            if (s[i] < mn && s[i] > 0) mn = s[i];
        }
        *kappa = (mn > 1e-15) ? (float)(mx / mn) : INFINITY;
    }
    free(s);
    return ok;
}

bool compute_pseudoinverse_natural_gradient(const ComplexFloat* g, const ComplexFloat* G, ComplexFloat* x, size_t P,
                                            float cutoff)
{
    if (!g || !G || !x || P == 0 || P > 8192) return false;
    double* y = (double*)malloc(sizeof(double) * 2 * P);
    if (!y) return false;
    int32_t sweeps = 0;
    bool ok = qgt_dev_svd_pinv((const float*)G, (int32_t)P, NULL, (const float*)g, (double)cutoff, y, NG_MAX_SWEEPS,
                               &sweeps) == 0;
    if (ok) for (size_t i = 0; i < P; i++) x[i] = (ComplexFloat){(float)y[2 * i], (float)y[2 * i + 1]};
    free(y);
    return ok;
}

bool compute_regularized_natural_gradient(const ComplexFloat* g, const ComplexFloat* G, ComplexFloat* x, size_t P,
                                          const natural_gradient_config_t* cfg)
{
    if (!g || !G || !x || !cfg || P == 0 || P > 8192) return false;
    /* quantum_geometric_gradient.c:2887-2964: lambda grows to 1e-6 sqrt(kappa) above the threshold */
    float lambda = cfg->regularization_param;
    if (cfg->use_adaptive_regularization) {
        float kappa;
        if (compute_complex_matrix_condition_number(G, P, &kappa) && kappa > cfg->condition_threshold) {
            float a = 1e-6f * sqrtf(kappa);
            if (a > lambda) lambda = a;
        }
    }
    double* y = (double*)malloc(sizeof(double) * 2 * P);
    if (!y) return false;
    int32_t singular = 1;
    bool ok = qgt_dev_lu_solve((const float*)G, (int32_t)P, (double)lambda, (const float*)g, y, &singular) == 0;
    if (ok && !singular) {
        for (size_t i = 0; i < P; i++) x[i] = (ComplexFloat){(float)y[2 * i], (float)y[2 * i + 1]};
        free(y);
        return true;
    }
    free(y);
    if (ok && cfg->use_pseudoinverse_fallback)   /* the fallback uses the unregularised metric, as the reference */
        return compute_pseudoinverse_natural_gradient(g, G, x, P, cfg->singular_value_cutoff);
    return false;
}

/* The reference's GPU entry point runs its CPU conjugate gradients
 * (classical_optimization_engine.c:612-623 -> :543-611); here the same
 * iteration (x0 = 0, <= 100 steps, |p^T F p| < 1e-15 or |r| < 1e-8 stops it)
 * runs on the GPU in FP64.  On a failure of the device the plain gradient is
 * returned, as the reference does when its buffers cannot be allocated. */
void compute_natural_gradient_gpu(const double* F, const double* g, double* x, size_t P)
{
    if (!F || !g || !x || P == 0) return;
    if (P > 8192 || qgt_dev_ref_cg(F, g, (int32_t)P, x) != 0) memcpy(x, g, sizeof(double) * P);
}
