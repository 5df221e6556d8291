/*
 * qgt_tune.c -- measured choice of a plan's configuration.
 *
 * Which register tile (13 or 14 qubits), which pass kernels (the program
 * interpreter or compiled straight-line kernels) and how many amplitudes per
 * thread (32, or 16 with compiled kernels) run a circuit fastest
 * depends on its shape: how many gates a pass packs, how many vectors cross
 * it, how far the derivative states travel.  qgt_plan_autotune builds each
 * candidate plan, times its step graph on the GPU with CUDA events and keeps
 * the fastest.  Results go to a text cache, one line per circuit structure
 * and base options:
 *
 *     <key (16 hex digits)> <tile_bits> <pass_kernels> <thread_amps> <ms per step>
 *
 * so a structure is timed once; ragged batches consult the cache for every
 * structural group (qgt_batch_options_t.tune_cache).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../qgt_internal.h"
#include "qgt_gb300.h"

#define E_INVAL (-1)

static uint64_t fnv(uint64_t h, const void* p, size_t n)
{
    const unsigned char* s = (const unsigned char*)p;
    for (size_t i = 0; i < n; i++) {
        h ^= s[i];
        h *= 1099511628211ull;
    }
    return h;
}

/* the circuit's structure (gates, qubits, parameter slots, fixed angles) and the options that shape the plan */
static uint64_t tune_key(const qgt_circuit_desc_t* c, const qgt_plan_options_t* o)
{
    uint64_t h = 1469598103934665603ull;
    h = fnv(h, &c->num_qubits, sizeof c->num_qubits);
    h = fnv(h, &c->num_params, sizeof c->num_params);
    for (int g = 0; g < c->num_gates; g++) {
        const qgt_gate_desc_t* d = &c->gates[g];
        h = fnv(h, &d->type, sizeof d->type);
        h = fnv(h, d->qubits, sizeof d->qubits);
        h = fnv(h, &d->param, sizeof d->param);
        if (d->param < 0) h = fnv(h, &d->angle, sizeof d->angle);
    }
    const int32_t f[7] = {(int32_t)o->precision, (int32_t)o->hamiltonian, o->batch, o->num_deriv_params, o->transport,
                          o->num_pauli_terms, 3 /* candidate set: tile x kernels x amplitudes per thread */};
    return fnv(h, f, sizeof f);
}

static int cache_lookup(const char* path, uint64_t key, int* tile, int* kern, int* amps, double* ms)
{
    if (!path) return 0;
    FILE* f = fopen(path, "r");
    if (!f) return 0;
    char line[256];
    int found = 0;
    while (fgets(line, sizeof line, f)) {
        unsigned long long k;
        int t, kk, a;
        double m;
        if (line[0] == '#') continue;
        if (sscanf(line, "%llx %d %d %d %lf", &k, &t, &kk, &a, &m) == 5 && k == key) {
            *tile = t;
            *kern = kk;
            *amps = a;
            *ms = m;
            found = 1;   /* the last line for a key wins */
        }
    }
    fclose(f);
    return found;
}

static void cache_store(const char* path, uint64_t key, int tile, int kern, int amps, double ms)
{
    if (!path) return;
    FILE* f = fopen(path, "a");
    if (!f) return;
    fprintf(f, "%016llx %d %d %d %.9g\n", (unsigned long long)key, tile, kern, amps, ms);
    fclose(f);
}

/* ms per step of one configuration, -1 when the plan cannot be built */
static double time_config(const qgt_circuit_desc_t* c, const qgt_plan_options_t* o, int steps, const double* theta)
{
    qgt_plan_t* p = NULL;
    if (qgt_plan_create(c, o, &p) != 0) { qgt_clear_error(); return -1.0; }
    double ms = -1.0;
    void *e0 = NULL, *e1 = NULL;
    int rc = qgt_dev_event_create(&e0);
    if (!rc) rc = qgt_dev_event_create(&e1);
    if (!rc) rc = qgt_plan_execute_host(p, theta, NULL, NULL, NULL, NULL);   /* theta in, first step */
    for (int i = 0; i < 2 && !rc; i++) rc = qgt_plan_execute_device(p, NULL, NULL, NULL, NULL, NULL);
    if (!rc) rc = qgt_dev_event_record(e0, qgt_plan_stream(p));
    for (int i = 0; i < steps && !rc; i++) rc = qgt_plan_execute_device(p, NULL, NULL, NULL, NULL, NULL);
    if (!rc) rc = qgt_dev_event_record(e1, qgt_plan_stream(p));
    if (!rc) rc = qgt_plan_synchronize(p);
    float t = 0;
    if (!rc) rc = qgt_dev_event_elapsed(e0, e1, &t);
    if (!rc) ms = (double)t / steps;
    else qgt_clear_error();
    if (e0) qgt_dev_event_destroy(e0);
    if (e1) qgt_dev_event_destroy(e1);
    qgt_plan_destroy(p);
    return ms;
}

int qgt_plan_autotune(const qgt_circuit_desc_t* c, const qgt_plan_options_t* base, const char* cache_path,
                      int32_t steps, qgt_plan_options_t* tuned, double* best_ms)
{
    if (!c || !tuned) return qgt_set_error(E_INVAL, "qgt_plan_autotune: NULL argument");
    qgt_plan_options_t o;
    if (base) o = *base;
    else qgt_plan_default_options(&o);
    if (steps < 1) steps = 5;
    *tuned = o;
    if (best_ms) *best_ms = -1.0;
    const uint64_t key = tune_key(c, &o);
    int tile = 0, kern = 0, amps = 0;
    double ms = -1.0;
    if (cache_lookup(cache_path, key, &tile, &kern, &amps, &ms)) {
        tuned->tile_bits = tile;
        tuned->pass_kernels = kern;
        tuned->thread_amps = amps;
        if (best_ms) *best_ms = ms;
        return 0;
    }
    /* candidates: complex64 plans choose the tile from 14 qubits and the pass kernels from 13 */
    const int mixed = o.precision == QGT_PRECISION_MIXED;
    const int n = c->num_qubits;
    int tiles[2] = {0, 0}, nt = 1, kerns[2] = {0, 0}, nk = 1;
    if (mixed && n >= 14) { tiles[0] = 13; tiles[1] = 14; nt = 2; }
    if (mixed && n >= 13) { kerns[0] = QGT_PASS_INTERPRET; kerns[1] = QGT_PASS_COMPILED; nk = 2; }
    const int P = c->num_params > 0 ? c->num_params : 1, B = o.batch > 0 ? o.batch : 1;
    double* theta = (double*)malloc(sizeof(double) * (size_t)P * B);
    if (!theta) return qgt_set_error(-2, "qgt_plan_autotune: out of host memory");
    uint64_t st = 0x5eed5eedULL;
    for (size_t i = 0; i < (size_t)P * B; i++) {   /* splitmix64 angles in [0, 2 pi) */
        uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        theta[i] = 6.283185307179586 * (double)(z >> 11) * (1.0 / 9007199254740992.0);
    }
    double best = -1.0;
    for (int a = 0; a < nt; a++)
        for (int b = 0; b < nk; b++)
            for (int m = 0; m < 2; m++) {
                /* 16 amplitudes per thread: 13- / 14-qubit tiles with compiled kernels only */
                const int am = m ? 16 : 0;
                if (m && !(mixed && n >= 13 && kerns[b] != QGT_PASS_INTERPRET)) continue;
                qgt_plan_options_t x = o;
                x.use_graph = 1;
                x.tile_bits = tiles[a];
                x.pass_kernels = m ? QGT_PASS_COMPILED : kerns[b];
                x.thread_amps = am;
                const double t = time_config(c, &x, steps, theta);
                if (t > 0 && (best < 0 || t < best)) {
                    best = t;
                    tile = x.tile_bits;
                    kern = x.pass_kernels;
                    amps = am;
                }
            }
    free(theta);
    if (best < 0) return qgt_set_error(-6, "qgt_plan_autotune: no configuration of the circuit could be built");
    tuned->tile_bits = tile;
    tuned->pass_kernels = kern;
    tuned->thread_amps = amps;
    if (best_ms) *best_ms = best;
    cache_store(cache_path, key, tile, kern, amps, best);
    return 0;
}
