/*
 * qgt_precond.c -- learned metric preconditioner (training / inference
 * driver), GPU PCG and the natural-gradient VQE loop.
 *
 * No reference counterpart: the reference's learning pipeline trains a CPU
 * float MLP for classification (src/quantum_geometric/learning/
 * quantum_pipeline_impl.c:577-790) and solves the natural-gradient system
 * by unpreconditioned CG (src/quantum_geometric/hybrid/
 * classical_optimization_engine.c:543-611) or by Cholesky with lambda x10
 * retries (quantum_pipeline_impl.c:1601-1682); its VQE loop is
 * src/quantum_geometric/hybrid/quantum_classical_algorithms.c:854-886.
 *
 * Here the MLP theta -> (d, U) approximates Re Q + lambda I by
 * diag(d) + U U^T, is trained on exact metrics that the plans generate on the
 * GPU (theta-batched), and serves as the PCG preconditioner.  All of its
 * forward, backward and optimiser kernels are in qgt_learned.cu.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../qgt_internal.h"
#include "qgt_gb300.h"

#define E_INVAL (-1)
#define E_NOMEM (-2)

struct qgt_precond {
    qgt_precond_config_t cfg;
    int P, W, r, in, od;
    int64_t nw;                 /* number of weights (all layers, biases included) */
    int64_t off[6];             /* W1 b1 W2 b2 W3 b3 */
    float *w, *g, *m1, *m2;     /* device: masters, gradients, Adam moments */
    void* wb;                   /* device BF16 copy */
    int step;                   /* Adam step */
    void* stream;
    /* activations for up to `cap` samples */
    int cap;
    float *X, *Z1, *H1, *Z2, *H2, *O, *dO, *dH1, *dH2, *loss;
    int32_t* idx;
    double *theta_d, *d_d, *U_d;
};

static uint64_t sm64(uint64_t* s)
{
    uint64_t z = (*s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static double u01(uint64_t* s) { return (double)(sm64(s) >> 11) * (1.0 / 9007199254740992.0); }

void qgt_precond_default_config(qgt_precond_config_t* c)
{
    memset(c, 0, sizeof *c);
    c->num_params = 0;
    c->width = 512;
    c->rank = 16;
    c->lambda = 1e-3;
    c->u_scale = 0.1;
    c->seed = 1;
    c->device = 0;
}

void qgt_precond_default_train_options(qgt_precond_train_options_t* o)
{
    memset(o, 0, sizeof *o);
    o->epochs = 30;
    o->batch = 256;
    o->lr = 1e-3;
    o->weight_decay = 0.0;
    o->seed = 7;
}

static void free_acts(qgt_precond_t* p)
{
    void* a[] = {p->X, p->Z1, p->H1, p->Z2, p->H2, p->O, p->dO, p->dH1, p->dH2, p->loss, p->idx, p->theta_d,
                 p->d_d, p->U_d};
    for (size_t i = 0; i < sizeof a / sizeof a[0]; i++) qgt_dev_free(a[i]);
    p->X = p->Z1 = p->H1 = p->Z2 = p->H2 = p->O = p->dO = p->dH1 = p->dH2 = p->loss = NULL;
    p->idx = NULL;
    p->theta_d = p->d_d = p->U_d = NULL;
    p->cap = 0;
}

static int ensure_acts(qgt_precond_t* p, int n)
{
    if (n <= p->cap) return 0;
    free_acts(p);
    int rc = 0;
    const size_t B = (size_t)n;
#define A_(ptr, cnt) if (!rc) rc = qgt_dev_malloc((void**)&(ptr), sizeof(*(ptr)) * (cnt))
    A_(p->X, B * p->in);
    A_(p->Z1, B * p->W);
    A_(p->H1, B * p->W);
    A_(p->Z2, B * p->W);
    A_(p->H2, B * p->W);
    A_(p->O, B * p->od);
    A_(p->dO, B * p->od);
    A_(p->dH1, B * p->W);
    A_(p->dH2, B * p->W);
    A_(p->loss, 4);
    A_(p->idx, B);
    A_(p->theta_d, B * p->P);
    A_(p->d_d, B * p->P);
    A_(p->U_d, B * p->P * (p->r > 0 ? p->r : 1));
#undef A_
    if (rc) { free_acts(p); return rc; }
    p->cap = n;
    return 0;
}

void qgt_precond_destroy(qgt_precond_t* p)
{
    if (!p) return;
    if (p->stream) qgt_dev_stream_sync(p->stream);
    free_acts(p);
    qgt_dev_free(p->w); qgt_dev_free(p->g); qgt_dev_free(p->m1); qgt_dev_free(p->m2); qgt_dev_free(p->wb);
    if (p->stream) qgt_dev_stream_destroy(p->stream);
    free(p);
}

int qgt_precond_create(const qgt_precond_config_t* cfg, qgt_precond_t** out)
{
    if (!cfg || !out) return qgt_set_error(E_INVAL, "qgt_precond_create: NULL argument");
    *out = NULL;
    if (cfg->num_params < 1 || cfg->num_params > 1024 || cfg->width < 1 || cfg->width > 8192 || cfg->rank < 0 ||
        cfg->rank > 32 || !(cfg->lambda > 0) || !(cfg->u_scale > 0))
        return qgt_set_error(E_INVAL, "qgt_precond_create: P in [1, 1024], width in [1, 8192], rank in [0, 32], "
                                      "lambda > 0, u_scale > 0");
    qgt_precond_t* p = (qgt_precond_t*)calloc(1, sizeof *p);
    if (!p) return qgt_set_error(E_NOMEM, "qgt_precond_create: out of memory");
    p->cfg = *cfg;
    p->P = cfg->num_params;
    p->W = cfg->width;
    p->r = cfg->rank;
    p->in = 2 * p->P;
    p->od = p->P + p->P * p->r;
    const int64_t sz[6] = {(int64_t)p->W * p->in, p->W, (int64_t)p->W * p->W, p->W, (int64_t)p->od * p->W, p->od};
    p->nw = 0;
    for (int i = 0; i < 6; i++) { p->off[i] = p->nw; p->nw += sz[i]; }
    int rc = qgt_dev_set_device(cfg->device);
    if (!rc) rc = qgt_dev_stream_create(&p->stream);
    if (!rc) rc = qgt_dev_malloc((void**)&p->w, sizeof(float) * (size_t)p->nw);
    if (!rc) rc = qgt_dev_malloc((void**)&p->g, sizeof(float) * (size_t)p->nw);
    if (!rc) rc = qgt_dev_malloc((void**)&p->m1, sizeof(float) * (size_t)p->nw);
    if (!rc) rc = qgt_dev_malloc((void**)&p->m2, sizeof(float) * (size_t)p->nw);
    if (!rc) rc = qgt_dev_malloc(&p->wb, 2 * (size_t)p->nw);
    float* h = (float*)malloc(sizeof(float) * (size_t)p->nw);
    if (!rc && !h) rc = qgt_set_error(E_NOMEM, "qgt_precond_create: out of memory");
    if (!rc) {
        /* uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases; output layer scaled by 0.1 */
        uint64_t s = cfg->seed;
        const int fan[3] = {p->in, p->W, p->W};
        for (int l = 0; l < 3; l++) {
            const double a = (l == 2 ? 0.1 : 1.0) / sqrt((double)fan[l]);
            for (int64_t i = 0; i < sz[2 * l]; i++) h[p->off[2 * l] + i] = (float)(a * (2.0 * u01(&s) - 1.0));
            for (int64_t i = 0; i < sz[2 * l + 1]; i++) h[p->off[2 * l + 1] + i] = 0.f;
        }
        rc = qgt_dev_memcpy_h2d(p->w, h, sizeof(float) * (size_t)p->nw, p->stream);
    }
    free(h);
    if (!rc) rc = qgt_dev_memset(p->m1, 0, sizeof(float) * (size_t)p->nw, p->stream);
    if (!rc) rc = qgt_dev_memset(p->m2, 0, sizeof(float) * (size_t)p->nw, p->stream);
    if (!rc) rc = qgt_dev_lr_to_bf16(p->w, p->wb, p->nw, p->stream);
    if (!rc) rc = qgt_dev_stream_sync(p->stream);
    if (rc) { qgt_precond_destroy(p); return rc; }
    *out = p;
    return 0;
}

int64_t qgt_precond_num_weights(const qgt_precond_t* p) { return p ? p->nw : 0; }

int qgt_precond_get_weights(const qgt_precond_t* p, float* w)
{
    if (!p || !w) return qgt_set_error(E_INVAL, "qgt_precond_get_weights: NULL argument");
    int rc = qgt_dev_memcpy_d2h(w, p->w, sizeof(float) * (size_t)p->nw, p->stream);
    if (!rc) rc = qgt_dev_stream_sync(p->stream);
    return rc;
}

int qgt_precond_set_weights(qgt_precond_t* p, const float* w)
{
    if (!p || !w) return qgt_set_error(E_INVAL, "qgt_precond_set_weights: NULL argument");
    int rc = qgt_dev_memcpy_h2d(p->w, w, sizeof(float) * (size_t)p->nw, p->stream);
    if (!rc) rc = qgt_dev_lr_to_bf16(p->w, p->wb, p->nw, p->stream);
    if (!rc) rc = qgt_dev_stream_sync(p->stream);
    return rc;
}

static const void* wb_at(const qgt_precond_t* p, int k) { return (const char*)p->wb + 2 * (size_t)p->off[k]; }

/* forward for n samples: theta rows idx (device) of theta_src (device) -> O */
static int forward(qgt_precond_t* p, const double* theta_src, const int32_t* idx, int n)
{
    int rc = qgt_dev_lr_features(theta_src, idx, n, p->P, p->X, p->stream);
    if (!rc) rc = qgt_dev_lr_linear(n, p->W, p->in, p->X, wb_at(p, 0), p->w + p->off[1], p->H1, 1, p->Z1, p->stream);
    if (!rc) rc = qgt_dev_lr_linear(n, p->W, p->W, p->H1, wb_at(p, 2), p->w + p->off[3], p->H2, 1, p->Z2, p->stream);
    if (!rc) rc = qgt_dev_lr_linear(n, p->od, p->W, p->H2, wb_at(p, 4), p->w + p->off[5], p->O, 0, NULL, p->stream);
    return rc;
}

/* loss + gradients into p->g for n samples (metric rows idx of metric_d, FP32) */
static int backward(qgt_precond_t* p, const float* metric_d, const int32_t* idx, int n)
{
    const float lam = (float)p->cfg.lambda, us = (float)p->cfg.u_scale;
    int rc = qgt_dev_lr_loss(p->O, metric_d, idx, n, p->P, p->r, lam, us, p->dO, p->loss, p->stream);
    if (!rc) rc = qgt_dev_lr_linear_dw(n, p->od, p->W, p->dO, p->H2, p->g + p->off[4], p->g + p->off[5], p->stream);
    if (!rc) rc = qgt_dev_lr_linear_dx(n, p->od, p->W, p->dO, wb_at(p, 4), p->dH2, p->stream);
    if (!rc) rc = qgt_dev_lr_silu_back(p->Z2, p->dH2, (int64_t)n * p->W, p->stream);
    if (!rc) rc = qgt_dev_lr_linear_dw(n, p->W, p->W, p->dH2, p->H1, p->g + p->off[2], p->g + p->off[3], p->stream);
    if (!rc) rc = qgt_dev_lr_linear_dx(n, p->W, p->W, p->dH2, wb_at(p, 2), p->dH1, p->stream);
    if (!rc) rc = qgt_dev_lr_silu_back(p->Z1, p->dH1, (int64_t)n * p->W, p->stream);
    if (!rc) rc = qgt_dev_lr_linear_dw(n, p->W, p->in, p->dH1, p->X, p->g + p->off[0], p->g + p->off[1], p->stream);
    return rc;
}

/* training on device data: theta_d S x P (double), metric_d S x P x P (float) */
static int train_device(qgt_precond_t* p, const double* theta_d, const float* metric_d, int S,
                        const qgt_precond_train_options_t* o, double* hist)
{
    const int B = o->batch < 1 ? 1 : (o->batch > S ? S : o->batch);
    int rc = ensure_acts(p, B);
    if (rc) return rc;
    int32_t* perm = (int32_t*)malloc(sizeof(int32_t) * (size_t)S);
    float* lossh = NULL;
    if (!perm) return qgt_set_error(E_NOMEM, "qgt_precond_train: out of memory");
    int32_t* perm_d = NULL;
    rc = qgt_dev_malloc((void**)&perm_d, sizeof(int32_t) * (size_t)S);
    if (!rc) rc = qgt_dev_host_alloc((void**)&lossh, sizeof(float) * 4);
    uint64_t sd = o->seed;
    const int nb = S / B;   /* full batches only */
    for (int e = 0; e < o->epochs && !rc; e++) {
        for (int i = 0; i < S; i++) perm[i] = i;
        for (int i = S - 1; i > 0; i--) {
            int j = (int)(sm64(&sd) % (uint64_t)(i + 1));
            int32_t t = perm[i]; perm[i] = perm[j]; perm[j] = t;
        }
        rc = qgt_dev_memcpy_h2d(perm_d, perm, sizeof(int32_t) * (size_t)S, p->stream);
        if (!rc) rc = qgt_dev_memset(p->loss, 0, sizeof(float), p->stream);
        for (int b = 0; b < nb && !rc; b++) {
            const int32_t* idx = perm_d + (size_t)b * B;
            rc = forward(p, theta_d, idx, B);
            if (!rc) rc = backward(p, metric_d, idx, B);
            if (!rc) rc = qgt_dev_lr_adam(p->w, p->wb, p->g, p->m1, p->m2, p->nw, (float)o->lr, 0.9f, 0.999f, 1e-8f,
                                          ++p->step, (float)o->weight_decay, p->stream);
        }
        if (!rc) rc = qgt_dev_memcpy_d2h(lossh, p->loss, sizeof(float), p->stream);
        if (!rc) rc = qgt_dev_stream_sync(p->stream);
        if (!rc && hist) hist[e] = (double)lossh[0] / (nb > 0 ? nb : 1);
    }
    /* perm must not be reused before the stream is done with it */
    qgt_dev_stream_sync(p->stream);
    qgt_dev_free(perm_d);
    qgt_dev_host_free(lossh);
    free(perm);
    return rc;
}

int qgt_precond_train(qgt_precond_t* p, const double* theta, const double* metric, int32_t S,
                      const qgt_precond_train_options_t* opt, double* hist)
{
    if (!p || !theta || !metric || S < 1) return qgt_set_error(E_INVAL, "qgt_precond_train: bad argument");
    qgt_precond_train_options_t o;
    if (opt) o = *opt; else qgt_precond_default_train_options(&o);
    const size_t PP = (size_t)p->P * p->P;
    double *th_d = NULL, *m64 = NULL;
    float* m_d = NULL;
    int rc = qgt_dev_malloc((void**)&th_d, sizeof(double) * (size_t)S * p->P);
    if (!rc) rc = qgt_dev_malloc((void**)&m_d, sizeof(float) * (size_t)S * PP);
    if (!rc) rc = qgt_dev_malloc((void**)&m64, sizeof(double) * 2 * PP);
    if (!rc) rc = qgt_dev_memcpy_h2d(th_d, theta, sizeof(double) * (size_t)S * p->P, p->stream);
    /* metric rows as complex pairs (imaginary 0) so the Re Q extraction kernel serves both paths */
    double* tmp = (double*)malloc(sizeof(double) * 2 * PP);
    if (!rc && !tmp) rc = qgt_set_error(E_NOMEM, "qgt_precond_train: out of memory");
    for (int s = 0; s < S && !rc; s++) {
        for (size_t i = 0; i < PP; i++) { tmp[2 * i] = metric[(size_t)s * PP + i]; tmp[2 * i + 1] = 0.0; }
        rc = qgt_dev_memcpy_h2d(m64, tmp, sizeof(double) * 2 * PP, p->stream);
        if (!rc) rc = qgt_dev_metric_f32(m64, (int64_t)PP, m_d + (size_t)s * PP, p->stream);
        if (!rc) rc = qgt_dev_stream_sync(p->stream);
    }
    free(tmp);
    if (!rc) rc = train_device(p, th_d, m_d, S, &o, hist);
    qgt_dev_free(th_d);
    qgt_dev_free(m_d);
    qgt_dev_free(m64);
    return rc;
}

/* exact metrics of S points on the GPU, written to m_d (FP32, S x P x P) */
static int metrics_device(const qgt_circuit_desc_t* c, const double* theta, int S, qgt_precision_t prec, int device,
                          float* m_d, void* stream)
{
    const int P = c->num_params;
    int B = S < 64 ? S : 64;
    qgt_plan_options_t o;
    qgt_plan_default_options(&o);
    o.precision = prec;
    o.hamiltonian = QGT_HAMILTONIAN_NONE;
    o.device = device;
    o.use_graph = 0;
    o.batch = B;
    qgt_plan_t* pl = NULL;
    int rc = qgt_plan_create(c, &o, &pl);
    for (int s0 = 0; s0 < S && !rc; s0 += B) {
        const int n = (S - s0) < B ? (S - s0) : B;
        /* the last chunk repeats its final point to fill the batch */
        double* th = (double*)malloc(sizeof(double) * (size_t)B * P);
        if (!th) { rc = qgt_set_error(E_NOMEM, "metric dataset: out of memory"); break; }
        for (int k = 0; k < B; k++)
            memcpy(th + (size_t)k * P, theta + (size_t)(s0 + (k < n ? k : n - 1)) * P, sizeof(double) * (size_t)P);
        rc = qgt_dev_memcpy_h2d(qgt_plan_dev_theta(pl), th, sizeof(double) * (size_t)B * P, stream);
        if (!rc) rc = qgt_plan_enqueue_step(pl, stream);
        if (!rc) rc = qgt_dev_metric_f32(qgt_plan_dev_Q(pl), (int64_t)n * P * P, m_d + (size_t)s0 * P * P, stream);
        if (!rc) rc = qgt_dev_stream_sync(stream);
        free(th);
        if (!rc) rc = qgt_plan_device_status(pl, NULL);
    }
    qgt_plan_destroy(pl);
    return rc;
}

int qgt_metric_dataset(const qgt_circuit_desc_t* c, const double* theta, int32_t S, qgt_precision_t prec,
                       int32_t device, double* metric)
{
    if (!c || !theta || !metric || S < 1) return qgt_set_error(E_INVAL, "qgt_metric_dataset: bad argument");
    const size_t PP = (size_t)c->num_params * c->num_params;
    void* s = NULL;
    float* m_d = NULL;
    int rc = qgt_dev_set_device(device);
    if (!rc) rc = qgt_dev_stream_create(&s);
    if (!rc) rc = qgt_dev_malloc((void**)&m_d, sizeof(float) * (size_t)S * PP);
    if (!rc) rc = metrics_device(c, theta, S, prec, device, m_d, s);
    float* h = (float*)malloc(sizeof(float) * (size_t)S * PP);
    if (!rc && !h) rc = qgt_set_error(E_NOMEM, "qgt_metric_dataset: out of memory");
    if (!rc) rc = qgt_dev_memcpy_d2h(h, m_d, sizeof(float) * (size_t)S * PP, s);
    if (!rc) rc = qgt_dev_stream_sync(s);
    if (!rc) for (size_t i = 0; i < (size_t)S * PP; i++) metric[i] = h[i];
    free(h);
    qgt_dev_free(m_d);
    if (s) qgt_dev_stream_destroy(s);
    return rc;
}

int qgt_precond_train_circuit(qgt_precond_t* p, const qgt_circuit_desc_t* c, const double* theta, int32_t S,
                              qgt_precision_t prec, const qgt_precond_train_options_t* opt, double* hist)
{
    if (!p || !c || !theta || S < 1) return qgt_set_error(E_INVAL, "qgt_precond_train_circuit: bad argument");
    if (c->num_params != p->P)
        return qgt_set_error(E_INVAL, "qgt_precond_train_circuit: circuit has %d parameters, network %d", c->num_params, p->P);
    qgt_precond_train_options_t o;
    if (opt) o = *opt; else qgt_precond_default_train_options(&o);
    const size_t PP = (size_t)p->P * p->P;
    double* th_d = NULL;
    float* m_d = NULL;
    int rc = qgt_dev_malloc((void**)&th_d, sizeof(double) * (size_t)S * p->P);
    if (!rc) rc = qgt_dev_malloc((void**)&m_d, sizeof(float) * (size_t)S * PP);
    if (!rc) rc = qgt_dev_memcpy_h2d(th_d, theta, sizeof(double) * (size_t)S * p->P, p->stream);
    if (!rc) rc = metrics_device(c, theta, S, prec, p->cfg.device, m_d, p->stream);
    if (!rc) rc = train_device(p, th_d, m_d, S, &o, hist);
    qgt_dev_free(th_d);
    qgt_dev_free(m_d);
    return rc;
}

int qgt_precond_loss_grad(qgt_precond_t* p, const double* theta, const double* metric, int32_t S, double* loss,
                          float* grad)
{
    if (!p || !theta || !metric || S < 1) return qgt_set_error(E_INVAL, "qgt_precond_loss_grad: bad argument");
    const size_t PP = (size_t)p->P * p->P;
    int rc = ensure_acts(p, S);
    float* m_d = NULL;
    float* mh = (float*)malloc(sizeof(float) * (size_t)S * PP);
    float lh = 0.f;
    if (!rc && !mh) rc = qgt_set_error(E_NOMEM, "qgt_precond_loss_grad: out of memory");
    if (!rc) rc = qgt_dev_malloc((void**)&m_d, sizeof(float) * (size_t)S * PP);
    if (!rc) {
        for (size_t i = 0; i < (size_t)S * PP; i++) mh[i] = (float)metric[i];
        rc = qgt_dev_memcpy_h2d(m_d, mh, sizeof(float) * (size_t)S * PP, p->stream);
    }
    if (!rc) rc = qgt_dev_memcpy_h2d(p->theta_d, theta, sizeof(double) * (size_t)S * p->P, p->stream);
    if (!rc) rc = qgt_dev_memset(p->loss, 0, sizeof(float), p->stream);
    if (!rc) rc = forward(p, p->theta_d, NULL, S);
    if (!rc) rc = backward(p, m_d, NULL, S);
    if (!rc) rc = qgt_dev_memcpy_d2h(&lh, p->loss, sizeof(float), p->stream);
    if (!rc && grad) rc = qgt_dev_memcpy_d2h(grad, p->g, sizeof(float) * (size_t)p->nw, p->stream);
    if (!rc) rc = qgt_dev_stream_sync(p->stream);
    if (!rc && loss) *loss = lh;
    qgt_dev_free(m_d);
    free(mh);
    return rc;
}

/* d (S x P), U (S x P x r) on the device for S points of theta_dev (device) */
static int predict_device(qgt_precond_t* p, const double* theta_dev, int S, double* d_dev, double* U_dev, void* stream)
{
    void* own = p->stream;
    p->stream = stream;
    int rc = forward(p, theta_dev, NULL, S);
    if (!rc) rc = qgt_dev_lr_outputs(p->O, S, p->P, p->r, (float)p->cfg.lambda, (float)p->cfg.u_scale, d_dev, U_dev, stream);
    p->stream = own;
    return rc;
}

int qgt_precond_predict(qgt_precond_t* p, const double* theta, int32_t S, double* d, double* U)
{
    if (!p || !theta || S < 1) return qgt_set_error(E_INVAL, "qgt_precond_predict: bad argument");
    int rc = ensure_acts(p, S);
    if (!rc) rc = qgt_dev_memcpy_h2d(p->theta_d, theta, sizeof(double) * (size_t)S * p->P, p->stream);
    if (!rc) rc = predict_device(p, p->theta_d, S, p->d_d, p->U_d, p->stream);
    if (!rc && d) rc = qgt_dev_memcpy_d2h(d, p->d_d, sizeof(double) * (size_t)S * p->P, p->stream);
    if (!rc && U && p->r > 0) rc = qgt_dev_memcpy_d2h(U, p->U_d, sizeof(double) * (size_t)S * p->P * p->r, p->stream);
    if (!rc) rc = qgt_dev_stream_sync(p->stream);
    return rc;
}

int qgt_pcg_solve_f64(const double* A, const double* b, double lambda, int32_t P, const double* d, const double* U,
                      int32_t r, double tol, int32_t max_iter, double* x, int32_t* iters, double* resid)
{
    if (!A || !b || !x || P < 1 || (r > 0 && !U)) return qgt_set_error(E_INVAL, "qgt_pcg_solve_f64: bad argument");
    void* s = NULL;
    double *A_d = NULL, *b_d = NULL, *x_d = NULL, *d_d = NULL, *U_d = NULL, *res_d = NULL;
    int32_t* it_d = NULL;
    int32_t it = 0;
    double res = 0;
    int rc = qgt_dev_stream_create(&s);
    if (!rc) rc = qgt_dev_malloc((void**)&A_d, sizeof(double) * (size_t)P * P);
    if (!rc) rc = qgt_dev_malloc((void**)&b_d, sizeof(double) * (size_t)P);
    if (!rc) rc = qgt_dev_malloc((void**)&x_d, sizeof(double) * (size_t)P);
    if (!rc) rc = qgt_dev_malloc((void**)&res_d, sizeof(double));
    if (!rc) rc = qgt_dev_malloc((void**)&it_d, sizeof(int32_t));
    if (!rc && d) rc = qgt_dev_malloc((void**)&d_d, sizeof(double) * (size_t)P);
    if (!rc && r > 0) rc = qgt_dev_malloc((void**)&U_d, sizeof(double) * (size_t)P * r);
    if (!rc) rc = qgt_dev_memcpy_h2d(A_d, A, sizeof(double) * (size_t)P * P, s);
    if (!rc) rc = qgt_dev_memcpy_h2d(b_d, b, sizeof(double) * (size_t)P, s);
    if (!rc && d) rc = qgt_dev_memcpy_h2d(d_d, d, sizeof(double) * (size_t)P, s);
    if (!rc && r > 0) rc = qgt_dev_memcpy_h2d(U_d, U, sizeof(double) * (size_t)P * r, s);
    if (!rc) rc = qgt_dev_pcg(A_d, 0, 0, b_d, P, lambda, d_d, U_d, r, tol, max_iter, x_d, it_d, res_d, 1, s);
    if (!rc) rc = qgt_dev_memcpy_d2h(x, x_d, sizeof(double) * (size_t)P, s);
    if (!rc) rc = qgt_dev_memcpy_d2h(&it, it_d, sizeof(int32_t), s);
    if (!rc) rc = qgt_dev_memcpy_d2h(&res, res_d, sizeof(double), s);
    if (!rc) rc = qgt_dev_stream_sync(s);
    if (!rc && iters) *iters = it;
    if (!rc && resid) *resid = res;
    void* f[] = {A_d, b_d, x_d, d_d, U_d, res_d, it_d};
    for (size_t i = 0; i < sizeof f / sizeof f[0]; i++) qgt_dev_free(f[i]);
    if (s) qgt_dev_stream_destroy(s);
    return rc;
}

void qgt_vqe_default_options(qgt_vqe_options_t* o)
{
    memset(o, 0, sizeof *o);
    o->steps = 500;
    o->eta = 0.05;
    o->pcg_tol = 1e-10;
    o->pcg_max_iter = 1000;
    o->solver = QGT_VQE_SOLVER_CHOLESKY;
}

int qgt_vqe_run(const qgt_circuit_desc_t* c, const qgt_plan_options_t* popt, qgt_precond_t* pc,
                const qgt_vqe_options_t* vopt, const double* theta0, double* energies, int32_t* pcg_iters,
                double* theta_out)
{
    if (!c || !theta0 || !energies) return qgt_set_error(E_INVAL, "qgt_vqe_run: bad argument");
    qgt_vqe_options_t vo;
    if (vopt) vo = *vopt; else qgt_vqe_default_options(&vo);
    if (vo.steps < 1) return qgt_set_error(E_INVAL, "qgt_vqe_run: steps must be >= 1");
    if (vo.solver == QGT_VQE_SOLVER_PCG_LEARNED && (!pc || pc->P != c->num_params))
        return qgt_set_error(E_INVAL, "qgt_vqe_run: the learned solver needs a preconditioner for %d parameters", c->num_params);
    qgt_plan_options_t o;
    if (popt) o = *popt; else qgt_plan_default_options(&o);
    if (o.hamiltonian == QGT_HAMILTONIAN_NONE) o.hamiltonian = QGT_HAMILTONIAN_TFIM;
    o.batch = 1;
    o.num_deriv_params = 0;
    const int P = c->num_params;
    qgt_plan_t* pl = NULL;
    int rc = qgt_plan_create(c, &o, &pl);
    if (rc) return rc;
    void* s = qgt_plan_stream(pl);
    double *th_d = NULL, *x_d = NULL, *E_d = NULL, *res_d = NULL, *dj = NULL, *Uj = NULL;
    int32_t* it_d = NULL;
    const int r = pc ? pc->r : 0;
    rc = qgt_dev_malloc((void**)&th_d, sizeof(double) * (size_t)P);
    if (!rc) rc = qgt_dev_malloc((void**)&x_d, sizeof(double) * (size_t)P);
    if (!rc) rc = qgt_dev_malloc((void**)&E_d, sizeof(double) * (size_t)vo.steps);
    if (!rc) rc = qgt_dev_malloc((void**)&res_d, sizeof(double) * (size_t)vo.steps);
    if (!rc) rc = qgt_dev_malloc((void**)&it_d, sizeof(int32_t) * (size_t)vo.steps);
    if (!rc) rc = qgt_dev_malloc((void**)&dj, sizeof(double) * (size_t)P);
    if (!rc) rc = qgt_dev_malloc((void**)&Uj, sizeof(double) * (size_t)P * (r > 0 ? r : 1));
    if (!rc) rc = qgt_dev_memset(it_d, 0, sizeof(int32_t) * (size_t)vo.steps, s);
    if (!rc) rc = qgt_dev_memcpy_h2d(th_d, theta0, sizeof(double) * (size_t)P, s);
    if (!rc && pc) rc = ensure_acts(pc, 1);
    if (!rc && pc) rc = qgt_dev_stream_sync(pc->stream);
    /* the whole loop is enqueued on the plan's stream: step graph, solve, update */
    for (int t = 0; t < vo.steps && !rc; t++) {
        rc = qgt_plan_execute_device(pl, th_d, NULL, NULL, NULL, NULL);
        if (!rc) rc = qgt_dev_memcpy_d2d(E_d + t, qgt_plan_dev_energy(pl), sizeof(double), s);
        if (rc) break;
        const double* step = qgt_plan_dev_natgrad(pl);
        if (vo.solver != QGT_VQE_SOLVER_CHOLESKY) {
            const double* dd = NULL;
            const double* UU = NULL;
            int rr = 0;
            if (vo.solver == QGT_VQE_SOLVER_PCG_LEARNED) {
                rc = predict_device(pc, th_d, 1, dj, Uj, s);
                dd = dj;
                UU = Uj;
                rr = r;
            }
            if (!rc) rc = qgt_dev_pcg(qgt_plan_dev_Q(pl), 1, 0, qgt_plan_dev_grad(pl), P, o.lambda, dd, UU, rr,
                                      vo.pcg_tol, vo.pcg_max_iter, x_d, it_d + t, res_d + t, 1, s);
            step = x_d;
        }
        if (!rc) rc = qgt_dev_axpy_update(th_d, step, vo.eta, P, s);
    }
    if (!rc) rc = qgt_dev_stream_sync(s);
    if (!rc) rc = qgt_plan_device_status(pl, NULL);
    if (!rc) rc = qgt_dev_memcpy_d2h(energies, E_d, sizeof(double) * (size_t)vo.steps, s);
    if (!rc && pcg_iters) rc = qgt_dev_memcpy_d2h(pcg_iters, it_d, sizeof(int32_t) * (size_t)vo.steps, s);
    if (!rc && theta_out) rc = qgt_dev_memcpy_d2h(theta_out, th_d, sizeof(double) * (size_t)P, s);
    if (!rc) rc = qgt_dev_stream_sync(s);
    void* f[] = {th_d, x_d, E_d, res_d, it_d, dj, Uj};
    for (size_t i = 0; i < sizeof f / sizeof f[0]; i++) qgt_dev_free(f[i]);
    qgt_plan_destroy(pl);
    return rc;
}
