/*
 * qgt_gb300.h -- C ABI of the GB300 quantum-geometric-tensor engine.
 *
 * One shared library, libqgt_gb300.so, exports two groups of entry points:
 *
 *   1. The reference library's own C entry points for this path, with the
 *      reference prototypes (the headers under include/quantum_geometric/core in this
 *      repository mirrors them): geometric_compute_fubini_study_metric,
 *      geometric_compute_berry_curvature, geometric_compute_full_qgt,
 *      compute_quantum_geometric_tensor, compute_quantum_natural_gradient,
 *      compute_regularized_natural_gradient, ...
 *   2. The extensions declared here: compiled circuit plans with FP64
 *      outputs, device-resident execution, the natural-gradient step, and
 *      ragged batches.  The reference has no counterpart for these; its
 *      closest interfaces are named beside each declaration.
 *
 * All pointers are plain host or device pointers; sizes are element counts.
 * Complex arrays are interleaved {re, im} doubles.  Functions return
 * qgt_error_t codes (0 = success, negative = error, values of the reference
 * include/quantum_geometric/core/error_codes.h:18-194) and set a thread-local
 * message readable with qgt_last_error().
 *
 * Circuit conventions (reference semantics):
 *   - basis index bit q = qubit q; start state |0...0>
 *     (src/quantum_geometric/core/quantum_geometric_tensor_network.c:87-89);
 *   - RX/RY/RZ(theta) = exp(-i theta G/2), G = X/Y/Z
 *     (src/quantum_geometric/hybrid/quantum_classical_algorithms.c:254-264);
 *     CNOT(c -> t) swaps |c=1,t=0> and |c=1,t=1>; CZ negates |11> (:195-226);
 *   - parameter k is the k-th entry of theta; several gates may share one.
 */
#ifndef QGT_GB300_H
#define QGT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Gate codes: the reference gate_type_t values
 * (include/quantum_geometric/core/quantum_base_types.h:32-71). */
enum {
    QGT_GATE_I = 0, QGT_GATE_X = 1, QGT_GATE_Y = 2, QGT_GATE_Z = 3, QGT_GATE_H = 4,
    QGT_GATE_S = 5, QGT_GATE_T = 6, QGT_GATE_RX = 7, QGT_GATE_RY = 8, QGT_GATE_RZ = 9,
    QGT_GATE_CNOT = 10, QGT_GATE_CZ = 12, QGT_GATE_SWAP = 13
};

typedef struct {
    int32_t type;       /* QGT_GATE_* */
    int32_t qubits[2];  /* 1q: {target, -1}; CNOT: {control, target}; CZ/SWAP: {a, b} */
    int32_t param;      /* index into theta for RX/RY/RZ, or -1 (fixed angle) */
    double angle;       /* angle when param < 0 */
} qgt_gate_desc_t;

typedef struct {
    int32_t num_qubits;           /* 1 .. 30 */
    int32_t num_gates;
    const qgt_gate_desc_t* gates;
    int32_t num_params;           /* length of theta (>= 1 + max param) */
} qgt_circuit_desc_t;

typedef enum {
    /* complex128 evolution, FP64 Gram, FP64 projector / solve */
    QGT_PRECISION_FP64 = 0,
    /* complex64 evolution; Gram on tcgen05 tensor cores from 3-term split
     * FP16 operands (power-of-two prescaled) with FP32 accumulation; FP64
     * split-K reduction, projector, renormalisation and Cholesky solve */
    QGT_PRECISION_MIXED = 1,
    /* as MIXED but the split operands are BF16 (hi + lo, 3 products) */
    QGT_PRECISION_MIXED_BF16X3 = 2
} qgt_precision_t;

typedef enum {
    QGT_HAMILTONIAN_NONE = 0,
    /* transverse-field Ising ring H = -J sum_i Z_i Z_{i+1 mod n} - h sum_i X_i
     * (n bonds for n >= 3, an open chain below) */
    QGT_HAMILTONIAN_TFIM = 1
} qgt_hamiltonian_t;

typedef struct {
    qgt_precision_t precision;
    qgt_hamiltonian_t hamiltonian;
    double tfim_J, tfim_h;
    double lambda;      /* Tikhonov lambda of the natural-gradient step (Re Q + lambda I) x = grad E */
    int32_t device;     /* CUDA device ordinal */
    int32_t use_graph;  /* capture the whole step in one CUDA graph (default 1) */
} qgt_plan_options_t;

typedef struct qgt_plan qgt_plan_t;

typedef struct {
    int32_t num_qubits, num_params, num_slots, num_rows;  /* rows = 2 + slots (psi, H psi, derivatives) */
    int32_t num_passes, num_launches;                      /* tile passes; kernels per step */
    int32_t tile_bits;                                     /* largest tile (qubits held on chip) */
    int64_t vector_passes;                                 /* sum over passes of vectors processed */
    int64_t gate_bytes;                                    /* algorithmic HBM bytes of the gate passes per step */
    int64_t gram_flops;                                    /* 4 P (P+1) N: algorithmic Gram flops per step */
    int64_t device_bytes;                                  /* device memory held by the plan */
} qgt_plan_info_t;

/* Default options: MIXED, TFIM J = h = 1, lambda = 1e-3, device 0, graph on. */
void qgt_plan_default_options(qgt_plan_options_t* opt);

/* Compile a circuit into a GB300 plan: pass schedule, device buffers, tensor
 * maps and (optionally) one CUDA graph for the whole step.
 * Replaces the per-element evaluation behind geometric_compute_full_qgt
 * (src/quantum_geometric/core/quantum_geometric_curvature.c:289-320). */
int qgt_plan_create(const qgt_circuit_desc_t* circuit, const qgt_plan_options_t* opt,
                    qgt_plan_t** plan);
void qgt_plan_destroy(qgt_plan_t* plan);
int qgt_plan_get_info(const qgt_plan_t* plan, qgt_plan_info_t* info);

/* One step from HOST buffers: copies theta in, runs QGT + energy gradient +
 * natural-gradient step, copies the requested outputs out, synchronises.
 *   Q       P x P complex (Q_mn, row-major), metric = Re Q, Berry curvature = Im Q
 *   grad    P      dE/dtheta (NULL allowed; needs a Hamiltonian)
 *   energy  1      <psi|H|psi>
 *   natgrad P      (Re Q + lambda I)^{-1} grad
 * Any output may be NULL. */
int qgt_plan_execute_host(qgt_plan_t* plan, const double* theta, double* Q, double* grad,
                          double* energy, double* natgrad);

/* The same step on DEVICE pointers (theta and outputs resident in HBM),
 * enqueued on the plan's stream without synchronising. */
int qgt_plan_execute_device(qgt_plan_t* plan, const double* theta_dev, double* Q_dev,
                            double* grad_dev, double* energy_dev, double* natgrad_dev);
int qgt_plan_synchronize(qgt_plan_t* plan);
/* cudaStream_t of the plan (all of its kernels run there). */
void* qgt_plan_stream(qgt_plan_t* plan);
/* Final state psi (2^n complex) of the last step, to a host buffer. */
int qgt_plan_get_state(qgt_plan_t* plan, double* psi);
/* Row r of the plan's vector buffer after the last step, as 2^n complex
 * doubles: r = 0 psi, r = 1 (H psi)/hscale, r = 2 + s derivative slot s
 * (d psi / d angle of the s-th parameterised gate).  FP64 plans only.
 * Replaces compute_quantum_gradient's state output
 * (src/quantum_geometric/core/quantum_geometric_gradient.c:1062). */
int qgt_plan_get_row(qgt_plan_t* plan, int row, double* out);
/* Status of the last step's device checks: 0 ok, otherwise a qgt_error_t
 * (e.g. the Cholesky solve found no positive pivot after its retries). */
int qgt_plan_device_status(qgt_plan_t* plan, double* lambda_used);

/* Device time of each phase of one step, from CUDA events recorded between
 * the phases on the plan's stream (the step runs eagerly, not from the graph;
 * theta already on the device).  The reference's closest facility is the
 * named-span profiler of src/quantum_geometric/core/quantum_geometric_profiling.c:12-110. */
typedef struct {
    double total_ms;
    double prepare_ms;      /* theta -> gate matrices */
    double passes_ms;       /* all tile passes (state + derivative evolution) */
    double hamiltonian_ms;  /* H psi */
    double gram_ms;         /* Gram contraction + split-K reduction */
    double post_ms;         /* projector, energy, gradient */
    double solve_ms;        /* natural-gradient Cholesky solve */
} qgt_step_profile_t;
int qgt_plan_profile_step(qgt_plan_t* plan, qgt_step_profile_t* prof);

/* One-shot helpers over a temporary plan (reference-style convenience). */
int qgt_compute_qgt_f64(const qgt_circuit_desc_t* circuit, const double* theta, double* Q,
                        qgt_precision_t precision);
int qgt_natgrad_step_f64(const qgt_circuit_desc_t* circuit, const double* theta,
                         const qgt_plan_options_t* opt, double* Q, double* grad,
                         double* energy, double* natgrad);

/* Q (P x P complex) from caller-supplied states: psi (dim complex) and the
 * derivative states D (P x dim complex, row k = d psi / d theta_k).  FP64:
 * Gram in FP64 on the GPU; MIXED / MIXED_BF16X3: states rounded to complex64,
 * split, tensor-core Gram; FP64 projector in all cases.  Replaces the serial
 * contraction of diffgeo_compute_fubini_study / diffgeo_compute_berry_curvature
 * (src/quantum_geometric/distributed/differential_geometry.c:2819-2906). */
int qgt_qgt_from_states(const double* psi, const double* D, int64_t dim, int32_t P,
                        qgt_precision_t precision, double* Q);

/* (Re Q + lambda I) x = g by FP64 Cholesky on the GPU, lambda x10 retries
 * (learning/quantum_pipeline_impl.c:1601-1682); A is P x P real, host buffers. */
int qgt_cholesky_solve_f64(const double* A, const double* g, double lambda, int32_t P,
                           double* x, double* lambda_used);

/* The same solve with no device allocation (no counterpart in the reference):
 * every device buffer comes from one static array sized for P up to
 * QGT_NOALLOC_SOLVE_MAX_P; larger P is rejected with an error.  For callers
 * whose device memory belongs to another allocator, or that cannot take
 * cudaFree's device-wide synchronisation in a loop.  The first call on each
 * device (that device current) looks up the array's address; make it before
 * any stream capture begins there.  Calls overlapping in time on one device
 * share the array and race: serialise them. */
#define QGT_NOALLOC_SOLVE_MAX_P 512
int qgt_cholesky_solve_f64_noalloc(const double* A, const double* g, double lambda, int32_t P,
                                   double* x, double* lambda_used);

/* Thread-local text of the last error. */
const char* qgt_last_error(void);
/* Library version string. */
const char* qgt_version(void);

#ifdef __cplusplus
}
#endif
#endif
