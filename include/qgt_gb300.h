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
    QGT_HAMILTONIAN_TFIM = 1,
    /* sum_k c_k P_k over Pauli strings (pauli_strings / pauli_coeffs of the
     * options), the convention of compute_pauli_expectation
     * (src/quantum_geometric/hybrid/quantum_classical_algorithms.c:320-382):
     * character [n-1-q] of a string acts on qubit q, X / Y / Z in either case,
     * any other character is the identity */
    QGT_HAMILTONIAN_PAULI = 2
} qgt_hamiltonian_t;

typedef struct {
    qgt_precision_t precision;
    qgt_hamiltonian_t hamiltonian;
    double tfim_J, tfim_h;
    double lambda;      /* Tikhonov lambda of the natural-gradient step (Re Q + lambda I) x = grad E */
    int32_t device;     /* CUDA device ordinal */
    int32_t use_graph;  /* capture the whole step in one CUDA graph (default 1) */
    /* parameter points evaluated per step (default 1): theta is batch x
     * num_params, every output one block per point; all points share one
     * launch per kernel (the point is a grid dimension) */
    int32_t batch;
    /* parameters [0, num_deriv_params) get derivative states and the outputs
     * are num_deriv_params wide (Q: Pd x Pd, grad / natgrad: Pd); the others
     * only set gate angles.  0 = all num_params. */
    int32_t num_deriv_params;
    /* QGT_HAMILTONIAN_PAULI: num_pauli_terms strings of num_qubits characters
     * back to back (term k at pauli_strings + k n) and their real coefficients;
     * copied at plan creation */
    int32_t num_pauli_terms;
    const char* pauli_strings;
    const double* pauli_coeffs;
    /* how derivative states reach the Gram: QGT_TRANSPORT_AUTO (meet in the
     * middle for mixed plans with >= 16 derivative slots, forward otherwise),
     * QGT_TRANSPORT_FORWARD (every state carried to the end of the circuit),
     * QGT_TRANSPORT_MEET (states of the first half carried forward to a cut,
     * those of the second half carried backward to it from the end through
     * the inverse gates; inner products are unchanged by the common unitary,
     * so Q is the same with about half the gate work) */
    int32_t transport;
    /* register tile of complex64 plans from 14 qubits: 0 = automatic (14 qubits when that saves at
     * least 8 % of the vector passes, else 13), 13 or 14 */
    int32_t tile_bits;
    /* pass kernels of complex64 plans on 13- / 14-qubit tiles: QGT_PASS_AUTO (each pass program
     * compiled into its own straight-line kernel at plan creation from 13 qubits, the program
     * interpreter below), QGT_PASS_INTERPRET, QGT_PASS_COMPILED; the environment variable
     * QGT_PASS_JIT=0 / 1 overrides it */
    int32_t pass_kernels;
    /* amplitudes each thread holds in registers on 13- / 14-qubit complex64 (MIXED) tiles: 0 or
     * 32, or 16 (twice the threads per tile and twice the warps per SM, about a quarter more
     * re-layouts; faster for some circuits, slower for others: qgt_plan_autotune measures it).
     * 16 needs compiled pass kernels. */
    int32_t thread_amps;
} qgt_plan_options_t;
enum { QGT_TRANSPORT_AUTO = 0, QGT_TRANSPORT_FORWARD = 1, QGT_TRANSPORT_MEET = 2 };
enum { QGT_PASS_AUTO = 0, QGT_PASS_INTERPRET = 1, QGT_PASS_COMPILED = 2 };

typedef struct qgt_plan qgt_plan_t;

typedef struct {
    int32_t num_qubits, num_params, num_slots, num_rows;  /* rows = 2 + slots (psi, H psi, derivatives) */
    int32_t num_passes, num_launches;                      /* tile passes; kernels per step */
    int32_t tile_bits;                                     /* largest tile (qubits held on chip) */
    int64_t vector_passes;                                 /* sum over passes of vectors processed */
    int64_t gate_bytes;                                    /* algorithmic HBM bytes of the gate passes per step */
    int64_t gram_flops;                                    /* 4 P (P+1) N: algorithmic Gram flops per step */
    int64_t device_bytes;                                  /* device memory held by the plan */
    int32_t batch, num_deriv_params;                       /* points per step; output width Pd */
    int32_t meet_in_middle, cut_gate;                      /* transport used; first gate of the backward half */
    int32_t jit_passes;                                    /* passes running as compiled straight-line kernels */
    int32_t thread_amps;                                   /* amplitudes per thread of the register tiles */
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
 * Any output may be NULL.  With batch B and Pd derivative parameters theta is
 * B x num_params and the outputs B x Pd x Pd, B x Pd, B, B x Pd. */
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
 * (d psi / d angle of the s-th parameterised gate).  With meet-in-the-middle
 * transport the rows are those states carried to the cut (U_2^dagger applied,
 * U_2 the gates from the cut on), which leaves every inner product as it is.
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

/* ---- ragged batches ------------------------------------------------------
 * Many circuits (any mix of qubit counts, depths and parameters) evaluated
 * by ONE CUDA-graph launch.  Circuits with the same structure share one
 * batched plan (the parameter point is a grid dimension of every kernel);
 * optionally each circuit also gets a G x G Berry-curvature map
 * Omega_ab(theta_a, theta_b) = Im Q_ab over two of its parameters on the
 * lattice theta = 2 pi k / G, k = 0 .. G-1, the other parameters at the
 * circuit's theta.  The reference has no batch interface: it evaluates each
 * circuit through geometric_compute_full_qgt
 * (src/quantum_geometric/core/quantum_geometric_curvature.c:289-320) and the
 * pointwise curvature of quantum_geometric_curvature.c:181-198. */
typedef struct qgt_batch qgt_batch_t;

typedef struct {
    qgt_precision_t precision;  /* QGT_PRECISION_FP64 or QGT_PRECISION_MIXED */
    int32_t berry_grid;         /* G (0 = no maps; default 32) */
    int32_t device;
    int32_t streams;            /* concurrent branches inside the graph (default 4, max 16) */
    /* autotuning cache (qgt_plan_autotune): each structural group's plan takes the fastest
     * configuration found for it, timing the groups not in the file yet; NULL = no tuning */
    const char* tune_cache;
} qgt_batch_options_t;

typedef struct {
    int32_t num_circuits, num_groups, num_berry_plans;
    int32_t graph_kernels;      /* kernels and copies per batch launch */
    int64_t device_bytes;
} qgt_batch_info_t;

void qgt_batch_default_options(qgt_batch_options_t* opt);
/* berry_params: 2 per circuit (a, b), required when berry_grid > 0. */
int qgt_batch_create(const qgt_circuit_desc_t* circuits, int32_t count, const int32_t* berry_params,
                     const qgt_batch_options_t* opt, qgt_batch_t** batch);
/* theta: the circuits' parameter vectors back to back (num_params each);
 * Q: their P x P complex QGTs back to back (NULL allowed); berry: count x G x G
 * doubles, map[i][j] at (theta_a, theta_b) = (2 pi i / G, 2 pi j / G) (NULL allowed). */
int qgt_batch_execute_host(qgt_batch_t* batch, const double* theta, double* Q, double* berry);
/* the batch's work on the inputs already on the device (the thetas of the last
 * qgt_batch_execute_host), results left on the device: one graph launch on
 * qgt_batch_stream(batch), asynchronous (measurement of the device-resident batch) */
int qgt_batch_execute_device(qgt_batch_t* batch);
void* qgt_batch_stream(const qgt_batch_t* batch);
int qgt_batch_get_info(const qgt_batch_t* batch, qgt_batch_info_t* info);
void qgt_batch_destroy(qgt_batch_t* batch);

/* ---- plaquette Berry flux over a two-parameter lattice ------------------
 * The Wilson-loop curvature of the reference's berry_curvature_kernel
 * (src/cuda/quantum_phase_cuda.cu:245-313): for the plaquette at site (i, j)
 * W = <p00|p10> <p10|p11> <p11|p01> <p01|p00> and flux = arg W (0 when
 * |W| <= 1e-15), with p_kl the site (i + k, j + l).  There a site holds one
 * complex number; here it holds the circuit's full state at
 * (theta_a, theta_b) = (a0 + i da, b0 + j db), the other parameters at theta,
 * and each link is a 2^n-amplitude inner product on the GPU.  For small
 * spacings flux ~ 2 Im Q_ab da db at the plaquette centre.  The states of a
 * block of lattice rows are made by one theta-batched plan; with periodic = 1
 * site rows and columns wrap (a torus: the fluxes of all rows x cols
 * plaquettes sum to 2 pi times an integer), with periodic = 0 the last row and
 * column of flux are 0 as in the reference kernel. */
typedef struct {
    int32_t param_a, param_b;   /* distinct indices into theta */
    int32_t rows, cols;         /* sites along theta_a and theta_b, each in [2, 4096] */
    double a0, da, b0, db;      /* site (i, j) at theta_a = a0 + i da, theta_b = b0 + j db */
    int32_t periodic;
    qgt_precision_t precision;  /* QGT_PRECISION_FP64 or QGT_PRECISION_MIXED (complex64 states) */
    int32_t device;
} qgt_flux_options_t;

/* Defaults: params 0 and 1, 32 x 32 sites on [0, 2 pi)^2, periodic, MIXED, device 0. */
void qgt_flux_default_options(qgt_flux_options_t* opt);
/* flux: rows x cols doubles (row-major, flux[i * cols + j]); total (NULL
 * allowed): their sum. */
int qgt_berry_flux_grid(const qgt_circuit_desc_t* circuit, const double* theta, const qgt_flux_options_t* opt,
                        double* flux, double* total);

/* ---- learned metric preconditioner -------------------------------------
 * No reference counterpart.  A 3-layer MLP (hidden width W, BF16 weights,
 * FP32 accumulation) maps theta (P) to M = diag(d) + U U^T (U: P x r)
 * approximating Re Q + lambda I; trained on the GPU by hand-written forward,
 * backward and Adam kernels on exact metrics that theta-batched plans
 * generate; used as the preconditioner of a GPU PCG natural-gradient solve.
 * The exact-metric Cholesky step stays the reference solve
 * (src/quantum_geometric/learning/quantum_pipeline_impl.c:1601-1682); the
 * unpreconditioned CG it is compared with is
 * src/quantum_geometric/hybrid/classical_optimization_engine.c:543-611. */
typedef struct qgt_precond qgt_precond_t;

typedef struct {
    int32_t num_params;  /* P (1 .. 1024) */
    int32_t width;       /* hidden width (default 512) */
    int32_t rank;        /* r of U (default 16, max 32) */
    double lambda;       /* target Re Q + lambda I; d >= lambda (default 1e-3) */
    double u_scale;      /* U = u_scale x raw outputs (default 0.1) */
    uint64_t seed;       /* weight initialisation */
    int32_t device;
} qgt_precond_config_t;

typedef struct {
    int32_t epochs;      /* default 30 */
    int32_t batch;       /* default 256 (full batches only) */
    double lr;           /* Adam learning rate (default 1e-3) */
    double weight_decay; /* default 0 */
    uint64_t seed;       /* shuffling */
} qgt_precond_train_options_t;

void qgt_precond_default_config(qgt_precond_config_t* cfg);
void qgt_precond_default_train_options(qgt_precond_train_options_t* opt);
int qgt_precond_create(const qgt_precond_config_t* cfg, qgt_precond_t** pc);
void qgt_precond_destroy(qgt_precond_t* pc);
/* weights as FP32 masters: W1 (W x 2P), b1 (W), W2 (W x W), b2 (W),
 * W3 (O x W), b3 (O), O = P + P r; the products use their BF16 rounding.
 * Input features are [cos theta, sin theta]; d = softplus(o[0:P]) + lambda,
 * U = u_scale o[P:] (row-major P x r). */
int64_t qgt_precond_num_weights(const qgt_precond_t* pc);
int qgt_precond_get_weights(const qgt_precond_t* pc, float* w);
int qgt_precond_set_weights(qgt_precond_t* pc, const float* w);
/* exact metrics Re Q of S parameter points (theta S x P) on the GPU: metric S x P x P */
int qgt_metric_dataset(const qgt_circuit_desc_t* circuit, const double* theta, int32_t S,
                       qgt_precision_t precision, int32_t device, double* metric);
/* train on host pairs (theta S x P, metric S x P x P); loss_history: epochs (NULL allowed) */
int qgt_precond_train(qgt_precond_t* pc, const double* theta, const double* metric, int32_t S,
                      const qgt_precond_train_options_t* opt, double* loss_history);
/* train on the exact metrics of a circuit at S parameter points, generated on the GPU */
int qgt_precond_train_circuit(qgt_precond_t* pc, const qgt_circuit_desc_t* circuit, const double* theta,
                              int32_t S, qgt_precision_t precision, const qgt_precond_train_options_t* opt,
                              double* loss_history);
/* mean loss ||M - T||_F^2 / ||T||_F^2 over S samples and its gradient (num_weights floats), no update */
int qgt_precond_loss_grad(qgt_precond_t* pc, const double* theta, const double* metric, int32_t S,
                          double* loss, float* grad);
/* d (S x P) and U (S x P x r) for S parameter points */
int qgt_precond_predict(qgt_precond_t* pc, const double* theta, int32_t S, double* d, double* U);

/* PCG on the GPU: (A + lambda I) x = b, A real P x P (host buffers);
 * M = diag(d) + U U^T by Woodbury (d NULL: identity; r = 0: diagonal only).
 * Stops at ||r|| <= tol ||b|| or max_iter; iters / resid: what it reached. */
int qgt_pcg_solve_f64(const double* A, const double* b, double lambda, int32_t P, const double* d,
                      const double* U, int32_t r, double tol, int32_t max_iter, double* x,
                      int32_t* iters, double* resid);

/* Natural-gradient VQE on the TFIM ring: theta <- theta - eta x per step, x
 * from the exact Cholesky step, from CG, or from PCG with the learned
 * preconditioner; the whole loop is enqueued on the device (one graph
 * launch, one solve and one update per step).  Reference loop:
 * src/quantum_geometric/hybrid/quantum_classical_algorithms.c:854-886. */
enum { QGT_VQE_SOLVER_CHOLESKY = 0, QGT_VQE_SOLVER_CG = 1, QGT_VQE_SOLVER_PCG_LEARNED = 2 };
typedef struct {
    int32_t steps;        /* default 500 */
    double eta;           /* default 0.05 */
    double pcg_tol;       /* relative residual (default 1e-10) */
    int32_t pcg_max_iter; /* default 1000 */
    int32_t solver;       /* QGT_VQE_SOLVER_* (default Cholesky) */
} qgt_vqe_options_t;
void qgt_vqe_default_options(qgt_vqe_options_t* opt);
/* energies: steps values E(theta_t) before each update; pcg_iters: steps (NULL allowed) */
int qgt_vqe_run(const qgt_circuit_desc_t* circuit, const qgt_plan_options_t* plan_opt, qgt_precond_t* pc,
                const qgt_vqe_options_t* opt, const double* theta0, double* energies, int32_t* pcg_iters,
                double* theta_out);

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

/* Fault-injection hook for tests of the failure path (no reference
 * counterpart).  Every mbarrier wait of the integer-digit Gram kernel is
 * bounded by the GPU's global timer; when one runs out the CTA stops, waits
 * (bounded) for its own TMA loads and MMAs in flight, frees its tensor memory
 * and records QGT_ERROR_TIMEOUT, which the step then returns.  With stall = 1
 * the kernel's converter warps wait on a barrier that nothing arrives on, so
 * that limit (timeout_ns, in (0, 4e9]) runs out on purpose; stall = 0 and
 * timeout_ns = 0 restore the default (no stall, 4 s limit).  Plans of
 * MIXED precision with more than 8 rows only; no GPU fault is involved. */
int qgt_plan_test_gram_stall(qgt_plan_t* plan, int stall, int64_t timeout_ns);

/* ---- autotuning --------------------------------------------------------
 * Times the candidate configurations of a circuit's plan on the GPU (the
 * register tile, 13 or 14 qubits; interpreted or compiled pass kernels; 32
 * or 16 amplitudes per thread with compiled kernels) for the given base options
 * (precision, batch, derivative parameters, Hamiltonian), each over `steps`
 * graph launches after two warm-up steps, and returns the fastest as *tuned
 * (base with tile_bits, pass_kernels and thread_amps set) and its time per
 * step.  Results are kept in the text file cache_path
 * (one line per circuit structure and base options; NULL: no file): a circuit
 * already in the file is not timed again.  No reference counterpart. */
int qgt_plan_autotune(const qgt_circuit_desc_t* circuit, const qgt_plan_options_t* base, const char* cache_path,
                      int32_t steps, qgt_plan_options_t* tuned, double* best_ms);

/* Thread-local text of the last error. */
const char* qgt_last_error(void);
/* Library version string. */
const char* qgt_version(void);

#ifdef __cplusplus
}
#endif
#endif
