/*
 * qgt_internal.h -- structures shared by the C host (pass compiler, plan
 * driver, reference API) and the CUDA translation units, and the thin
 * qgt_dev_* C ABI through which host code reaches the device.
 *
 * Data layout in HBM (per plan):
 *   V       (rows + 1) x N amplitudes, complex128 (FP64 plan) or complex64
 *           (mixed plan).  Row 0 = psi, row 1 = H psi, row 2 + s = derivative
 *           slot s; row `rows` is the second psi buffer (psi ping-pongs
 *           between row 0 and row `rows` across passes, ending in row 0).
 *   SPLIT   (mixed only) 4 planes {Re hi, Re lo, Im hi, Im lo} x rows_pad x N
 *           half-precision values, K-major (amplitude index contiguous), the
 *           operands of the tensor-core Gram.
 *   PART    split-K partial Gram blocks; HG = (rows x rows) complex FP64 Gram.
 */
#ifndef QGT_INTERNAL_H
#define QGT_INTERNAL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QGT_MAX_QUBITS 30
#define QGT_TILE_MAX_F32 13   /* 2^13 complex64 = 64 KiB of shared memory */
#define QGT_TILE_WIDE_F32 14  /* 2^14 complex64 = 128 KiB: registers tiles of 512 threads, from 14 qubits */
#define QGT_TILE_MAX_F64 12   /* 2^12 complex128 = 64 KiB */
#define QGT_LANE_BITS 5       /* qubits 0..4 are always tile bits: 256 B coalesced segments */
#define QGT_PASS_THREADS 256

/* ops of a tile pass (one per gate, in pass order) */
enum {
    QOP_1Q = 1,     /* dense 2x2 on tile bit lb (coef: m00 m01 m10 m11) */
    QOP_PHASE = 2,  /* diag(p0, p1) on qubit q (coef: m00 = p0, m11 = p1) */
    QOP_CZ = 3,     /* -1 on |11> of qubits (q, q2) */
    QOP_CNOT = 4,   /* X on tile bit lb when qubit q2 (control) is 1 */
    QOP_SWAP = 5    /* swap tile bits lb and lb2 */
};

/* generator inserted for a derivative: (-i/2) G after the op */
enum { QGEN_NONE = 0, QGEN_X = 1, QGEN_Y = 2, QGEN_Z = 3 };

typedef struct {
    int8_t kind;    /* QOP_* */
    int8_t lb;      /* tile-local bit of the target / first qubit, -1 if outside the tile */
    int8_t lb2;     /* tile-local bit of the second qubit (CNOT control, CZ/SWAP second), or -1 */
    int8_t gen;     /* QGEN_* for parameterised rotations */
    int8_t q;       /* physical qubit of lb */
    int8_t q2;      /* physical qubit of lb2 */
    int16_t pad;
    int32_t coef;   /* coefficient index, -1 if none */
    int32_t slot;   /* derivative slot of this gate, -1 if none */
} qgt_dev_op_t;

/* gate coefficient source: the prepare kernel turns theta into matrices;
 * type | QGT_COEF_INVERSE asks for the gate's inverse */
#define QGT_COEF_INVERSE 0x100
typedef struct {
    int32_t type;   /* QGT_GATE_* */
    int32_t param;  /* theta index, -1 = fixed */
    double angle;
} qgt_dev_coef_desc_t;

enum {
    QENT_STORE_V = 1,      /* write the result to V[dst_row] */
    QENT_STORE_SPLIT = 2,  /* write the result to SPLIT row split_row */
    QENT_SRC_ZERO = 4,     /* source is |0...0> (no read) */
    QENT_ROWMAX = 8        /* atomically fold max |x| of the result into rowmax[dst_row] */
};

typedef struct {
    int32_t src_row;
    int32_t dst_row;
    int32_t spawn_op;   /* op index (in the pass) after which (-i/2)G is inserted; -1 = transport */
    int32_t flags;      /* QENT_* */
    int32_t split_row;
    int32_t start_op;   /* register-resident passes: the entry runs the pass program from this op (a
                           Q2_SEG) on; 0 = the whole program */
    int8_t lay[32];     /* register-resident passes: the layout of op start_op (its 16 local bits,
                           then their physical qubits), so that the tile loads need no program */
} qgt_dev_entry_t;

typedef struct {
    void* V;                        /* vector buffer (c64 or c128) */
    int64_t N;                      /* 2^n */
    const qgt_dev_op_t* ops;        /* device pointer to this pass's ops */
    int32_t nops;
    const qgt_dev_entry_t* entries; /* device pointer */
    int32_t nentries;
    const double* coef;             /* device coefficient table, 8 doubles per coef */
    void* split;                    /* SPLIT base (mixed) */
    int64_t split_ld;               /* row length of a split plane (N rounded up to 32) */
    int64_t split_plane_stride;     /* elements between planes = rows_pad * split_ld */
    float split_scale;              /* power of two applied before splitting */
    int32_t split_bf16;             /* 0: FP16 planes, 1: BF16 planes */
    int32_t n;
    int32_t tile_bits;
    uint32_t tile_mask;             /* physical qubits held in the tile */
    int8_t local_to_phys[16];
    uint32_t* rowmax;               /* per-row max |amplitude| as float bits (QENT_ROWMAX) */
    /* parameter-point batch: grid.z = point; point p works on V + p point_stride
     * (amplitudes), coefficients + p coef_stride and rowmax + p rowmax_stride
     * (npoints 0 = one point) */
    int32_t npoints;
    int32_t coef_stride;
    int64_t point_stride;
    int32_t rowmax_stride;
} qgt_dev_pass_args_t;

/* ---- register-resident passes (qgt_pass2.cu) ----
 * A pass program is a list of ops; Q2_SEG ops switch the layout (which local
 * bits are register bits / warp bits) through shared memory.  Bits are
 * role-encoded: 0..4 lane bit, 8 + i register bit i, 16 + w warp bit w,
 * 32 outside the tile (physical qubit in q / q2). */
enum { Q2_SEG = 1, Q2_U = 2, Q2_UR = 3, Q2_PHASE = 4, Q2_CZ = 5, Q2_CNOT = 6, Q2_DIAG = 7,
       Q2_CZT = 9,    /* in a diagonal run: the thread factor flips when thread bit q and popc(thread bits & slot) are odd */
       Q2_ZGEN = 10,  /* in a diagonal run: marks a derivative spawned by the rotation on (ra, q) */
       Q2_UM = 11 };  /* header of `seg` commuting Q2_U / Q2_UR ops on distinct bits: `ra` lane ops, then one
                         op per register bit set in `rb`, ascending */
/* Q2_DIAG: header of a run of diagonal gates applied as one per-thread phase
 * table; `seg` sub-ops follow: RB register-bit entries (Q2_PHASE on register
 * bit i = 0 .. RB-1 in order, coef -1 = no phase, slot = the physical qubits
 * outside the register bits that share a CZ with bit i), then `ra` thread
 * phase entries (Q2_PHASE on a lane, warp or outside qubit), then `rb` Q2_CZT
 * entries, then Q2_ZGEN markers.  The header's `slot` is the sign mask over
 * the register index of the run's CZs between two register bits. */
typedef struct {
    uint8_t kind;
    uint8_t ra;     /* target / first bit (role-encoded) */
    uint8_t rb;     /* control / second bit (role-encoded) */
    uint8_t gen;    /* QGEN_* inserted after this op for a spawn entry */
    int8_t q, q2;   /* physical qubits of ra / rb */
    int16_t seg;    /* Q2_SEG: layout index */
    int32_t coef;
    int32_t slot;
} qgt_dev_op2_t;

typedef struct {
    void* V;
    int64_t N;
    const qgt_dev_op2_t* ops;       /* program; ops[0] is the initial Q2_SEG */
    int32_t nops;
    const int8_t* segs;             /* 16 per layout: [0, RB) register local bits, [8, 11) warp local bits */
    const qgt_dev_entry_t* entries; /* spawn_op = program index */
    int32_t nentries;
    const double* coef;             /* FP64 coefficients (complex128 path) */
    const float* coef32;            /* complex64 coefficients with exact angles */
    void* split;
    int64_t split_ld, split_plane_stride;
    float split_scale;
    int32_t n, tile_bits;
    uint32_t tile_mask;
    int8_t local_to_phys[16];
    uint32_t* rowmax;
    int32_t npoints;                /* batch fields as in qgt_dev_pass_args_t */
    int32_t coef_stride;
    int64_t point_stride;
    int32_t rowmax_stride;
    int32_t ckpt;                   /* 1: the entries store their state before every Q2_SEG op with slot >= 0
                                       into row slot (checkpoints for spawns that start at that segment) */
} qgt_dev_pass2_args_t;
int qgt_dev_pass2(const qgt_dev_pass2_args_t* args, int fp64, void* stream);

/* ---- pass programs compiled to straight-line kernels (qgt_jit.c, qgt_jit_rt.cu) ---- */
typedef struct {
    const qgt_dev_op2_t* prog;  /* the pass program (prog[0] is its initial Q2_SEG) */
    int32_t nops;
    const int8_t* segs;         /* layouts, 16 per index (as qgt_dev_pass2_args_t.segs) */
    const int8_t* l2p;          /* local bit -> physical qubit of the pass's tile */
    int32_t n, tile_bits, RB, WB;
    uint32_t tile_mask;
    int32_t ckpt;               /* 1: entries store checkpoints before Q2_SEG ops with slot >= 0 */
    const int32_t* starts;      /* program indices at which the launched entries start */
    const int8_t* start_zero;   /* per start: 1 if an entry starting there reads |0...0> (QENT_SRC_ZERO) */
    int32_t nstarts;
    const char* kname;          /* kernel name */
} qgt_jit_pass_desc_t;
/* CUDA source of one pass program (malloc'd; NULL and an error message on failure) */
char* qgt_jit_pass_source(const qgt_jit_pass_desc_t* d);
typedef struct qgt_jit_kernel qgt_jit_kernel_t;
/* compile (or take from the process / disk cache) and load for `device`; smem = dynamic shared bytes,
 * nthreads = the kernel's block size (its __launch_bounds__) */
int qgt_dev_jit_compile(const char* body, const char* kname, int32_t smem, int32_t nthreads, int32_t device,
                        qgt_jit_kernel_t** out);
/* launch over the entries of a, as qgt_dev_pass2 (complex64 register tiles only) */
int qgt_dev_jit_launch(const qgt_jit_kernel_t* k, const qgt_dev_pass2_args_t* a, void* stream);
/* seconds spent in the compiler by this process (cache hits cost nothing) */
double qgt_dev_jit_compile_seconds(void);
/* compile a pass kernel body without loading it (no device needed); *seconds = compile time */
int qgt_jit_nvrtc_check(const char* body, double* seconds);
/* every compiled pass kernel of a plan, without a device (qgt_plan.c): sources to dump_dir (NULL:
 * none), compile = 1 also runs each through the compiler; returns the kernel count or an error */
int qgt_plan_jit_check(const void* circuit, const void* options, const char* dump_dir, int compile, double* seconds);
/* rho[point][m] = product over groups 0..m of the amplitude scales |column 0|
 * of the complex64 coefficient entries src[ptr[g] .. ptr[g+1]) */
/* per pass and point: multiply the pass's designated entry ren[pass] by 1 / prod of the scales
 * (|column 0|) of the pass's entries src[ptr[pass] .. ptr[pass + 1]) (complex64 tables) */
int qgt_dev_renorm_passes(float* coef32, int32_t coef_stride, const int32_t* ptr, const int32_t* src,
                          const int32_t* ren, int32_t npasses, int32_t npoints, void* stream);
int qgt_dev_scale_product(const float* coef32, int32_t coef_stride, const int32_t* ptr, const int32_t* src,
                          int32_t ngroups, double* rho, int32_t npoints, void* stream);
int qgt_dev_prepare32(const qgt_dev_coef_desc_t* descs_dev, int32_t ncoef, const double* theta_dev,
                      float* coef32_dev, int32_t npoints, int32_t theta_stride, int32_t coef_stride, void* stream);

/* internal plan helpers used by the reference API layer and the batch driver */
struct qgt_plan;
int qgt_plan_combine_slots(struct qgt_plan* p, const double* c, double* out);
/* enqueue one step of the plan on `stream` (theta already in qgt_plan_dev_theta) */
int qgt_plan_enqueue_step(struct qgt_plan* p, void* stream);
double* qgt_plan_dev_theta(struct qgt_plan* p);   /* batch x num_params */
double* qgt_plan_dev_Q(struct qgt_plan* p);       /* batch x Pd x Pd complex */
int qgt_plan_launches(const struct qgt_plan* p);
/* the host-side schedule of a circuit as JSON, without a device (circuit /
 * options: qgt_circuit_desc_t / qgt_plan_options_t of qgt_gb300.h) */
int qgt_plan_schedule_dump(const void* circuit, const void* options, const char* path);
/* the same with the segment checkpoints of the register-tile passes (a writer entry first; entries
 * that start at a later segment read its checkpoint row) */
int qgt_plan_schedule_dump_ckpt(const void* circuit, const void* options, const char* path);

/* thread-local last error (host/qgt_error.c): stores the message and returns code */
int qgt_set_error(int code, const char* fmt, ...);
void qgt_clear_error(void);

/* ---- device context / memory (qgt_device.cu) ---- */
int qgt_dev_set_device(int device);
int qgt_dev_malloc(void** p, size_t bytes);
int qgt_dev_free(void* p);
int qgt_dev_memcpy_h2d(void* dst, const void* src, size_t bytes, void* stream);
int qgt_dev_memcpy_d2h(void* dst, const void* src, size_t bytes, void* stream);
int qgt_dev_memcpy_d2d(void* dst, const void* src, size_t bytes, void* stream);
int qgt_dev_memset(void* dst, int value, size_t bytes, void* stream);
int qgt_dev_stream_create(void** stream);
int qgt_dev_stream_destroy(void* stream);
int qgt_dev_stream_sync(void* stream);
int qgt_dev_graph_begin(void* stream);
int qgt_dev_graph_end(void* stream, void** exec);
int qgt_dev_graph_launch(void* exec, void* stream);
int qgt_dev_graph_destroy(void* exec);
int qgt_dev_host_alloc(void** p, size_t bytes);   /* pinned */
int qgt_dev_host_free(void* p);
int qgt_dev_last_error(void);                     /* cudaGetLastError as qgt_error_t */
const char* qgt_dev_error_string(void);

int qgt_dev_event_create(void** ev);
int qgt_dev_event_destroy(void* ev);
int qgt_dev_event_record(void* ev, void* stream);
int qgt_dev_event_sync(void* ev);
int qgt_dev_stream_wait_event(void* stream, void* ev);
int qgt_dev_event_elapsed(void* start, void* end, float* ms);

/* ---- kernels ---- */
/* gate matrices for npoints parameter points: theta + p theta_stride -> coef + 8 p ncoef */
int qgt_dev_prepare(const qgt_dev_coef_desc_t* descs_dev, int32_t ncoef, const double* theta_dev,
                    double* coef_dev, int32_t npoints, int32_t theta_stride, int32_t coef_stride, void* stream);
/* combined diagonal entries: entry base + k of each point = product of the
 * diagonals (m0 + i m1, m6 + i m7) of entries src[ptr[k] .. ptr[k+1]), in the
 * FP64 table and / or the complex64 table (either may be NULL) */
int qgt_dev_combine_diag(double* coef, float* coef32, int32_t coef_stride, int32_t base, const int32_t* ptr,
                         const int32_t* src, int32_t ncomb, int32_t npoints, void* stream);
int qgt_dev_pass(const qgt_dev_pass_args_t* args, int fp64, void* stream);
/* out (row 1 of V, and split row 1 when split != NULL) = H psi / hscale, for
 * npoints points point_stride amplitudes apart (rowmax slots rowmax_stride apart) */
int qgt_dev_tfim(const void* psi, void* out, int32_t n, double J, double h, double inv_hscale,
                 int fp64, void* split, int64_t split_ld, int64_t split_plane_stride, int32_t split_row,
                 float split_scale, int32_t split_bf16, uint32_t* rowmax_slot, int32_t npoints,
                 int64_t point_stride, int32_t rowmax_stride, void* stream);
/* one Pauli term: P|j> = i^ny (-1)^popc(j & z) |j ^ x> */
typedef struct {
    double c;
    uint32_t x, z;
    int32_t ny, pad;
} qgt_dev_pauli_term_t;
/* out = (sum_k c_k P_k) psi * inv_hscale per point (rowmax slot as for qgt_dev_tfim) */
int qgt_dev_pauli(const void* psi, void* out, int32_t n, const qgt_dev_pauli_term_t* terms, int32_t nterms,
                  double inv_hscale, int fp64, uint32_t* rowmax_slot, int32_t npoints, int64_t point_stride,
                  int32_t rowmax_stride, void* stream);
/* complex128 -> complex64 rows */
int qgt_dev_c128_to_c64(const double* X, int64_t count, float* Y, void* stream);
/* rowmax[row0 + r] = max(rowmax, max_k |V[row0 + r][k]|) over complex64 rows (float bits) */
int qgt_dev_rowmax(const void* V, int64_t N, int32_t row0, int32_t nrows, uint32_t* rowmax, void* stream);
/* mixed-precision Gram of complex64 rows [0, rows) of V with exactly accumulated
 * integer high digits (per-row power-of-two units from rowmax); HG as above */
typedef struct qgt_dg_gram qgt_dg_gram_t;
/* npoints points point_rows rows apart; rowmax holds npoints x rows maxima and
 * HG npoints x rows x rows blocks */
int qgt_dev_dg_gram_create(const void* V, int64_t N, int32_t rows, const uint32_t* rowmax, int32_t npoints,
                           int32_t point_rows, qgt_dg_gram_t** g);
int qgt_dev_dg_gram_run(qgt_dg_gram_t* g, double* HG, void* stream);
int qgt_dev_dg_gram_status(qgt_dg_gram_t* g, void* stream);
/* wait settings read by every later run (tests of the bounded-wait error path): stall = 1 makes the
 * converter warps wait on a barrier nothing arrives on; timeout_ns = each wait's limit (0: 4 s) */
int qgt_dev_dg_gram_set_stall(qgt_dg_gram_t* g, int stall, int64_t timeout_ns, void* stream);
/* device address of the kernel's error flag (int; 0 = no error), for a copy queued with others */
const int* qgt_dev_dg_gram_err(const qgt_dg_gram_t* g);
void qgt_dev_dg_gram_destroy(qgt_dg_gram_t* g);
int64_t qgt_dev_dg_gram_scratch_bytes(const qgt_dg_gram_t* g);
void qgt_dev_dg_gram_shape(const qgt_dg_gram_t* g, int* ntp, int* nsplit, int64_t* kchunk);
/* complex128 rows X (rows x N) -> split planes rows [row0, row0 + rows) */
int qgt_dev_split_rows(const double* X, int32_t rows, int64_t N, void* split, int64_t split_ld, int64_t split_plane_stride,
                       int32_t row0, float scale, int32_t bf16, void* stream);
/* out = sum_k c[k] V[row0 + k] over complex128 rows (c on the device) */
int qgt_dev_combine_rows(const void* V, int64_t N, int32_t row0, const double* c, int32_t K, void* out, void* stream);
/* FP64 Gram of rows [0, rows) of V (complex128): HG = V V^H (HG_ij = <V_i|V_j>),
 * for npoints points point_stride amplitudes apart (part holds
 * npoints x nsplit x tile pairs blocks, HG npoints x rows x rows) */
int qgt_dev_gram_f64(const void* V, int64_t N, int32_t rows, double* part, int32_t nsplit,
                     double* HG, int32_t npoints, int64_t point_stride, void* stream);
/* tensor-core Gram on the split operands; HG as above, scaled back by 1/scale^2 */
typedef struct qgt_tc_gram qgt_tc_gram_t;
int qgt_dev_tc_gram_create(void* split, int64_t N, int32_t rows, int32_t rows_pad, int32_t bf16,
                           qgt_tc_gram_t** g);
int qgt_dev_tc_gram_run(qgt_tc_gram_t* g, double inv_scale2, double* HG, void* stream);
void qgt_dev_tc_gram_destroy(qgt_tc_gram_t* g);
/* device error word of the last run (0 ok, QGT_ERROR_TIMEOUT on an expired wait); synchronises */
int qgt_dev_tc_gram_status(qgt_tc_gram_t* g, void* stream);
const int* qgt_dev_tc_gram_err(const qgt_tc_gram_t* g);
int64_t qgt_dev_tc_gram_scratch_bytes(const qgt_tc_gram_t* g);
/* HG -> Q, grad, energy (FP64 renormalisation + projector + slot->param sum) */
typedef struct {
    const double* HG;
    int32_t rows;           /* 2 + slots */
    int32_t P;              /* parameters */
    const int32_t* slot_param;  /* slot -> param */
    const int32_t* param_ptr;   /* CSR over params: slots of param p = param_slots[param_ptr[p] .. param_ptr[p+1]) */
    const int32_t* param_slots;
    double hscale;          /* H psi row was divided by this */
    int32_t has_h;
    double* Q;              /* P x P complex */
    double* grad;           /* P */
    double* energy;         /* 1 */
    int32_t npoints;        /* parameter points (0 = 1): HG, Q, grad, energy blocks per point */
    /* meet in the middle with complex64 gates: row r carries the extra
     * amplitude scale rho[point][row_group[r]] (row_group < 0: none; rho NULL: no rows) */
    const double* rho;
    const int32_t* row_group;
    int32_t ngroups;
} qgt_dev_post_args_t;
int qgt_dev_post(const qgt_dev_post_args_t* a, void* stream);
/* (Re Q + lambda I) x = b, FP64 Cholesky; A taken as Re of the complex Q when
 * complex_input, else a real P x P matrix.  status[0] = 0 ok / error code,
 * status[1] = lambda used (as double bits in the second slot). */
int qgt_dev_cholesky(const double* A, int complex_input, const double* b, int32_t P,
                     double lambda, double* work, double* x, double* status, void* stream);
/* the same solve, blocked over many CTAs, without retries (status[0] =
 * QGT_ERROR_NOT_POSITIVE_DEFINITE on a non-positive pivot); P <= 2048 */
int qgt_dev_cholesky_blocked(const double* A, int complex_input, const double* b, int32_t P,
                             double lambda, double* work, double* x, double* status, void* stream);
int qgt_dev_cholesky_launches(int32_t P);
/* the same solve with an FP32 blocked factorisation and FP64 iterative
 * refinement (FP64-accurate; status[0] = QGT_ERROR_CONVERGENCE_FAILED or
 * QGT_ERROR_NOT_POSITIVE_DEFINITE asks for the FP64 solver); work holds
 * qgt_dev_cholesky_refined_work(P) doubles; P <= 2048 */
int qgt_dev_cholesky_refined(const double* A, int complex_input, const double* b, int32_t P, double lambda,
                             double* work, double* x, double* status, void* stream);
int64_t qgt_dev_cholesky_refined_work(int32_t P);
int qgt_dev_cholesky_refined_launches(int32_t P);
/* nsys independent single-CTA solves with retries, systems contiguous
 * (A: nsys x P x P, b / x: nsys x P, work: nsys x P x P, status: nsys x 2) */
int qgt_dev_cholesky_batch(const double* A, int complex_input, const double* b, int32_t P, double lambda,
                           double* work, double* x, double* status, int32_t nsys, void* stream);
/* small Gram (rows <= 8) of complex64 (fp64 = 0; FP32 sums of 32-amplitude
 * blocks, added in FP64) or complex128 rows (FP64): HG per point (npoints
 * points point_stride amplitudes apart); skip_row1 = 1 leaves row 1 (H psi of
 * a plan without Hamiltonian) unread and writes its entries as zeros; part
 * holds npoints x nsplit x 36 complex partials */
int qgt_dev_gram_small(const void* V, int64_t N, int32_t rows, int32_t skip_row1, int32_t fp64, double* part,
                       int32_t nsplit, double* HG, int32_t npoints, int64_t point_stride, void* stream);

/* <V + a_off[k] | V + b_off[k]> over N amplitudes (offsets in amplitudes), pair k split in nchunk
 * ranges: part[k * nchunk + c] (complex double) holds the sum over range c */
int qgt_dev_overlaps(const void* V, int32_t fp64, int64_t N, const int64_t* a_off, const int64_t* b_off, int32_t n,
                     int32_t nchunk, double* part, void* stream);
/* chunks per pair that fill the GPU for n pairs of N amplitudes */
int32_t qgt_overlap_chunks(int64_t N, int32_t n);
/* the G x G Berry maps of ncirc circuits from the overlaps of their states at (theta_a, theta_b) in
 * {0, pi}^2 (part: per circuit 10 pairs x nchunk partial sums, qgt_dev_overlaps layout); maps: ncirc
 * x G x G doubles (qgt_gram_f64.cu) */
int qgt_dev_berry_closed(const double* part, int32_t nchunk, int32_t ncirc, int32_t G, double* maps, void* stream);
/* the device vector buffer of a plan and the amplitudes between its points */
const void* qgt_plan_dev_V(struct qgt_plan* p, int64_t* point_stride, int32_t* fp64);

/* ---- learned preconditioner and PCG (qgt_learned.cu) ---- */
/* X = [cos theta, sin theta] of theta rows idx[0..S) (idx NULL: rows 0..S) */
int qgt_dev_lr_features(const double* theta, const int32_t* idx, int32_t S, int32_t P, float* X, void* stream);
int qgt_dev_lr_linear(int32_t M, int32_t N, int32_t K, const float* X, const void* Wbf16, const float* b, float* Y,
                      int32_t act, float* Z, void* stream);
int qgt_dev_lr_linear_dx(int32_t M, int32_t N, int32_t K, const float* dY, const void* Wbf16, float* dX, void* stream);
int qgt_dev_lr_linear_dw(int32_t M, int32_t N, int32_t K, const float* dY, const float* X, float* dW, float* db,
                         void* stream);
int qgt_dev_lr_silu_back(const float* Z, float* dH, int64_t n, void* stream);
/* mean loss over S samples (metric rows idx[s]) added to *loss; dO = its gradient */
int qgt_dev_lr_loss(const float* O, const float* metric, const int32_t* idx, int32_t S, int32_t P, int32_t r,
                    float lambda, float u_scale, float* dO, float* loss, void* stream);
int qgt_dev_lr_outputs(const float* O, int32_t S, int32_t P, int32_t r, float lambda, float u_scale, double* d,
                       double* U, void* stream);
int qgt_dev_lr_adam(float* w, void* wbf16, const float* g, float* m1, float* m2, int64_t n, float lr, float b1,
                    float b2, float eps, int32_t step, float wd, void* stream);
int qgt_dev_lr_to_bf16(const float* w, void* wbf16, int64_t n, void* stream);
int qgt_dev_metric_f32(const double* Q, int64_t count, float* out, void* stream);
/* nsys PCG solves of (Re Q + lambda I) x = b, systems sys_stride doubles apart */
int qgt_dev_pcg(const double* Q, int32_t complex_input, int64_t sys_stride, const double* b, int32_t P, double lambda,
                const double* d, const double* U, int32_t r, double tol, int32_t max_iter, double* x, int32_t* iters,
                double* resid, int32_t nsys, void* stream);
int qgt_dev_axpy_update(double* theta, const double* x, double eta, int32_t n, void* stream);

/* ---- dense complex linear algebra of the reference entry points (qgt_linalg.cu; host buffers in
 * and out, P <= 8192) ---- */
/* singular values of the P x P complex64 matrix G (row-major {re, im} floats) by one-sided Jacobi in
 * FP64 (sigma: P doubles, NULL allowed); with g (P complex64) also the pseudo-inverse solution
 * x = V S^+ U^H g, S^+ dropping sigma <= cutoff (x: 2P doubles) */
int qgt_dev_svd_pinv(const float* G, int32_t P, double* sigma, const float* g, double cutoff, double* x,
                     int32_t max_sweeps, int32_t* sweeps);
/* (G + lambda I) x = g by LU with partial pivoting in FP64 (x: 2P doubles); *singular = 1 when a pivot
 * has |a|^2 < 1e-10 (the last pivot: when it is zero) */
int qgt_dev_lu_solve(const float* G, int32_t P, double lambda, const float* g, double* x, int32_t* singular);
/* F x = g by the reference's conjugate gradients (FP64, F real P x P) */
int qgt_dev_ref_cg(const double* F, const double* g, int32_t P, double* x);
/* out (dim x dim complex64) = delta_ij - conj(psi_i) psi_j */
int qgt_dev_fs_metric(const float* psi, int64_t dim, float* out);

/* more plan accessors (device buffers of a plan) */
double* qgt_plan_dev_grad(struct qgt_plan* p);
double* qgt_plan_dev_energy(struct qgt_plan* p);
double* qgt_plan_dev_natgrad(struct qgt_plan* p);

#ifdef __cplusplus
}
#endif
#endif
