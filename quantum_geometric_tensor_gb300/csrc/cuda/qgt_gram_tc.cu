// qgt_gram_tc.cu -- the Gram contraction HG_ij = <V_i|V_j> on tcgen05 tensor
// cores (sm_103a), fed by TMA, accumulating in TMEM.
//
// Operands: 4 half-precision planes (Re hi, Re lo, Im hi, Im lo) of the rows
// (psi, H psi, derivative slots), each row K-major (amplitude index
// contiguous) and prescaled by a power of two.  With x = hi + lo per real
// component, the complex Gram of a 128 x 128 tile pair (row block m, row
// block n) is accumulated as twelve real MMAs per k-step:
//   Re += Rh Rh' + Rh Rl' + Rl Rh' + Ih Ih' + Ih Il' + Il Ih'
//   Im += Rh Ih' + Rh Il' + Rl Ih' - Ih Rh' - Ih Rl' - Il Rh'
// (X Y' = X_m Y_n^T; the minus sign is the instruction's negate-A bit; the
// lo*lo products are dropped, which leaves ~2^-22 relative error for FP16
// operands).  FP32 accumulators live in TMEM (256 columns: Re, Im).
//
// Warp roles per CTA (192 threads): warp 0 = TMA producer (one thread),
// warp 1 = TMEM allocator + MMA issuer (one thread), warps 2..5 = epilogue
// (TMEM -> registers -> global partials).  A 3-stage mbarrier ring of
// 64 KiB stages (8 tiles of 128 rows x 32 amplitudes, SWIZZLE_64B).
//
// Grid = (tile pairs mb <= nb) x (K splits).  Each CTA writes its FP32
// partial block to the scratch buffer; a reduction kernel sums the splits in
// FP64 in a fixed order and rescales.
//
// Every mbarrier wait is bounded (globaltimer deadline); on expiry the CTA
// records an error code in *err, stops issuing, waits (bounded) for its own
// MMAs, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../qgt_internal.h"

#define TC_STAGES 3
#define TC_BK 32                                   // amplitudes per stage
#define TC_TILE_BYTES (128 * TC_BK * 2)            // 8 KiB
#define TC_STAGE_BYTES (8 * TC_TILE_BYTES)         // 64 KiB
#define TC_SMEM_BYTES (TC_STAGES * TC_STAGE_BYTES + 1024)
#define TC_TIMEOUT_NS 4000000000ull
#define TC_ERR_TIMEOUT (-13)

struct qgt_tc_gram {
    CUtensorMap tmap;
    void* split;
    int64_t N;       // padded row length (multiple of 32)
    int rows, rows_pad, bf16;
    int nbk, ntp, nsplit;
    int64_t kchunk;
    float* part;
    int* err;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint64_t deadline)
{
    for (uint32_t it = 0;; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255u) == 255u && globaltimer() > deadline) return false;
    }
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}

// UMMA shared-memory descriptor: K-major, SWIZZLE_64B, 8-row groups 512 B apart.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
    d |= (uint64_t)1 << 16;                    // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(512 >> 4) << 32;           // stride byte offset
    d |= (uint64_t)1 << 46;                    // descriptor version (sm_100 family)
    d |= (uint64_t)4 << 61;                    // SWIZZLE_64B
    return d;
}

// instruction descriptor, kind::f16: D = F32, A/B = F16 (0) or BF16 (1), K-major, M = N = 128
__device__ __forceinline__ uint32_t idesc(int bf16, int negA)
{
    uint32_t f = bf16 ? 1u : 0u;
    return (1u << 4) | (f << 7) | (f << 10) | ((uint32_t)negA << 13) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v)
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tile_pair(int tp, int nb, int* mb, int* nbo)
{
    int i = 0, rem = tp;
    while (rem >= nb - i) { rem -= nb - i; i++; }
    *mb = i;
    *nbo = i + rem;
}

// 12 terms: (A plane, B plane, Im accumulator, negate A)
__constant__ int8_t c_terms[12][4] = {
    {0, 0, 0, 0}, {0, 1, 0, 0}, {1, 0, 0, 0}, {2, 2, 0, 0}, {2, 3, 0, 0}, {3, 2, 0, 0},
    {0, 2, 1, 0}, {0, 3, 1, 0}, {1, 2, 1, 0}, {2, 0, 1, 1}, {2, 1, 1, 1}, {3, 0, 1, 1}};

__global__ void __launch_bounds__(192, 1)
    tc_gram_kernel(const __grid_constant__ CUtensorMap tmap, int nbk, int64_t N, int64_t kchunk, int bf16,
                   float* __restrict__ part, int* __restrict__ err)
{
    extern __shared__ uint8_t smem_dyn[];
    __shared__ __align__(8) uint64_t full_bar[TC_STAGES];
    __shared__ __align__(8) uint64_t empty_bar[TC_STAGES];
    __shared__ __align__(8) uint64_t done_bar;
    __shared__ uint32_t tmem_base_sh;
    __shared__ volatile int abort_flag;

    uint8_t* sbase = (uint8_t*)(((uintptr_t)smem_dyn + 1023) & ~(uintptr_t)1023);
    const uint32_t s0 = smem_u32(sbase);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int mb, nbo;
    tile_pair(blockIdx.x, nbk, &mb, &nbo);
    const bool diag = (mb == nbo);
    const int64_t k0 = (int64_t)blockIdx.y * kchunk;
    int64_t k1 = k0 + kchunk;
    if (k1 > N) k1 = N;
    const int nk = (int)((k1 - k0) / TC_BK);
    const uint64_t deadline = globaltimer() + TC_TIMEOUT_NS;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; s++) {
            mbar_init(smem_u32(&full_bar[s]), 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);
        }
        mbar_init(smem_u32(&done_bar), 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(&tmem_base_sh)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_sh;
    bool mma_issued_all = false;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer ----------------
        const uint32_t bytes = (diag ? 4u : 8u) * TC_TILE_BYTES;
        int issued = 0;
        for (int kt = 0; kt < nk; kt++) {
            const int s = kt % TC_STAGES;
            if (kt >= TC_STAGES) {
                if (!mbar_wait(smem_u32(&empty_bar[s]), ((kt / TC_STAGES) & 1) ^ 1, deadline)) {
                    atomicExch(err, TC_ERR_TIMEOUT);
                    abort_flag = 1;
                    break;
                }
            }
            if (abort_flag) break;
            const uint32_t st = s0 + s * TC_STAGE_BYTES;
            const uint32_t fb = smem_u32(&full_bar[s]);
            mbar_expect_tx(fb, bytes);
            const int kc = (int)(k0 + (int64_t)kt * TC_BK);
            for (int p = 0; p < 4; p++) {
                tma_load_3d(st + p * TC_TILE_BYTES, &tmap, kc, mb * 128, p, fb);
                if (!diag) tma_load_3d(st + (4 + p) * TC_TILE_BYTES, &tmap, kc, nbo * 128, p, fb);
            }
            issued = kt + 1;
        }
        // drain: the last issued load of every stage has landed before the CTA can exit
        for (int u = issued - TC_STAGES; u < issued; u++) {
            if (u < 0) continue;
            (void)mbar_wait(smem_u32(&full_bar[u % TC_STAGES]), (u / TC_STAGES) & 1, deadline + TC_TIMEOUT_NS);
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer ----------------
        const uint32_t id_pos = idesc(bf16, 0), id_neg = idesc(bf16, 1);
        int kt = 0;
        for (; kt < nk; kt++) {
            const int s = kt % TC_STAGES;
            if (!mbar_wait(smem_u32(&full_bar[s]), (kt / TC_STAGES) & 1, deadline)) {
                atomicExch(err, TC_ERR_TIMEOUT);
                abort_flag = 1;
                break;
            }
            if (abort_flag) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = s0 + s * TC_STAGE_BYTES;
            const uint32_t sb = diag ? sa : sa + 4 * TC_TILE_BYTES;
#pragma unroll
            for (int ks = 0; ks < TC_BK / 16; ks++) {
#pragma unroll
                for (int t = 0; t < 12; t++) {
                    const int pa = c_terms[t][0], pb = c_terms[t][1], im = c_terms[t][2], ng = c_terms[t][3];
                    const uint64_t da = sdesc(sa + pa * TC_TILE_BYTES + ks * 32);
                    const uint64_t db = sdesc(sb + pb * TC_TILE_BYTES + ks * 32);
                    const uint32_t acc = (kt > 0 || ks > 0 || (t != 0 && t != 6)) ? 1u : 0u;
                    mma_f16(tmem + (im ? 128u : 0u), da, db, ng ? id_neg : id_pos, acc);
                }
            }
            mma_commit(smem_u32(&empty_bar[s]));
        }
        // commit even after an abort: done_bar then tracks every MMA this thread issued
        mma_commit(smem_u32(&done_bar));
        mma_issued_all = true;
    } else if (warp >= 2) {
        // ---------------- epilogue ----------------
        const bool ok = mbar_wait(smem_u32(&done_bar), 0, deadline);
        if (!ok) {
            atomicExch(err, TC_ERR_TIMEOUT);
            abort_flag = 1;
        } else if (!abort_flag && nk > 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int quad = warp & 3;
            const int row = quad * 32 + lane;
            float* out = part + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * (2 * 128 * 128);
            float v[32];
            for (int c = 0; c < 4; c++) {
                tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + c * 32, v);
                float4* o = reinterpret_cast<float4*>(out + row * 128 + c * 32);
#pragma unroll
                for (int j = 0; j < 8; j++) o[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + 128 + c * 32, v);
                float4* oi = reinterpret_cast<float4*>(out + 128 * 128 + row * 128 + c * 32);
#pragma unroll
                for (int j = 0; j < 8; j++) oi[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            }
        } else if (nk == 0) {
            float* out = part + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * (2 * 128 * 128);
            const int row = (warp & 3) * 32 + lane;
            for (int c = 0; c < 128; c++) { out[row * 128 + c] = 0.f; out[128 * 128 + row * 128 + c] = 0.f; }
        }
    }
    // the MMA issuer makes sure its MMAs have drained before TMEM is freed
    if (warp == 1 && lane == 0 && mma_issued_all) (void)mbar_wait(smem_u32(&done_bar), 0, deadline + TC_TIMEOUT_NS);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
    }
}

__global__ void tc_reduce_kernel(const float* __restrict__ part, int rows, int nbk, int ntp, int nsplit, double scale,
                                 double2* __restrict__ HG)
{
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= (int64_t)rows * rows) return;
    int i = (int)(idx / rows), j = (int)(idx % rows);
    if (i > j) return;
    int ti = i >> 7, tj = j >> 7;
    int tp = ti * nbk - ti * (ti - 1) / 2 + (tj - ti);
    int64_t off = (int64_t)(i & 127) * 128 + (j & 127);
    double re = 0, im = 0;
    for (int s = 0; s < nsplit; s++) {
        const float* b = part + ((int64_t)s * ntp + tp) * (2 * 128 * 128);
        re += (double)b[off];
        im += (double)b[128 * 128 + off];
    }
    HG[(int64_t)i * rows + j] = make_double2(re * scale, im * scale);
    HG[(int64_t)j * rows + i] = make_double2(re * scale, -im * scale);
}

static PFN_cuTensorMapEncodeTiled_v12000 get_encode(void)
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = NULL;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = NULL;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

extern "C" int qgt_dev_tc_gram_create(void* split, int64_t N, int32_t rows, int32_t rows_pad, int32_t bf16,
                                      qgt_tc_gram_t** out)
{
    *out = NULL;
    if (N % TC_BK || rows_pad % 128 || rows > rows_pad || ((uintptr_t)split & 15))
        return qgt_set_error(-1, "tc gram: N (%lld) must be a multiple of 32, rows_pad of 128", (long long)N);
    if (N > 0x7fffffffLL) return qgt_set_error(-1, "tc gram: row length too large for TMA coordinates");
    PFN_cuTensorMapEncodeTiled_v12000 enc = get_encode();
    if (!enc) return qgt_set_error(-6, "tc gram: cuTensorMapEncodeTiled unavailable");
    qgt_tc_gram_t* g = (qgt_tc_gram_t*)calloc(1, sizeof(qgt_tc_gram_t));
    if (!g) return qgt_set_error(-2, "tc gram: out of host memory");
    g->split = split;
    g->N = N;
    g->rows = rows;
    g->rows_pad = rows_pad;
    g->bf16 = bf16;
    g->nbk = rows_pad / 128;
    g->ntp = g->nbk * (g->nbk + 1) / 2;
    int nsplit = (int)((2 * 152 + g->ntp - 1) / g->ntp) / 2;
    if (nsplit < 1) nsplit = 1;
    int64_t maxsplit = N / (TC_BK * TC_STAGES);
    if (maxsplit < 1) maxsplit = 1;
    if (nsplit > maxsplit) nsplit = (int)maxsplit;
    int64_t kchunk = (N + nsplit - 1) / nsplit;
    kchunk = (kchunk + TC_BK - 1) / TC_BK * TC_BK;
    g->kchunk = kchunk;
    g->nsplit = (int)((N + kchunk - 1) / kchunk);

    cuuint64_t dims[3] = {(cuuint64_t)N, (cuuint64_t)rows_pad, 4};
    cuuint64_t strides[2] = {(cuuint64_t)N * 2, (cuuint64_t)N * 2 * rows_pad};
    cuuint32_t box[3] = {TC_BK, 128, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(&g->tmap, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, split, dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        free(g);
        return qgt_set_error(-6, "tc gram: cuTensorMapEncodeTiled failed (%d)", (int)r);
    }
    size_t pbytes = (size_t)g->nsplit * g->ntp * 2 * 128 * 128 * sizeof(float);
    cudaError_t e = cudaMalloc((void**)&g->part, pbytes);
    if (e == cudaSuccess) e = cudaMalloc((void**)&g->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(g->err, 0, sizeof(int));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(tc_gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_BYTES);
    if (e != cudaSuccess) {
        cudaFree(g->part);
        cudaFree(g->err);
        free(g);
        return qgt_set_error(e == cudaErrorMemoryAllocation ? -2 : -6, "tc gram: %s", cudaGetErrorString(e));
    }
    *out = g;
    return 0;
}

extern "C" int qgt_dev_tc_gram_run(qgt_tc_gram_t* g, double inv_scale2, double* HG, void* stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    // the error word describes this run only (a run after a failed one starts clean)
    cudaError_t e = cudaMemsetAsync(g->err, 0, sizeof(int), s);
    if (e != cudaSuccess) return qgt_set_error(-6, "tc gram: %s", cudaGetErrorString(e));
    tc_gram_kernel<<<dim3(g->ntp, g->nsplit), 192, TC_SMEM_BYTES, s>>>(g->tmap, g->nbk, g->N, g->kchunk, g->bf16,
                                                                       g->part, g->err);
    int rc = qgt_dev_last_error();
    if (rc) return rc;
    int64_t cnt = (int64_t)g->rows * g->rows;
    tc_reduce_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(g->part, g->rows, g->nbk, g->ntp, g->nsplit,
                                                                   inv_scale2, (double2*)HG);
    return qgt_dev_last_error();
}

extern "C" const int* qgt_dev_tc_gram_err(const qgt_tc_gram_t* g) { return g ? g->err : NULL; }

extern "C" int qgt_dev_tc_gram_status(qgt_tc_gram_t* g, void* stream)
{
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, g->err, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return qgt_set_error(-6, "tc gram status: %s", cudaGetErrorString(e));
    return h;
}

extern "C" void qgt_dev_tc_gram_destroy(qgt_tc_gram_t* g)
{
    if (!g) return;
    cudaFree(g->part);
    cudaFree(g->err);
    free(g);
}

extern "C" int64_t qgt_dev_tc_gram_scratch_bytes(const qgt_tc_gram_t* g)
{
    return g ? (int64_t)g->nsplit * g->ntp * 2 * 128 * 128 * (int64_t)sizeof(float) : 0;
}
