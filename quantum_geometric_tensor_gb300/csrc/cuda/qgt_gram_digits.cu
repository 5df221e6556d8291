// qgt_gram_digits.cu -- the mixed-precision Gram HG_ij = <V_i|V_j> on tcgen05
// tensor cores with exactly accumulated high digits.
//
// Why: the tensor cores' FP32 accumulation truncates, which over long K
// chains biases every large sum (the diagonal by ~-3e-8 per MMA), so a plain
// hi/lo split cannot reach 1e-6 relative on 2^20 amplitudes.  Here every
// complex64 amplitude of row r is written, in units of a per-row power of two
// u_r (max_k |x_rk| < M u_r, M = 2^mbits), as
//     x = u_r (D + l),  D = rint(x / u_r) in [-M, M],  |l| <= 1/2,
// with D exact in FP16 and l = l1 + l2 carried by two FP16 values (a single
// FP16 residual leaves ~1e-6 relative error in Q on real derivative states,
// where the representation errors of rows with equal magnitudes coincide).  The D*D' products are
// integers and every partial sum of them over a CTA's K range is at most
// 2^23 (Cauchy-Schwarz; M is chosen per plan from the K range, M = 64 for
// 1024 amplitudes, up to 1024 for short ranges), so their FP32 tensor
// accumulation is EXACT.  K ranges stay at <= 1024 amplitudes: the residual
// accumulator's truncating FP32 chain over 4096 amplitudes left 9.7e-7 of
// relative metric error at 20 qubits, over 1024 it leaves 1.2e-7.  The D*l1', l1*D', l1*l1', D*l2', l2*D' terms (a few
// percent of the total) accumulate in a second TMEM accumulator; their
// rounding is ~1e-8 relative to the sum.
//
// Data path per CTA (tile pair mb <= nb, K range of <= 1024 amplitudes):
//   TMA: 128 rows x 16 amplitudes of complex64 per row block -> raw smem (128-byte swizzle)
//   8 converter warps: raw -> FP16 planes in the SWIZZLE_32B K-major UMMA
//                      layout: the A block as 6 planes {Re D, Im D, Re l1,
//                      Im l1, Re l2, Im l2}, the B block as 9 planes
//                      {Re D, Im D, -Re D, Re l1, Im l1, -Re l1, Re l2, Im l2,
//                      -Re l2}, so that every (Re, Im) pair of B operands that
//                      one A plane meets is two adjacent planes; B planes
//                      hold the block's valid rows rounded up to 16 (rbB)
//   1 thread: 12 tcgen05.mma (M = 128, N = 2 rbB <= 256 = [Re partner |
//             Im partner], K = 16) per k-step into TMEM [D*D Re | D*D Im |
//             rest Re | rest Im] (two regions of 256 columns)
//   epilogue (the converter warps): TMEM -> FP32 (hh + rest) -> partials
// The raw ring (3 stages) and the plane ring (2 stages) are decoupled, so a
// raw buffer is refilled as soon as it has been converted; the converters load
// a k-step's raw values into registers before they wait for a free plane stage.
// A second kernel sums the partials in FP64 and applies u_i u_j.
//
// Every mbarrier wait is bounded (globaltimer); on expiry the CTA records an
// error in *err, stops, drains its own TMA loads and MMAs, frees TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include "../qgt_internal.h"

#define DG_BK 16                                    // amplitudes per k-step (one MMA K)
#define DG_RAW_BYTES (128 * DG_BK * 8)              // 16 KiB: 128 rows x 16 complex64
#define DG_PLANE_BYTES (128 * DG_BK * 2)            // 4 KiB: 128 rows x 16 fp16
#define DG_RAW_STAGES 3                             // raw ring: 3 x 2 blocks x 16 KiB
#define DG_PL_STAGES 2                              // plane ring: 2 x 2 blocks x 6 planes x 4 KiB
#define DG_CONV_WARPS 8
#define DG_THREADS (64 + 32 * DG_CONV_WARPS)
#define DG_PL_A 6                                   // planes of the A block
#define DG_PL_B 9                                   // planes of the B block (with the negated real ones)
#define DG_PL_STAGE ((DG_PL_A + DG_PL_B) * DG_PLANE_BYTES)
#define DG_SMEM_BYTES (DG_RAW_STAGES * 2 * DG_RAW_BYTES + DG_PL_STAGES * DG_PL_STAGE + 1024)
#define DG_KMAX 1024                                // amplitudes per CTA (exactness bound; shorter FP32 chains)
#define DG_TIMEOUT_NS 4000000000ull
#define DG_ERR_TIMEOUT (-13)
#define DG_ERR_INEXACT (-24)

// device control block of a Gram: the status word the kernel writes (cleared on the stream before
// every run) and the wait settings it reads at start.  `stall` and `timeout_ns` exist for the tests of
// the bounded-wait error path: with stall set, the converter warps wait on an mbarrier that nothing
// arrives on, so their wait runs out after timeout_ns (0 = DG_TIMEOUT_NS) and the CTA takes its
// abort path (drain its own loads and MMAs, free TMEM, report DG_ERR_TIMEOUT).
struct dg_ctl_t {
    int err;
    int stall;
    long long timeout_ns;
};

struct qgt_dg_gram {
    CUtensorMap tmap;
    const void* V;
    int64_t N;
    int rows, nbk, ntp, nsplit, npoints;
    int64_t kchunk;
    int mbits;                 /* digits D in [-2^mbits, 2^mbits] */
    const uint32_t* rowmax;
    float* part;
    dg_ctl_t* ctl;
};

static __device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

static __device__ __forceinline__ uint64_t gtimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

static __device__ __forceinline__ void bar_init(uint32_t b, uint32_t c)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(b), "r"(c) : "memory");
}

static __device__ __forceinline__ void bar_expect_tx(uint32_t b, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
}

static __device__ __forceinline__ void bar_arrive(uint32_t b)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(b) : "memory");
}

static __device__ __forceinline__ bool bar_wait(uint32_t b, uint32_t parity, uint64_t deadline)
{
    for (uint32_t it = 0;; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(b), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255u) == 255u && gtimer() > deadline) return false;
    }
}

// 3D box {32 floats, 128 rows, 1 point}: coordinates (float index, row, point)
static __device__ __forceinline__ void tma_3d(uint32_t dst, const CUtensorMap* m, int c0, int c1, int c2, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"((uint64_t)m), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}

// two half2 (four consecutive k of one row) as one 8-byte shared store
static __device__ __forceinline__ void st_h4(uint8_t* p, __half2 a, __half2 b)
{
    uint2 u;
    u.x = *reinterpret_cast<const uint32_t*>(&a);
    u.y = *reinterpret_cast<const uint32_t*>(&b);
    *reinterpret_cast<uint2*>(p) = u;
}

// K-major SWIZZLE_32B operand: rows of 32 B (16 fp16), 8-row groups 256 B apart
static __device__ __forceinline__ uint64_t desc_sw32(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(256 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)6 << 61;  // SWIZZLE_32B
    return d;
}

// kind::f16, D = F32, A = B = F16, K-major, M = 128, N = n (a multiple of 16, 16 .. 256)
static __device__ __forceinline__ uint32_t idesc_f16(uint32_t n)
{
    return (1u << 4) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

static __device__ __forceinline__ void umma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}

static __device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

static __device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v)
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

static __device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

static __device__ __forceinline__ void pair_of(int tp, int nb, int* mb, int* nbo)
{
    int i = 0, rem = tp;
    while (rem >= nb - i) { rem -= nb - i; i++; }
    *mb = i;
    *nbo = i + rem;
}

// unit exponent: rowmax < 2^e, u = 2^(e - mbits), so |x| < 2^mbits u
static __device__ __forceinline__ int unit_exp(uint32_t bits, int mbits)
{
    float m = __uint_as_float(bits);
    if (!(m > 0.f)) return 0;
    int e;
    frexpf(m, &e);  // m = f 2^e, f in [0.5, 1)
    return e - mbits;
}

// 12 terms per k-step: (A plane as (level, part), first B plane of the pair, accumulator region).
// A planes: level 0 D, 1 l1, 2 l2; part 0 Re, 1 Im (A layout index 2 level + part; a diagonal
// pair reads its A planes from the B layout, index 3 level + part).  B pairs [Re partner | Im
// partner]: 0 [Re D | Im D], 1 [Im D | -Re D], 3 [Re l1 | Im l1], 4 [Im l1 | -Re l1],
// 6 [Re l2 | Im l2], 7 [Im l2 | -Re l2].  Region 0 = exact D*D (Re, Im), 1 = the residual terms.
//   Re <x|y> = xr yr + xi yi,  Im <x|y> = xr yi - xi yr  (x from A, y from B)
__constant__ int8_t dg_terms[12][4] = {
    {0, 0, 0, 0}, {0, 1, 1, 0},                                  // D  x D
    {0, 0, 3, 1}, {0, 0, 6, 1}, {1, 0, 0, 1}, {1, 0, 3, 1}, {2, 0, 0, 1},   // Re parts of A
    {0, 1, 4, 1}, {0, 1, 7, 1}, {1, 1, 1, 1}, {1, 1, 4, 1}, {2, 1, 1, 1}};  // Im parts of A

__global__ void __launch_bounds__(DG_THREADS, 1)
    dg_gram_kernel(const __grid_constant__ CUtensorMap tmap, int nbk, int64_t N, int64_t kchunk,
                   const uint32_t* __restrict__ rowmax, int rows, int mbits, float* __restrict__ part,
                   dg_ctl_t* __restrict__ ctl)
{
    int* err = &ctl->err;
    extern __shared__ uint8_t dg_smem[];
    __shared__ __align__(8) uint64_t raw_full[DG_RAW_STAGES];
    __shared__ __align__(8) uint64_t raw_empty[DG_RAW_STAGES];
    __shared__ __align__(8) uint64_t pl_full[DG_PL_STAGES];
    __shared__ __align__(8) uint64_t pl_empty[DG_PL_STAGES];
    __shared__ __align__(8) uint64_t done_bar;
    __shared__ __align__(8) uint64_t never_bar;   // test stall: initialised, never arrived on
    __shared__ uint32_t tmem_sh;
    __shared__ volatile int abort_sh;
    __shared__ float inv_u[2][128];

    uint8_t* sb = (uint8_t*)(((uintptr_t)dg_smem + 1023) & ~(uintptr_t)1023);
    uint8_t* raw_base = sb;                                        // DG_RAW_STAGES x 2 blocks x 16 KiB
    uint8_t* pl_base = sb + DG_RAW_STAGES * 2 * DG_RAW_BYTES;       // DG_PL_STAGES x 2 blocks x 6 planes x 4 KiB
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int mb, nbo;
    const int ntp = nbk * (nbk + 1) / 2;   // blockIdx.x = K range x ntp + tile pair
    pair_of((int)(blockIdx.x % ntp), nbk, &mb, &nbo);
    const bool diag = (mb == nbo);
    const int nblk = diag ? 1 : 2;
    // the B block's planes hold its valid rows rounded up to 16 (the last block of a plan is
    // partly padding): plane stride pbB, MMA N = 2 rbB ([Re partner | Im partner])
    const int vb = rows - 128 * nbo < 128 ? rows - 128 * nbo : 128;
    const int rbB = (vb + 15) & ~15;
    const uint32_t pbB = (uint32_t)rbB * DG_BK * 2;
    const int64_t k0 = (int64_t)(blockIdx.x / ntp) * kchunk;
    int64_t k1 = k0 + kchunk;
    if (k1 > N) k1 = N;
    const int nk = (int)((k1 - k0) / DG_BK);
    const long long tmo = ctl->timeout_ns;
    const bool stall = ctl->stall != 0;
    const uint64_t deadline = gtimer() + (tmo > 0 ? (uint64_t)tmo : DG_TIMEOUT_NS);
    rowmax += (int64_t)blockIdx.z * rows;   // parameter point
    part += (int64_t)blockIdx.z * gridDim.x * (2 * 128 * 128);

    if (threadIdx.x < 128) {
        for (int b = 0; b < 2; b++) {
            int r = (b == 0 ? mb : nbo) * 128 + threadIdx.x;
            float iu = 0.f;
            if (r < rows) iu = ldexpf(1.0f, -unit_exp(rowmax[r], mbits));
            inv_u[b][threadIdx.x] = iu;
        }
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < DG_RAW_STAGES; s++) {
            bar_init(smem_u32(&raw_full[s]), 1);
            bar_init(smem_u32(&raw_empty[s]), DG_CONV_WARPS);
        }
        for (int s = 0; s < DG_PL_STAGES; s++) {
            bar_init(smem_u32(&pl_full[s]), DG_CONV_WARPS);
            bar_init(smem_u32(&pl_empty[s]), 1);
        }
        bar_init(smem_u32(&done_bar), 1);
        bar_init(smem_u32(&never_bar), 1);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_sh)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_sh;
    bool mma_done_commit = false;

    if (warp == 0 && lane == 0) {
        // ---------- TMA producer: complex64 rows ----------
        const uint32_t bytes = (uint32_t)nblk * DG_RAW_BYTES;
        int issued = 0;
        for (int kt = 0; kt < nk; kt++) {
            const int s = kt % DG_RAW_STAGES;
            if (kt >= DG_RAW_STAGES &&
                !bar_wait(smem_u32(&raw_empty[s]), ((kt / DG_RAW_STAGES) & 1) ^ 1, deadline)) {
                atomicExch(err, DG_ERR_TIMEOUT);
                abort_sh = 1;
                break;
            }
            if (abort_sh) break;
            const uint32_t st = smem_u32(raw_base + s * 2 * DG_RAW_BYTES);
            const uint32_t fb = smem_u32(&raw_full[s]);
            bar_expect_tx(fb, bytes);
            const int x = (int)(2 * (k0 + (int64_t)kt * DG_BK));  // float index
            tma_3d(st, &tmap, x, mb * 128, (int)blockIdx.z, fb);
            if (!diag) tma_3d(st + DG_RAW_BYTES, &tmap, x, nbo * 128, (int)blockIdx.z, fb);
            issued = kt + 1;
        }
        for (int u = issued - DG_RAW_STAGES; u < issued; u++)
            if (u >= 0)
                (void)bar_wait(smem_u32(&raw_full[u % DG_RAW_STAGES]), (u / DG_RAW_STAGES) & 1, deadline + DG_TIMEOUT_NS);
    } else if (warp == 1 && lane == 0) {
        // ---------- MMA issuer ----------
        const uint32_t id = idesc_f16(2u * (uint32_t)rbB);
        for (int kt = 0; kt < nk; kt++) {
            const int s = kt % DG_PL_STAGES;
            if (!bar_wait(smem_u32(&pl_full[s]), (kt / DG_PL_STAGES) & 1, deadline)) {
                atomicExch(err, DG_ERR_TIMEOUT);
                abort_sh = 1;
                break;
            }
            if (abort_sh) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // stage: A planes at 0 (6 x 4 KiB), B planes at 6 planes (9 x 4 KiB); a diagonal pair
            // keeps only the B layout and reads its A planes from it
            const uint32_t st = smem_u32(pl_base + s * DG_PL_STAGE);
            const uint32_t pb = st + (diag ? 0 : DG_PL_A * DG_PLANE_BYTES);
#pragma unroll
            for (int t = 0; t < 12; t++) {
                const int lv = dg_terms[t][0], pt = dg_terms[t][1], b = dg_terms[t][2], rg = dg_terms[t][3];
                // a diagonal pair's A rows past rbB read other planes: those output rows are padding
                const uint32_t pa = diag ? pb + (3 * lv + pt) * pbB : st + (2 * lv + pt) * DG_PLANE_BYTES;
                const uint32_t first = (kt == 0) && (t == 0 || t == 2);
                umma(tmem + (uint32_t)rg * 256u, desc_sw32(pa), desc_sw32(pb + b * pbB), id, first ? 0u : 1u);
            }
            umma_commit(smem_u32(&pl_empty[s]));
        }
        umma_commit(smem_u32(&done_bar));
        mma_done_commit = true;
    } else if (warp >= 2) {
        // ---------- converters: complex64 -> {Re D, Re l1, Re l2, Im D, Im l1, Im l2} ----------
        const int cw = warp - 2;
        // lane -> (row r = 8 cw + 64 i + lane / 4, amplitudes kq .. kq + 3): two 16-byte loads of
        // (re, im, re, im), then one 8-byte store of two half2 pairs into each plane
        const int sub = lane >> 2, kq = (lane & 3) * 4;
        for (int kt = 0; kt < nk; kt++) {
            const int rs = kt % DG_RAW_STAGES, ps = kt % DG_PL_STAGES;
            bool ok = bar_wait(stall ? smem_u32(&never_bar) : smem_u32(&raw_full[rs]), (kt / DG_RAW_STAGES) & 1,
                               deadline);
            const uint8_t* rawst = raw_base + rs * 2 * DG_RAW_BYTES;
            uint8_t* plst = pl_base + ps * DG_PL_STAGE;
            constexpr int NIT = 128 / (8 * DG_CONV_WARPS);
            // all of the k-step's raw values first (independent shared loads, issued while the plane
            // stage may still be in use by the MMAs), then the digit planes
            float4 q[2][NIT][2];
            float iuv[2][NIT];
            if (ok) {
#pragma unroll
                for (int b = 0; b < 2; b++) {
                    const float* raw = reinterpret_cast<const float*>(rawst + b * DG_RAW_BYTES);
                    const int rlim = (diag || b == 1) ? rbB : 128;
#pragma unroll
                    for (int it = 0; it < NIT; it++) {
                        // rlim is a multiple of 16, so a group of 8 rows is all below it or all above
                        const int rr = 8 * cw + 8 * DG_CONV_WARPS * it, r = rr + sub;
                        if (b < nblk && rr < rlim) {
                            // the raw rows arrive 128-byte swizzled (16-byte chunk c of row r at
                            // c ^ (r & 7)), so the two rows of a quarter-warp read different banks
                            const int sw = r & 7, c0 = kq >> 1;
                            q[b][it][0] = *reinterpret_cast<const float4*>(raw + r * 32 + 4 * (c0 ^ sw));
                            q[b][it][1] = *reinterpret_cast<const float4*>(raw + r * 32 + 4 * ((c0 + 1) ^ sw));
                            iuv[b][it] = inv_u[b][r];
                        } else {
                            q[b][it][0] = q[b][it][1] = make_float4(0.f, 0.f, 0.f, 0.f);
                            iuv[b][it] = 0.f;
                        }
                    }
                }
            }
            if (ok && kt >= DG_PL_STAGES) ok = bar_wait(smem_u32(&pl_empty[ps]), ((kt / DG_PL_STAGES) & 1) ^ 1, deadline);
            if (!ok) {
                atomicExch(err, DG_ERR_TIMEOUT);
                abort_sh = 1;
            }
            if (abort_sh) break;
#pragma unroll
            for (int b = 0; b < 2; b++) {
                if (b >= nblk) break;
                // the B layout (9 planes) for the B block and for a diagonal pair's only block
                const bool blay = diag || b == 1;
                uint8_t* planes = plst + (diag ? 0 : b * DG_PL_A * DG_PLANE_BYTES);
                const uint32_t ps_ = blay ? pbB : (uint32_t)DG_PLANE_BYTES;   // plane stride
                const int rlim = blay ? rbB : 128;
#pragma unroll
                for (int it = 0; it < NIT; it++) {
                    const int rr = 8 * cw + 8 * DG_CONV_WARPS * it;
                    if (rr >= rlim) break;   // warp-uniform (rr depends on the warp only)
                    const int r = rr + sub;
                    const float iu = iuv[b][it];
                    // SWIZZLE_32B: 16-byte chunk (k / 8) xor bit 2 of the row; kq .. kq + 3 share a chunk
                    const int off = r * 32 + ((((kq >> 3) ^ (r >> 2)) & 1) << 4) + (kq & 7) * 2;
#pragma unroll
                    for (int c = 0; c < 2; c++) {   // 0: real parts, 1: imaginary parts
                        __half2 hd[2], h1[2], h2[2];
#pragma unroll
                        for (int h = 0; h < 2; h++) {
                            const float4 qq = q[b][it][h];
                            const float x0 = (c ? qq.y : qq.x) * iu, x1 = (c ? qq.w : qq.z) * iu;
                            const float d0 = rintf(x0), d1 = rintf(x1);
                            const float l0 = x0 - d0, l1 = x1 - d1;
                            h1[h] = __floats2half2_rn(l0, l1);
                            const float2 f1 = __half22float2(h1[h]);
                            h2[h] = __floats2half2_rn(l0 - f1.x, l1 - f1.y);
                            hd[h] = __floats2half2_rn(d0, d1);
                        }
                        // level l plane: A layout 2 l + c, B layout 3 l + c (+ the negated real part at 3 l + 2)
                        const int ls = blay ? 3 : 2;
                        uint8_t* pD = planes + c * ps_ + off;
                        st_h4(pD, hd[0], hd[1]);
                        st_h4(pD + ls * ps_, h1[0], h1[1]);
                        st_h4(pD + 2 * ls * ps_, h2[0], h2[1]);
                        if (blay && c == 0) {
                            uint8_t* pN = planes + 2 * ps_ + off;
                            st_h4(pN, __hneg2(hd[0]), __hneg2(hd[1]));
                            st_h4(pN + 3 * ps_, __hneg2(h1[0]), __hneg2(h1[1]));
                            st_h4(pN + 6 * ps_, __hneg2(h2[0]), __hneg2(h2[1]));
                        }
                    }
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                bar_arrive(smem_u32(&raw_empty[rs]));
                bar_arrive(smem_u32(&pl_full[ps]));
            }
        }
        // ---------- epilogue: warps 2..9; lane quadrant = warp & 3, column half = (warp - 2) / 4 ----------
        const bool ok = nk > 0 && !abort_sh && bar_wait(smem_u32(&done_bar), 0, deadline);
        float* out = part + (int64_t)blockIdx.x * (2 * 128 * 128);
        const int quad = warp & 3, half = (warp - 2) >> 2;
        const int row = quad * 32 + lane;
        if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t lanebase = tmem + ((uint32_t)(quad * 32) << 16);
            if ((rbB & 31) == 0) {
                // 32-column chunks (full blocks and rows rounded to 32)
                float hh[32], rsd[32];
                for (int ri = 0; ri < 2; ri++) {
                    for (int c = 2 * half; c < 2 * half + 2; c++) {
                        if (c * 32 >= rbB) continue;   // columns past the B block's rows (never read)
                        tmem_ld32(lanebase + ri * rbB + c * 32, hh);
                        tmem_ld32(lanebase + 256 + ri * rbB + c * 32, rsd);
                        if (diag && ri == 0 && c == (row >> 5) && hh[row & 31] > 8388608.0f)
                            atomicExch(err, DG_ERR_INEXACT);
                        float4* o = reinterpret_cast<float4*>(out + ri * 128 * 128 + row * 128 + c * 32);
#pragma unroll
                        for (int j = 0; j < 8; j++)
                            o[j] = make_float4(hh[4 * j] + rsd[4 * j], hh[4 * j + 1] + rsd[4 * j + 1],
                                               hh[4 * j + 2] + rsd[4 * j + 2], hh[4 * j + 3] + rsd[4 * j + 3]);
                    }
                }
            } else {
                // 16-column chunks: the Im half starts at column rbB, a multiple of 16
                float hh[16], rsd[16];
                for (int ri = 0; ri < 2; ri++) {
                    for (int c = 4 * half; c < 4 * half + 4; c++) {
                        if (c * 16 >= rbB) continue;
                        tmem_ld16(lanebase + ri * rbB + c * 16, hh);
                        tmem_ld16(lanebase + 256 + ri * rbB + c * 16, rsd);
                        if (diag && ri == 0 && c == (row >> 4) && hh[row & 15] > 8388608.0f)
                            atomicExch(err, DG_ERR_INEXACT);
                        float4* o = reinterpret_cast<float4*>(out + ri * 128 * 128 + row * 128 + c * 16);
#pragma unroll
                        for (int j = 0; j < 4; j++)
                            o[j] = make_float4(hh[4 * j] + rsd[4 * j], hh[4 * j + 1] + rsd[4 * j + 1],
                                               hh[4 * j + 2] + rsd[4 * j + 2], hh[4 * j + 3] + rsd[4 * j + 3]);
                    }
                }
            }
        } else {
            atomicExch(err, DG_ERR_TIMEOUT);
            for (int c = 64 * half; c < 64 * half + 64; c++) {
                out[row * 128 + c] = 0.f;
                out[128 * 128 + row * 128 + c] = 0.f;
            }
        }
    }
    if (warp == 1 && lane == 0 && mma_done_commit) (void)bar_wait(smem_u32(&done_bar), 0, deadline + DG_TIMEOUT_NS);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
    }
}

// hi + lo += x with the exact rounding error of hi + x kept in lo (Knuth's TwoSum)
static __device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x)
{
    const float sum = __fadd_rn(hi, x);
    const float bp = __fsub_rn(sum, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(sum, bp)), __fsub_rn(x, bp));
    hi = sum;
    lo = __fadd_rn(lo, err);
}

// HG_ij for 32 consecutive j of row i (blockIdx.x = j chunk, blockIdx.y = i, blockIdx.z = point): warp w
// sums the K ranges s = w (mod 8) as FP32 double-float (TwoSum) pairs, four of them for independent
// loads; the 8 warps' pairs are added in FP64 in a fixed order (deterministic).  FP64 conversions and
// adds are scarce on this part, so only the final pairs go to FP64.
__global__ void __launch_bounds__(256) dg_reduce_kernel(const float* __restrict__ part, const uint32_t* __restrict__ rowmax,
                                                         int rows, int nbk, int ntp, int nsplit, int mbits,
                                                         double2* __restrict__ HG)
{
    __shared__ float red[4][8][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i = blockIdx.y, j = blockIdx.x * 32 + lane;
    if (blockIdx.x * 32 + 31 < i) return;   // the whole chunk is below the diagonal
    part += (int64_t)blockIdx.z * nsplit * ntp * (2 * 128 * 128);   // parameter point
    rowmax += (int64_t)blockIdx.z * rows;
    HG += (int64_t)blockIdx.z * rows * rows;
    const bool live = j < rows && j >= i;
    const int jj = live ? j : i;
    const int ti = i >> 7, tj = jj >> 7;
    const int tp = ti * nbk - ti * (ti - 1) / 2 + (tj - ti);
    const int64_t off = (int64_t)(i & 127) * 128 + (jj & 127);
    const int64_t sstride = (int64_t)ntp * (2 * 128 * 128);
    const float* b0 = part + (int64_t)tp * (2 * 128 * 128) + off;
    float rh[4] = {0, 0, 0, 0}, rl[4] = {0, 0, 0, 0}, ih[4] = {0, 0, 0, 0}, il[4] = {0, 0, 0, 0};
    int s = w;
    for (; s + 24 < nsplit; s += 32) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const float* b = b0 + (int64_t)(s + 8 * u) * sstride;
            two_sum_acc(rh[u], rl[u], __ldg(b));
            two_sum_acc(ih[u], il[u], __ldg(b + 128 * 128));
        }
    }
    for (; s < nsplit; s += 8) {
        const float* b = b0 + (int64_t)s * sstride;
        two_sum_acc(rh[0], rl[0], __ldg(b));
        two_sum_acc(ih[0], il[0], __ldg(b + 128 * 128));
    }
    // fold the four pairs (FP32 TwoSum), then hand the warp's pair to the block
#pragma unroll
    for (int u = 1; u < 4; u++) {
        two_sum_acc(rh[0], rl[0], rh[u]);
        rl[0] += rl[u];
        two_sum_acc(ih[0], il[0], ih[u]);
        il[0] += il[u];
    }
    red[0][w][lane] = rh[0];
    red[1][w][lane] = rl[0];
    red[2][w][lane] = ih[0];
    red[3][w][lane] = il[0];
    __syncthreads();
    if (w == 0 && live) {
        double re = 0, im = 0;
        for (int q = 0; q < 8; q++) {
            re += (double)red[0][q][lane] + (double)red[1][q][lane];
            im += (double)red[2][q][lane] + (double)red[3][q][lane];
        }
        const double uu = ldexp(1.0, unit_exp(rowmax[i], mbits) + unit_exp(rowmax[j], mbits));
        HG[(int64_t)i * rows + j] = make_double2(re * uu, im * uu);
        HG[(int64_t)j * rows + i] = make_double2(re * uu, -im * uu);
    }
}

static PFN_cuTensorMapEncodeTiled_v12000 dg_encode(void)
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

extern "C" int qgt_dev_dg_gram_create(const void* V, int64_t N, int32_t rows, const uint32_t* rowmax, int32_t npoints,
                                      int32_t point_rows, qgt_dg_gram_t** out)
{
    *out = NULL;
    if (N % DG_BK || rows < 1 || ((uintptr_t)V & 15))
        return qgt_set_error(-1, "digit gram: row length %lld must be a multiple of %d", (long long)N, DG_BK);
    if (npoints < 1 || npoints > 65535 || point_rows < rows || rows > 65535)
        return qgt_set_error(-1, "digit gram: %d points of %d rows (stride %d rows)", npoints, rows, point_rows);
    if (2 * N > 0x7fffffffLL) return qgt_set_error(-1, "digit gram: row length too large for TMA coordinates");
    PFN_cuTensorMapEncodeTiled_v12000 enc = dg_encode();
    if (!enc) return qgt_set_error(-6, "digit gram: cuTensorMapEncodeTiled unavailable");
    qgt_dg_gram_t* g = (qgt_dg_gram_t*)calloc(1, sizeof(qgt_dg_gram_t));
    if (!g) return qgt_set_error(-2, "digit gram: out of host memory");
    g->V = V;
    g->N = N;
    g->rows = rows;
    g->rowmax = rowmax;
    g->npoints = npoints;
    int rows_pad = (rows + 127) / 128 * 128;
    g->nbk = rows_pad / 128;
    g->ntp = g->nbk * (g->nbk + 1) / 2;
    /* K per CTA: at most DG_KMAX (exactness), and enough CTAs to fill the GPU */
    int64_t kc = DG_KMAX;
    int64_t want = (2 * 152 + g->ntp - 1) / g->ntp;
    while (kc > 4 * DG_BK && (N + kc - 1) / kc * npoints < want) kc /= 2;
    g->kchunk = kc;
    g->nsplit = (int)((N + kc - 1) / kc);
    if ((int64_t)g->ntp * g->nsplit > 0x7fffffffLL) {
        free(g);
        return qgt_set_error(-1, "digit gram: %d tile pairs x %d K ranges exceed the grid", g->ntp, g->nsplit);
    }
    /* widest digits whose products sum exactly over kc amplitudes:
     * kc (M^2 + sqrt(2) M + 1/2) <= 2^23 with M = 2^mbits, |D_re|^2 + |D_im|^2 bounded through |x| < M u;
     * M <= 1024 keeps D exact in FP16 */
    g->mbits = 10;
    while (g->mbits > 1) {
        double M = (double)(1 << g->mbits);
        if ((double)kc * (M * M + 1.4143 * M + 0.5) <= 8388608.0) break;
        g->mbits--;
    }
    /* rows past `rows` inside a point read as zeros (out-of-bounds fill) */
    cuuint64_t dims[3] = {(cuuint64_t)(2 * N), (cuuint64_t)rows, (cuuint64_t)npoints};
    cuuint64_t strides[2] = {(cuuint64_t)(2 * N * 4), (cuuint64_t)(2 * N * 4) * (cuuint64_t)point_rows};
    cuuint32_t box[3] = {2 * DG_BK, 128, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(&g->tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)V, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        free(g);
        return qgt_set_error(-6, "digit gram: cuTensorMapEncodeTiled failed (%d)", (int)r);
    }
    size_t pbytes = (size_t)npoints * g->nsplit * g->ntp * 2 * 128 * 128 * sizeof(float);
    cudaError_t e = cudaMalloc((void**)&g->part, pbytes);
    if (e == cudaSuccess) e = cudaMalloc((void**)&g->ctl, sizeof(dg_ctl_t));
    if (e == cudaSuccess) e = cudaMemset(g->ctl, 0, sizeof(dg_ctl_t));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(dg_gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, DG_SMEM_BYTES);
    if (e != cudaSuccess) {
        cudaFree(g->part);
        cudaFree(g->ctl);
        free(g);
        return qgt_set_error(e == cudaErrorMemoryAllocation ? -2 : -6, "digit gram: %s", cudaGetErrorString(e));
    }
    *out = g;
    return 0;
}

extern "C" int qgt_dev_dg_gram_run(qgt_dg_gram_t* g, double* HG, void* stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    // the status word describes this run only (a run after a failed one starts clean)
    cudaError_t e = cudaMemsetAsync(&g->ctl->err, 0, sizeof(int), s);
    if (e != cudaSuccess) return qgt_set_error(-6, "digit gram: %s", cudaGetErrorString(e));
    dg_gram_kernel<<<dim3((unsigned)(g->ntp * g->nsplit), 1, g->npoints), DG_THREADS, DG_SMEM_BYTES, s>>>(g->tmap, g->nbk, g->N, g->kchunk, g->rowmax,
                                                                       g->rows, g->mbits, g->part, g->ctl);
    int rc = qgt_dev_last_error();
    if (rc) return rc;
    dg_reduce_kernel<<<dim3((unsigned)((g->rows + 31) / 32), (unsigned)g->rows, g->npoints), 256, 0, s>>>(
        g->part, g->rowmax, g->rows, g->nbk, g->ntp, g->nsplit, g->mbits, (double2*)HG);
    return qgt_dev_last_error();
}

extern "C" const int* qgt_dev_dg_gram_err(const qgt_dg_gram_t* g) { return g ? &g->ctl->err : NULL; }

extern "C" int qgt_dev_dg_gram_set_stall(qgt_dg_gram_t* g, int stall, int64_t timeout_ns, void* stream)
{
    dg_ctl_t h;
    h.err = 0;
    h.stall = stall ? 1 : 0;
    h.timeout_ns = timeout_ns > 0 ? (long long)timeout_ns : 0;
    cudaError_t e = cudaMemcpyAsync(g->ctl, &h, sizeof h, cudaMemcpyHostToDevice, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    return e == cudaSuccess ? 0 : qgt_set_error(-6, "digit gram: %s", cudaGetErrorString(e));
}

extern "C" int qgt_dev_dg_gram_status(qgt_dg_gram_t* g, void* stream)
{
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, &g->ctl->err, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return qgt_set_error(-6, "digit gram status: %s", cudaGetErrorString(e));
    return h;
}

extern "C" void qgt_dev_dg_gram_destroy(qgt_dg_gram_t* g)
{
    if (!g) return;
    cudaFree(g->part);
    cudaFree(g->ctl);
    free(g);
}

extern "C" int64_t qgt_dev_dg_gram_scratch_bytes(const qgt_dg_gram_t* g)
{
    return g ? (int64_t)g->npoints * g->nsplit * g->ntp * 2 * 128 * 128 * (int64_t)sizeof(float) : 0;
}

extern "C" void qgt_dev_dg_gram_shape(const qgt_dg_gram_t* g, int* ntp, int* nsplit, int64_t* kchunk)
{
    if (ntp) *ntp = g->ntp;
    if (nsplit) *nsplit = g->nsplit;
    if (kchunk) *kchunk = g->kchunk;
}

// ---- row maxima: max_k |x_rk| (complex modulus) of complex64 rows, as float bits ----
__global__ void rowmax_kernel(const float2* __restrict__ V, int64_t N, int row0, int nrows, uint32_t* __restrict__ out)
{
    __shared__ float red[32];
    const int r = row0 + blockIdx.y;
    float m = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        float2 v = V[(int64_t)r * N + i];
        m = fmaxf(m, sqrtf(v.x * v.x + v.y * v.y));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) atomicMax(out + r, __float_as_uint(m));
    }
}

extern "C" int qgt_dev_rowmax(const void* V, int64_t N, int32_t row0, int32_t nrows, uint32_t* out, void* s)
{
    if (nrows <= 0) return 0;
    int bx = (int)((N + 255) / 256);
    if (bx > 64) bx = 64;
    rowmax_kernel<<<dim3(bx, nrows), 256, 0, (cudaStream_t)s>>>((const float2*)V, N, row0, nrows, out);
    return qgt_dev_last_error();
}
