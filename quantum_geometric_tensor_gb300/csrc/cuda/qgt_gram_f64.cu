// qgt_gram_f64.cu -- FP64 Gram HG_ij = <V_i|V_j> of the complex128 rows
// (psi, H psi, derivative slots) for the plain FP64 path.
//
// HG is Hermitian, so only tile pairs (ti <= tj) of 32 x 32 output tiles are
// computed.  The amplitude range is split over blockIdx.y (split-K); each CTA
// writes its partial tile to `part`, and a second kernel sums the partials in
// a fixed order (deterministic) and mirrors the lower triangle.
//
// Bound: FP64 FMA throughput (8 real flops per complex MAC), not HBM.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../qgt_internal.h"

#define GT 32      // output tile
#define KT 16      // amplitudes per smem stage

__device__ __forceinline__ void tile_pair_index(int tp, int nt, int* ti, int* tj)
{
    // enumerate (ti, tj), ti <= tj, row-major over ti
    int i = 0, rem = tp;
    while (rem >= nt - i) { rem -= nt - i; i++; }
    *ti = i;
    *tj = i + rem;
}

__global__ void __launch_bounds__(256) gram_f64_kernel(const double2* __restrict__ V, int64_t N, int rows, int nt,
                                                       int64_t kchunk, double2* __restrict__ part)
{
    __shared__ double2 As[KT][GT + 1];
    __shared__ double2 Bs[KT][GT + 1];
    int ti, tj;
    tile_pair_index(blockIdx.x, nt, &ti, &tj);
    const int64_t k0 = (int64_t)blockIdx.y * kchunk;
    int64_t k1 = k0 + kchunk;
    if (k1 > N) k1 = N;
    const int tid = threadIdx.x;
    const int tr = tid / 16, tc = tid % 16;  // 2x2 outputs per thread
    double2 acc[2][2];
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++) acc[a][b] = make_double2(0, 0);
    // loader: 256 threads load 32 rows x 16 amplitudes (2 per thread) for A and B
    const int lr = tid / 8, lk = (tid % 8) * 2;
    const int ra = ti * GT + lr, rb = tj * GT + lr;
    for (int64_t kb = k0; kb < k1; kb += KT) {
        for (int u = 0; u < 2; u++) {
            int64_t k = kb + lk + u;
            double2 va = make_double2(0, 0), vb = make_double2(0, 0);
            if (k < k1) {
                if (ra < rows) va = V[(int64_t)ra * N + k];
                if (rb < rows) vb = V[(int64_t)rb * N + k];
            }
            As[lk + u][lr] = va;
            Bs[lk + u][lr] = vb;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < KT; kk++) {
            double2 a0 = As[kk][tr * 2], a1 = As[kk][tr * 2 + 1];
            double2 b0 = Bs[kk][tc * 2], b1 = Bs[kk][tc * 2 + 1];
            // conj(a) * b
            acc[0][0].x += a0.x * b0.x + a0.y * b0.y; acc[0][0].y += a0.x * b0.y - a0.y * b0.x;
            acc[0][1].x += a0.x * b1.x + a0.y * b1.y; acc[0][1].y += a0.x * b1.y - a0.y * b1.x;
            acc[1][0].x += a1.x * b0.x + a1.y * b0.y; acc[1][0].y += a1.x * b0.y - a1.y * b0.x;
            acc[1][1].x += a1.x * b1.x + a1.y * b1.y; acc[1][1].y += a1.x * b1.y - a1.y * b1.x;
        }
        __syncthreads();
    }
    double2* out = part + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * (GT * GT);
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++) out[(tr * 2 + a) * GT + tc * 2 + b] = acc[a][b];
}

__global__ void gram_f64_reduce_kernel(const double2* __restrict__ part, int rows, int nt, int ntp, int nsplit,
                                       double2* __restrict__ HG)
{
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= (int64_t)rows * rows) return;
    int i = (int)(idx / rows), j = (int)(idx % rows);
    if (i > j) return;
    int ti = i / GT, tj = j / GT;
    // tile pair index of (ti, tj)
    int tp = ti * nt - ti * (ti - 1) / 2 + (tj - ti);
    double2 s = make_double2(0, 0);
    for (int sp = 0; sp < nsplit; sp++) {
        double2 v = part[((int64_t)sp * ntp + tp) * (GT * GT) + (i % GT) * GT + (j % GT)];
        s.x += v.x;
        s.y += v.y;
    }
    HG[(int64_t)i * rows + j] = s;
    HG[(int64_t)j * rows + i] = make_double2(s.x, -s.y);
}

extern "C" int qgt_dev_gram_f64(const void* V, int64_t N, int32_t rows, double* part, int32_t nsplit, double* HG,
                                void* stream)
{
    int nt = (rows + GT - 1) / GT;
    int ntp = nt * (nt + 1) / 2;
    int64_t kchunk = (N + nsplit - 1) / nsplit;
    kchunk = (kchunk + KT - 1) / KT * KT;
    int ns = (int)((N + kchunk - 1) / kchunk);
    cudaStream_t s = (cudaStream_t)stream;
    gram_f64_kernel<<<dim3(ntp, ns), 256, 0, s>>>((const double2*)V, N, rows, nt, kchunk, (double2*)part);
    int rc = qgt_dev_last_error();
    if (rc) return rc;
    int64_t cnt = (int64_t)rows * rows;
    gram_f64_reduce_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>((const double2*)part, rows, nt, ntp, ns,
                                                                         (double2*)HG);
    return qgt_dev_last_error();
}
