// qgt_cholesky.cu -- blocked FP64 Cholesky solve of (A + lambda I) x = b on
// the GPU, the natural-gradient step of a plan (learning/quantum_pipeline_impl.c:
// 1601-1682 restated in double and blocked).
//
// Right-looking, 32 x 32 blocks, lower triangle, row-major work matrix L:
//   for each block column j:
//     diag:   L_jj = chol(A_jj)                         (1 CTA)
//     panel:  L_ij = A_ij L_jj^-T        for i > j      (1 CTA per block row)
//     update: A_ik -= L_ij L_kj^T        for i >= k > j (1 CTA per block pair)
//   solve:    L y = b, L^T x = y, blocked             (1 CTA)
// 3 launches per block column + 2, all graph-capturable; no host round trip.
// A non-positive pivot sets status[0] = QGT_ERROR_NOT_POSITIVE_DEFINITE; the
// caller then reruns the retrying single-CTA solver (lambda x 10).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../qgt_internal.h"

#define CB 32
#define CHOL_BLOCKED_MAXP 2048   // the solve keeps y and 1 / L_ii in shared memory (32 KB)

__global__ void chol_init_kernel(const double* __restrict__ A, int cplx, int P, double lambda, double* __restrict__ L,
                                 double* status)
{
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx == 0) { status[0] = 0.0; status[1] = lambda; }
    if (idx >= (int64_t)P * P) return;
    int r = (int)(idx / P), c = (int)(idx % P);
    double v = cplx ? A[2 * idx] : A[idx];
    if (cplx) v = 0.5 * (v + A[2 * ((int64_t)c * P + r)]);  // symmetric part of Re Q
    L[idx] = (r == c) ? v + lambda : v;
}

// factor the diagonal block j (one CTA of 32 x 32 threads)
__global__ void __launch_bounds__(CB* CB) chol_diag_kernel(double* __restrict__ L, int P, int jb, double* status)
{
    __shared__ double a[CB][CB + 1];
    const int tx = threadIdx.x % CB, ty = threadIdx.x / CB;
    const int j0 = jb * CB, nb = min(CB, P - j0);
    a[ty][tx] = (ty < nb && tx < nb) ? L[(int64_t)(j0 + ty) * P + j0 + tx] : (ty == tx ? 1.0 : 0.0);
    __syncthreads();
    __shared__ int bad;
    __shared__ double inv;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    // FP64 divisions and square roots are scarce on this part: one of each per column
    for (int k = 0; k < nb; k++) {
        if (threadIdx.x == 0) {
            double d = a[k][k];
            if (!(d > 0.0)) { bad = 1; d = 1.0; }
            const double l = sqrt(d);
            a[k][k] = l;
            inv = 1.0 / l;
        }
        __syncthreads();
        if (tx == k && ty > k && ty < nb) a[ty][k] *= inv;
        __syncthreads();
        if (ty > k && tx > k && tx <= ty && ty < nb) a[ty][tx] -= a[ty][k] * a[tx][k];
        __syncthreads();
    }
    if (ty < nb && tx < nb) L[(int64_t)(j0 + ty) * P + j0 + tx] = (tx <= ty) ? a[ty][tx] : 0.0;
    if (threadIdx.x == 0 && bad) status[0] = -34.0;
}

// L_ij = A_ij L_jj^-T for block rows i > j: each warp solves one row of the block
__global__ void __launch_bounds__(CB* CB) chol_panel_kernel(double* __restrict__ L, int P, int jb)
{
    __shared__ double ljj[CB][CB + 1];
    __shared__ double rinv[CB];
    const int tx = threadIdx.x % CB, ty = threadIdx.x / CB;
    const int j0 = jb * CB, nb = min(CB, P - j0);
    const int i0 = (jb + 1 + blockIdx.x) * CB;
    ljj[ty][tx] = (ty < nb && tx < nb) ? L[(int64_t)(j0 + ty) * P + j0 + tx] : (ty == tx ? 1.0 : 0.0);
    __syncthreads();
    if (threadIdx.x < CB) rinv[threadIdx.x] = 1.0 / ljj[threadIdx.x][threadIdx.x];
    __syncthreads();
    const int r = i0 + ty;
    if (r >= P) return;
    // row r: x_c = (a_c - sum_{k<c} x_k ljj[c][k]) / ljj[c][c], lane = c
    double acur = (tx < nb) ? L[(int64_t)r * P + j0 + tx] : 0.0;
    double x = 0.0;
    for (int c = 0; c < nb; c++) {
        double xc = __shfl_sync(0xffffffffu, acur, c) * rinv[c];
        if (tx == c) x = xc;
        if (tx > c) acur -= xc * ljj[tx][c];
    }
    if (tx < nb) L[(int64_t)r * P + j0 + tx] = x;
}

// A_ik -= L_ij L_kj^T for the trailing block pairs i >= k > j
__global__ void __launch_bounds__(CB* CB) chol_update_kernel(double* __restrict__ L, int P, int jb, int nt)
{
    __shared__ double li[CB][CB + 1], lk[CB][CB + 1];
    // blockIdx.x -> (bi, bk) with jb < bk <= bi < nt
    int m = nt - jb - 1, t = blockIdx.x, bi = 0;
    while (t >= bi + 1) { t -= bi + 1; bi++; }
    if (bi >= m) return;
    const int I = (jb + 1 + bi) * CB, K = (jb + 1 + t) * CB, j0 = jb * CB;
    const int tx = threadIdx.x % CB, ty = threadIdx.x / CB;
    const int nb = min(CB, P - j0);
    li[ty][tx] = (I + ty < P && tx < nb) ? L[(int64_t)(I + ty) * P + j0 + tx] : 0.0;
    lk[ty][tx] = (K + ty < P && tx < nb) ? L[(int64_t)(K + ty) * P + j0 + tx] : 0.0;
    __syncthreads();
    const int r = I + ty, c = K + tx;
    if (r >= P || c >= P || c > r) return;
    double s = 0.0;
#pragma unroll 8
    for (int q = 0; q < CB; q++) s += li[ty][q] * lk[tx][q];
    L[(int64_t)r * P + c] -= s;
}

// L y = b then L^T x = y, blocked, one CTA
__global__ void __launch_bounds__(CB* CB) chol_solve_kernel(const double* __restrict__ L, const double* __restrict__ b,
                                                            double* __restrict__ x, int P)
{
    __shared__ double y[CHOL_BLOCKED_MAXP];
    __shared__ double rd[CHOL_BLOCKED_MAXP];   // 1 / L_ii
    const int tx = threadIdx.x % CB, ty = threadIdx.x / CB;
    const int nt = (P + CB - 1) / CB;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        y[i] = b[i];
        rd[i] = 1.0 / L[(int64_t)i * P + i];
    }
    __syncthreads();
    // forward
    for (int bb = 0; bb < nt; bb++) {
        const int r0 = bb * CB, nb = min(CB, P - r0);
        // y_blk -= L[blk, :r0] y[:r0]; warp ty handles row r0+ty, lanes stride over k
        double s = 0.0;
        if (ty < nb)
            for (int k = tx; k < r0; k += CB) s += L[(int64_t)(r0 + ty) * P + k] * y[k];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        __syncthreads();
        if (ty < nb && tx == 0) y[r0 + ty] -= s;
        __syncthreads();
        if (ty == 0) {  // one warp: triangular solve of the diagonal block
            double acur = (tx < nb) ? y[r0 + tx] : 0.0, xv = 0.0;
            for (int c = 0; c < nb; c++) {
                double xc = __shfl_sync(0xffffffffu, acur, c) * rd[r0 + c];
                if (tx == c) xv = xc;
                if (tx > c && tx < nb) acur -= xc * L[(int64_t)(r0 + tx) * P + r0 + c];
            }
            if (tx < nb) y[r0 + tx] = xv;
        }
        __syncthreads();
    }
    // backward: L^T x = y
    for (int bb = nt - 1; bb >= 0; bb--) {
        const int r0 = bb * CB, nb = min(CB, P - r0);
        double s = 0.0;
        if (ty < nb)
            for (int k = r0 + CB + tx; k < P; k += CB) s += L[(int64_t)k * P + r0 + ty] * y[k];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        __syncthreads();
        if (ty < nb && tx == 0) y[r0 + ty] -= s;
        __syncthreads();
        if (ty == 0) {
            double acur = (tx < nb) ? y[r0 + tx] : 0.0, xv = 0.0;
            for (int c = nb - 1; c >= 0; c--) {
                double xc = __shfl_sync(0xffffffffu, acur, c) * rd[r0 + c];
                if (tx == c) xv = xc;
                if (tx < c) acur -= xc * L[(int64_t)(r0 + c) * P + r0 + tx];
            }
            if (tx < nb) y[r0 + tx] = xv;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < P; i += blockDim.x) x[i] = y[i];
}

extern "C" int qgt_dev_cholesky_blocked(const double* A, int cplx, const double* b, int32_t P, double lambda,
                                        double* L, double* x, double* status, void* stream)
{
    if (P <= 0 || P > CHOL_BLOCKED_MAXP)
        return qgt_set_error(-1, "blocked cholesky: P = %d outside [1, %d]", P, CHOL_BLOCKED_MAXP);
    cudaStream_t s = (cudaStream_t)stream;
    int64_t PP = (int64_t)P * P;
    chol_init_kernel<<<(unsigned)((PP + 255) / 256), 256, 0, s>>>(A, cplx, P, lambda, L, status);
    int rc = qgt_dev_last_error();
    const int nt = (P + CB - 1) / CB;
    for (int jb = 0; jb < nt && !rc; jb++) {
        chol_diag_kernel<<<1, CB * CB, 0, s>>>(L, P, jb, status);
        int below = nt - jb - 1;
        if (below > 0) {
            chol_panel_kernel<<<below, CB * CB, 0, s>>>(L, P, jb);
            chol_update_kernel<<<below * (below + 1) / 2, CB * CB, 0, s>>>(L, P, jb, nt);
        }
        rc = qgt_dev_last_error();
    }
    if (!rc) {
        chol_solve_kernel<<<1, CB * CB, 0, s>>>(L, b, x, P);
        rc = qgt_dev_last_error();
    }
    return rc;
}

extern "C" int qgt_dev_cholesky_launches(int32_t P)
{
    const int nt = (P + CB - 1) / CB;
    return 2 + nt + 2 * (nt - 1);
}
