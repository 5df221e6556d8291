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
//
// FP64 is scarce on this part (about 2 FMA per clock per SM), and the
// factorisation's critical path (32 dependent pivots per diagonal block, each
// a square root and a reciprocal) is FP64-latency bound.  The refined solver
// (qgt_dev_cholesky_refined) therefore factors A + lambda I in FP32 with the
// same blocked kernels and recovers an FP64-accurate solution by iterative
// refinement against the FP64 residual (the mixed-precision scheme of
// LAPACK's DSPOSV): x_0 = (L L^T)^-1 b in FP32, then 3 times
// r = b - (A + lambda I) x in FP64, x += (L L^T)^-1 r.  Each step shrinks the
// error by about cond(A) 2^-24; if the last correction is still above
// 1e-10 |x| (cond(A) above ~1e5) status[0] = QGT_ERROR_CONVERGENCE_FAILED and
// the caller reruns the FP64 solver.
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
template <typename T>
__global__ void __launch_bounds__(CB* CB) chol_diag_kernel(T* __restrict__ L, int P, int jb, double* status)
{
    __shared__ T a[CB][CB + 1];
    const int tx = threadIdx.x % CB, ty = threadIdx.x / CB;
    const int j0 = jb * CB, nb = min(CB, P - j0);
    a[ty][tx] = (ty < nb && tx < nb) ? L[(int64_t)(j0 + ty) * P + j0 + tx] : (ty == tx ? (T)1 : (T)0);
    __syncthreads();
    __shared__ int bad;
    __shared__ T inv;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    // FP64 divisions and square roots are scarce on this part: one of each per column
    for (int k = 0; k < nb; k++) {
        if (threadIdx.x == 0) {
            T d = a[k][k];
            if (!(d > (T)0)) { bad = 1; d = (T)1; }
            const T l = sqrt(d);
            a[k][k] = l;
            inv = (T)1 / l;
        }
        __syncthreads();
        if (tx == k && ty > k && ty < nb) a[ty][k] *= inv;
        __syncthreads();
        if (ty > k && tx > k && tx <= ty && ty < nb) a[ty][tx] -= a[ty][k] * a[tx][k];
        __syncthreads();
    }
    if (ty < nb && tx < nb) L[(int64_t)(j0 + ty) * P + j0 + tx] = (tx <= ty) ? a[ty][tx] : (T)0;
    if (threadIdx.x == 0 && bad) status[0] = -34.0;
}

// L_ij = A_ij L_jj^-T for block rows i > j: each warp solves one row of the block
template <typename T>
__global__ void __launch_bounds__(CB* CB) chol_panel_kernel(T* __restrict__ L, int P, int jb)
{
    __shared__ T ljj[CB][CB + 1];
    __shared__ T rinv[CB];
    const int tx = threadIdx.x % CB, ty = threadIdx.x / CB;
    const int j0 = jb * CB, nb = min(CB, P - j0);
    const int i0 = (jb + 1 + blockIdx.x) * CB;
    ljj[ty][tx] = (ty < nb && tx < nb) ? L[(int64_t)(j0 + ty) * P + j0 + tx] : (ty == tx ? (T)1 : (T)0);
    __syncthreads();
    if (threadIdx.x < CB) rinv[threadIdx.x] = (T)1 / ljj[threadIdx.x][threadIdx.x];
    __syncthreads();
    const int r = i0 + ty;
    if (r >= P) return;
    // row r: x_c = (a_c - sum_{k<c} x_k ljj[c][k]) / ljj[c][c], lane = c
    T acur = (tx < nb) ? L[(int64_t)r * P + j0 + tx] : (T)0;
    T x = (T)0;
    for (int c = 0; c < nb; c++) {
        T xc = __shfl_sync(0xffffffffu, acur, c) * rinv[c];
        if (tx == c) x = xc;
        if (tx > c) acur -= xc * ljj[tx][c];
    }
    if (tx < nb) L[(int64_t)r * P + j0 + tx] = x;
}

// A_ik -= L_ij L_kj^T for the trailing block pairs i >= k > j
template <typename T>
__global__ void __launch_bounds__(CB* CB) chol_update_kernel(T* __restrict__ L, int P, int jb, int nt)
{
    __shared__ T li[CB][CB + 1], lk[CB][CB + 1];
    // blockIdx.x -> (bi, bk) with jb < bk <= bi < nt
    int m = nt - jb - 1, t = blockIdx.x, bi = 0;
    while (t >= bi + 1) { t -= bi + 1; bi++; }
    if (bi >= m) return;
    const int I = (jb + 1 + bi) * CB, K = (jb + 1 + t) * CB, j0 = jb * CB;
    const int tx = threadIdx.x % CB, ty = threadIdx.x / CB;
    const int nb = min(CB, P - j0);
    li[ty][tx] = (I + ty < P && tx < nb) ? L[(int64_t)(I + ty) * P + j0 + tx] : (T)0;
    lk[ty][tx] = (K + ty < P && tx < nb) ? L[(int64_t)(K + ty) * P + j0 + tx] : (T)0;
    __syncthreads();
    const int r = I + ty, c = K + tx;
    if (r >= P || c >= P || c > r) return;
    T s = (T)0;
#pragma unroll 8
    for (int q = 0; q < CB; q++) s += li[ty][q] * lk[tx][q];
    L[(int64_t)r * P + c] -= s;
}

// L y = b then L^T d = y, blocked, one CTA.  mode 0: x = d; 1: x += d; 2: x += d
// and status[0] = QGT_ERROR_CONVERGENCE_FAILED if max |d| > 1e-10 max |x| (refinement)
template <typename T>
__global__ void __launch_bounds__(CB* CB) chol_solve_kernel(const T* __restrict__ L, const double* __restrict__ b,
                                                            double* __restrict__ x, int P, int mode, double* status)
{
    __shared__ T y[CHOL_BLOCKED_MAXP];
    __shared__ T rd[CHOL_BLOCKED_MAXP];   // 1 / L_ii
    const int tx = threadIdx.x % CB, ty = threadIdx.x / CB;
    const int nt = (P + CB - 1) / CB;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        y[i] = (T)b[i];
        rd[i] = (T)1 / L[(int64_t)i * P + i];
    }
    __syncthreads();
    // forward
    for (int bb = 0; bb < nt; bb++) {
        const int r0 = bb * CB, nb = min(CB, P - r0);
        // y_blk -= L[blk, :r0] y[:r0]; warp ty handles row r0+ty, lanes stride over k
        T s = (T)0;
        if (ty < nb)
            for (int k = tx; k < r0; k += CB) s += L[(int64_t)(r0 + ty) * P + k] * y[k];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        __syncthreads();
        if (ty < nb && tx == 0) y[r0 + ty] -= s;
        __syncthreads();
        if (ty == 0) {  // one warp: triangular solve of the diagonal block
            T acur = (tx < nb) ? y[r0 + tx] : (T)0, xv = (T)0;
            for (int c = 0; c < nb; c++) {
                T xc = __shfl_sync(0xffffffffu, acur, c) * rd[r0 + c];
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
        T s = (T)0;
        if (ty < nb)
            for (int k = r0 + CB + tx; k < P; k += CB) s += L[(int64_t)k * P + r0 + ty] * y[k];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        __syncthreads();
        if (ty < nb && tx == 0) y[r0 + ty] -= s;
        __syncthreads();
        if (ty == 0) {
            T acur = (tx < nb) ? y[r0 + tx] : (T)0, xv = (T)0;
            for (int c = nb - 1; c >= 0; c--) {
                T xc = __shfl_sync(0xffffffffu, acur, c) * rd[r0 + c];
                if (tx == c) xv = xc;
                if (tx < c) acur -= xc * L[(int64_t)(r0 + c) * P + r0 + tx];
            }
            if (tx < nb) y[r0 + tx] = xv;
        }
        __syncthreads();
    }
    if (mode == 0) {
        for (int i = threadIdx.x; i < P; i += blockDim.x) x[i] = (double)y[i];
        return;
    }
    __shared__ double mx[2][CB];
    double dm = 0.0, xm = 0.0;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const double d = (double)y[i], xi = x[i] + d;
        x[i] = xi;
        dm = fmax(dm, fabs(d));
        xm = fmax(xm, fabs(xi));
        if (d != d) dm = INFINITY;
    }
    if (mode != 2) return;
    for (int o = 16; o > 0; o >>= 1) {
        dm = fmax(dm, __shfl_xor_sync(0xffffffffu, dm, o));
        xm = fmax(xm, __shfl_xor_sync(0xffffffffu, xm, o));
    }
    if (tx == 0) { mx[0][ty] = dm; mx[1][ty] = xm; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < CB; w++) { dm = fmax(dm, mx[0][w]); xm = fmax(xm, mx[1][w]); }
        if (!(dm <= 1e-10 * xm) && status[0] == 0.0) status[0] = -901.0;   // QGT_ERROR_CONVERGENCE_FAILED
    }
}

// refinement: A64 = sym(A) + lambda I (FP64, kept for residuals), L32 = FP32 copy to factor
__global__ void chol_init_mixed_kernel(const double* __restrict__ A, int cplx, int P, double lambda,
                                       double* __restrict__ A64, float* __restrict__ L32, double* status)
{
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx == 0) { status[0] = 0.0; status[1] = lambda; }
    if (idx >= (int64_t)P * P) return;
    int r = (int)(idx / P), c = (int)(idx % P);
    double v = cplx ? A[2 * idx] : A[idx];
    if (cplx) v = 0.5 * (v + A[2 * ((int64_t)c * P + r)]);
    if (r == c) v += lambda;
    A64[idx] = v;
    L32[idx] = (float)v;
}

// r = b - A64 x, one warp per row (FP64)
__global__ void chol_residual_kernel(const double* __restrict__ A64, const double* __restrict__ b,
                                     const double* __restrict__ x, double* __restrict__ r, int P, const int* conv)
{
    if (*conv) return;
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (row >= P) return;
    double s = 0.0;
    for (int c = lane; c < P; c += 32) s += A64[(int64_t)row * P + c] * x[c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) r[row] = b[row] - s;
}

// FP32 diagonal block jb in one warp, lane r holding row r in registers (no
// barriers): right-looking factorisation with the pivot and column broadcast by
// shuffles, then W_jb = L_jj^-1 column by column (lane c holds column c) for the
// solves.  Rows and columns past P are the identity.
__global__ void __launch_bounds__(32) chol32_diag_kernel(float* __restrict__ L, int P, int jb, float* __restrict__ W,
                                                         double* status)
{
    const int lane = threadIdx.x, j0 = jb * CB, nb = min(CB, P - j0);
    float a[CB];
#pragma unroll
    for (int c = 0; c < CB; c++) a[c] = (lane < nb && c < nb) ? L[(int64_t)(j0 + lane) * P + j0 + c] : (lane == c ? 1.f : 0.f);
    bool bad = false;
#pragma unroll
    for (int k = 0; k < CB; k++) {
        float piv = __shfl_sync(0xffffffffu, a[k], k);
        if (!(piv > 0.f)) { bad = true; piv = 1.f; }
        const float l = sqrtf(piv), il = 1.f / l;
        if (lane == k) a[k] = l;
        else if (lane > k) a[k] *= il;
        const float lk = a[k];
#pragma unroll
        for (int j = k + 1; j < CB; j++) {
            const float ljk = __shfl_sync(0xffffffffu, lk, j);
            if (lane >= j) a[j] -= lk * ljk;
        }
    }
    float w[CB];
#pragma unroll
    for (int r = 0; r < CB; r++) {
        const float drr = 1.f / __shfl_sync(0xffffffffu, a[r], r);
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < r; k++) acc += __shfl_sync(0xffffffffu, a[k], r) * w[k];
        w[r] = (lane == r) ? drr : ((lane < r) ? -acc * drr : 0.f);
    }
    if (lane < nb)
#pragma unroll
        for (int c = 0; c < CB; c++)
            if (c < nb) L[(int64_t)(j0 + lane) * P + j0 + c] = (c <= lane) ? a[c] : 0.f;
    float* out = W + (int64_t)jb * CB * CB;
#pragma unroll
    for (int r = 0; r < CB; r++) out[r * CB + lane] = w[r];
    if (lane == 0 && bad) status[0] = -34.0;
}

// (L L^T) d = rhs with the FP32 factor and its diagonal-block inverses W: per block a
// warp-per-row matrix-vector product with the solved part, then y_blk = W s (no
// sequential pivots).  mode 0: x = d; 1: x += d; 2: also the convergence check;
// conv[0] = 1 once a correction is below 1e-15 |x| (later refinement steps return at once)
__global__ void __launch_bounds__(CB* CB) chol32_solve_kernel(const float* __restrict__ L, const float* __restrict__ W,
                                                              const double* __restrict__ rhs, double* __restrict__ x,
                                                              int P, int mode, double* status, int* conv)
{
    __shared__ float y[CHOL_BLOCKED_MAXP];
    __shared__ float wbuf[2][CB][CB + 1];   // W of this block and the next (loaded a block ahead)
    __shared__ float t[CB];
    __shared__ float part[CB][CB + 1];
    if (mode != 0 && *conv) return;
    const int lane = threadIdx.x % CB, wp = threadIdx.x / CB;
    const int nt = (P + CB - 1) / CB;
    // forward: L y = rhs
    wbuf[0][wp][lane] = W[wp * CB + lane];
    __syncthreads();
    for (int bb = 0; bb < nt; bb++) {
        const int r0 = bb * CB;
        float(*wb)[CB + 1] = wbuf[bb & 1];
        if (bb + 1 < nt) wbuf[(bb + 1) & 1][wp][lane] = W[(int64_t)(bb + 1) * CB * CB + wp * CB + lane];
        const int row = r0 + wp;
        float s = 0.f;
        if (row < P)
            for (int k = lane; k < r0; k += CB) s += L[(int64_t)row * P + k] * y[k];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) t[wp] = row < P ? (float)rhs[row] - s : 0.f;
        __syncthreads();
        float v = wb[wp][lane] * t[lane];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && row < P) y[row] = v;
        __syncthreads();
    }
    // backward: L^T d = y, d stored over y
    wbuf[(nt - 1) & 1][wp][lane] = W[(int64_t)(nt - 1) * CB * CB + wp * CB + lane];
    __syncthreads();
    for (int bb = nt - 1; bb >= 0; bb--) {
        const int r0 = bb * CB;
        float(*wb)[CB + 1] = wbuf[bb & 1];
        if (bb > 0) wbuf[(bb - 1) & 1][wp][lane] = W[(int64_t)(bb - 1) * CB * CB + wp * CB + lane];
        // part[wp][c] = sum over rows k = r0 + CB + wp + CB m of L[k][r0 + c] d[k]
        float s = 0.f;
        if (r0 + lane < P)
            for (int k = r0 + CB + wp; k < P; k += CB) s += L[(int64_t)k * P + r0 + lane] * y[k];
        part[wp][lane] = s;
        __syncthreads();
        {   // u[c] = sum over warps q of part[q][c]: warp wp sums column c = wp (a shuffle tree)
            float u = part[lane][wp];
            for (int o = 16; o > 0; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
            if (lane == 0) t[wp] = (r0 + wp < P) ? y[r0 + wp] - u : 0.f;
        }
        __syncthreads();
        // d_blk[c] = sum_r W[r][c] t[r] (W^T t): warp wp computes column c = wp
        float v = wb[lane][wp] * t[lane];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && r0 + wp < P) y[r0 + wp] = v;
        __syncthreads();
    }
    if (mode == 0) {
        for (int i = threadIdx.x; i < P; i += blockDim.x) x[i] = (double)y[i];
        return;
    }
    __shared__ double mx[2][CB];
    double dm = 0.0, xm = 0.0;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const double d = (double)y[i], xi = x[i] + d;
        x[i] = xi;
        dm = fmax(dm, fabs(d));
        xm = fmax(xm, fabs(xi));
        if (d != d) dm = INFINITY;
    }
    for (int o = 16; o > 0; o >>= 1) {
        dm = fmax(dm, __shfl_xor_sync(0xffffffffu, dm, o));
        xm = fmax(xm, __shfl_xor_sync(0xffffffffu, xm, o));
    }
    if (lane == 0) { mx[0][wp] = dm; mx[1][wp] = xm; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < CB; q++) { dm = fmax(dm, mx[0][q]); xm = fmax(xm, mx[1][q]); }
        if (dm <= 1e-15 * xm) *conv = 1;
        if (mode == 2 && !(dm <= 1e-10 * xm) && status[0] == 0.0) status[0] = -901.0;   // QGT_ERROR_CONVERGENCE_FAILED
    }
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
        chol_diag_kernel<double><<<1, CB * CB, 0, s>>>(L, P, jb, status);
        int below = nt - jb - 1;
        if (below > 0) {
            chol_panel_kernel<double><<<below, CB * CB, 0, s>>>(L, P, jb);
            chol_update_kernel<double><<<below * (below + 1) / 2, CB * CB, 0, s>>>(L, P, jb, nt);
        }
        rc = qgt_dev_last_error();
    }
    if (!rc) {
        chol_solve_kernel<double><<<1, CB * CB, 0, s>>>(L, b, x, P, 0, status);
        rc = qgt_dev_last_error();
    }
    return rc;
}

#define CHOL_REFINE_STEPS 3

extern "C" int64_t qgt_dev_cholesky_refined_work(int32_t P)
{
    const int64_t PP = (int64_t)P * P, nt = (P + CB - 1) / CB;
    return PP + P + (PP + nt * CB * CB + 1) / 2 + 8;   // A64 | r | L32, W32 (floats) | convergence flag
}

extern "C" int qgt_dev_cholesky_refined(const double* A, int cplx, const double* b, int32_t P, double lambda,
                                        double* work, double* x, double* status, void* stream)
{
    if (P <= 0 || P > CHOL_BLOCKED_MAXP)
        return qgt_set_error(-1, "refined cholesky: P = %d outside [1, %d]", P, CHOL_BLOCKED_MAXP);
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t PP = (int64_t)P * P;
    const int nt = (P + CB - 1) / CB;
    double* A64 = work;
    double* r = work + PP;
    float* L = reinterpret_cast<float*>(work + PP + P);
    float* W = L + PP;
    int* conv = reinterpret_cast<int*>(work + PP + P + (PP + (int64_t)nt * CB * CB + 1) / 2);
    int rc = cudaMemsetAsync(conv, 0, sizeof(int), s) == cudaSuccess ? 0 : qgt_dev_last_error();
    if (!rc) {
        chol_init_mixed_kernel<<<(unsigned)((PP + 255) / 256), 256, 0, s>>>(A, cplx, P, lambda, A64, L, status);
        rc = qgt_dev_last_error();
    }
    for (int jb = 0; jb < nt && !rc; jb++) {
        chol32_diag_kernel<<<1, CB, 0, s>>>(L, P, jb, W, status);
        int below = nt - jb - 1;
        if (below > 0) {
            chol_panel_kernel<float><<<below, CB * CB, 0, s>>>(L, P, jb);
            chol_update_kernel<float><<<below * (below + 1) / 2, CB * CB, 0, s>>>(L, P, jb, nt);
        }
        rc = qgt_dev_last_error();
    }
    for (int it = -1; it < CHOL_REFINE_STEPS && !rc; it++) {
        const int mode = it < 0 ? 0 : (it == CHOL_REFINE_STEPS - 1 ? 2 : 1);
        const double* rhs = it < 0 ? b : r;
        if (it >= 0) chol_residual_kernel<<<(unsigned)((P + 7) / 8), 256, 0, s>>>(A64, b, x, r, P, conv);
        chol32_solve_kernel<<<1, CB * CB, 0, s>>>(L, W, rhs, x, P, mode, status, conv);
        rc = qgt_dev_last_error();
    }
    return rc;
}

extern "C" int qgt_dev_cholesky_refined_launches(int32_t P)
{
    const int nt = (P + CB - 1) / CB;
    return 2 + nt + 2 * (nt - 1) + 2 * CHOL_REFINE_STEPS;
}

extern "C" int qgt_dev_cholesky_launches(int32_t P)
{
    const int nt = (P + CB - 1) / CB;
    return 2 + nt + 2 * (nt - 1);
}
