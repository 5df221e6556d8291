// qgt_learned.cu -- the learned metric preconditioner: a small MLP that maps
// circuit parameters theta (P) to M = diag(d) + U U^T (U: P x r), trained on
// exact metrics Re Q + lambda I, and the Woodbury PCG solve that uses it.
//
// The reference has no learned counterpart; its nearest pieces are the CPU
// float MLP of src/quantum_geometric/learning/quantum_pipeline_impl.c:577-790
// and the unpreconditioned CG of
// src/quantum_geometric/hybrid/classical_optimization_engine.c:543-611.
//
// Network (all kernels here, FP32 accumulation, BF16 weights in the forward
// and backward products, FP32 master weights and Adam moments):
//   x  = [cos theta, sin theta]                     (2P features: periodic)
//   h1 = silu(W1 x + b1), h2 = silu(W2 h1 + b2)      (width W)
//   o  = W3 h2 + b3                                 (P + P r outputs)
//   d  = softplus(o[0:P]) + lambda,  U = u_scale * o[P:] (row-major P x r)
// Loss per sample: ||diag(d) + U U^T - T||_F^2 / ||T||_F^2, T = Re Q + lambda I.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../qgt_internal.h"

#define GT_M 64
#define GT_N 64
#define GT_K 16

template <typename T> __device__ __forceinline__ float ldf(const T* p);
template <> __device__ __forceinline__ float ldf<float>(const float* p) { return *p; }
template <> __device__ __forceinline__ float ldf<__nv_bfloat16>(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// C[m, n] (+)= sum_k A(m, k) B(k, n) (+ bias[n]); A(m, k) = A[m sAm + k sAk], B(k, n) = B[k sBk + n sBn].
// act 1: Z = pre-activation written to Zout, C = silu(Z).
template <typename TA, typename TB>
__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, const TA* __restrict__ A, int64_t sAm,
                                                   int64_t sAk, const TB* __restrict__ B, int64_t sBk, int64_t sBn,
                                                   float* __restrict__ C, int64_t ldc, const float* __restrict__ bias,
                                                   int act, float* __restrict__ Zout, int accumulate)
{
    __shared__ float As[GT_K][GT_M + 1];
    __shared__ float Bs[GT_K][GT_N + 1];
    const int m0 = blockIdx.y * GT_M, n0 = blockIdx.x * GT_N;
    const int tid = threadIdx.x, tr = tid / 16, tc = tid % 16;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
    for (int k0 = 0; k0 < K; k0 += GT_K) {
        for (int e = tid; e < GT_M * GT_K; e += 256) {
            const int mm = e / GT_K, kk = e % GT_K;
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < K) ? ldf<TA>(A + (int64_t)m * sAm + (int64_t)k * sAk) : 0.f;
        }
        for (int e = tid; e < GT_N * GT_K; e += 256) {
            const int nn = e % GT_N, kk = e / GT_N;
            const int n = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = (n < N && k < K) ? ldf<TB>(B + (int64_t)k * sBk + (int64_t)n * sBn) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GT_K; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][tr * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tc * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int m = m0 + tr * 4 + i, n = n0 + tc * 4 + j;
            if (m >= M || n >= N) continue;
            float z = acc[i][j] + (bias ? bias[n] : 0.f);
            float* c = C + (int64_t)m * ldc + n;
            if (act == 1) {
                Zout[(int64_t)m * ldc + n] = z;
                z = z / (1.f + __expf(-z));
            }
            *c = accumulate ? *c + z : z;
        }
}

template <typename TA, typename TB>
static int gemm(int M, int N, int K, const TA* A, int64_t sAm, int64_t sAk, const TB* B, int64_t sBk, int64_t sBn,
                float* C, int64_t ldc, const float* bias, int act, float* Z, int accumulate, cudaStream_t s)
{
    dim3 g((N + GT_N - 1) / GT_N, (M + GT_M - 1) / GT_M);
    gemm_kernel<TA, TB><<<g, 256, 0, s>>>(M, N, K, A, sAm, sAk, B, sBk, sBn, C, ldc, bias, act, Z, accumulate);
    return qgt_dev_last_error();
}

// features: X[s, p] = cos theta, X[s, P + p] = sin theta
// sample s reads theta row idx[s] (idx NULL: row s)
__global__ void features_kernel(const double* __restrict__ theta, const int32_t* __restrict__ idx, int S, int P,
                                float* __restrict__ X)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)S * P) return;
    const int s = (int)(i / P), p = (int)(i % P);
    const int64_t src = (int64_t)(idx ? idx[s] : s) * P + p;
    double sn, cs;
    sincos(theta[src], &sn, &cs);
    X[(int64_t)s * 2 * P + p] = (float)cs;
    X[(int64_t)s * 2 * P + P + p] = (float)sn;
}

// dZ = dH * silu'(Z)
__global__ void silu_back_kernel(const float* __restrict__ Z, float* __restrict__ dH, int64_t n)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float z = Z[i], sg = 1.f / (1.f + __expf(-z));
    dH[i] *= sg * (1.f + z * (1.f - sg));
}

// db[n] = sum_m dZ[m, n]
__global__ void colsum_kernel(const float* __restrict__ dZ, int M, int N, float* __restrict__ db)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int m = 0; m < M; m++) s += dZ[(int64_t)m * N + n];
    db[n] = s;
}

// per sample (one CTA): loss and dL/do for M = diag(d) + U U^T against T = metric + lambda I.
// metric: S x P x P floats.  o, dO: S x (P + P r).
__global__ void __launch_bounds__(256) lr_loss_kernel(const float* __restrict__ O, const float* __restrict__ metric,
                                                      const int32_t* __restrict__ idx, int P, int r, float lambda,
                                                      float u_scale, float* __restrict__ dO, float* __restrict__ loss,
                                                      float inv_batch)
{
    extern __shared__ float sh[];
    float* U = sh;               // P x r
    float* d = U + P * r;        // P
    __shared__ float red[8];
    __shared__ float nrm_s;
    const int s = blockIdx.x, tid = threadIdx.x;
    const int od = P + P * r;
    const float* o = O + (int64_t)s * od;
    const float* T = metric + (int64_t)(idx ? idx[s] : s) * P * P;
    for (int i = tid; i < P * r; i += blockDim.x) U[i] = u_scale * o[P + i];
    for (int i = tid; i < P; i += blockDim.x) {
        const float x = o[i];
        d[i] = (x > 20.f ? x : log1pf(__expf(x))) + lambda;
    }
    // ||T||^2
    float part = 0.f;
    for (int64_t e = tid; e < (int64_t)P * P; e += blockDim.x) {
        const int i = (int)(e / P), j = (int)(e % P);
        const float t = T[e] + (i == j ? lambda : 0.f);
        part += t * t;
    }
    for (int w = 16; w > 0; w >>= 1) part += __shfl_xor_sync(0xffffffffu, part, w);
    if ((tid & 31) == 0) red[tid >> 5] = part;
    __syncthreads();
    if (tid == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        nrm_s = t > 0.f ? t : 1.f;
    }
    __syncthreads();
    const float inv = 1.f / nrm_s;
    // row i per thread: residual E_ij = M_ij - T_ij, dM = 2 E / nrm; dU_i = 2 sum_j dM_ij U_j (dM symmetric)
    float lpart = 0.f;
    for (int i = tid; i < P; i += blockDim.x) {
        float du[32];
        for (int k = 0; k < r; k++) du[k] = 0.f;
        float ddi = 0.f;
        for (int j = 0; j < P; j++) {
            float m = (i == j) ? d[i] : 0.f;
            for (int k = 0; k < r; k++) m = fmaf(U[i * r + k], U[j * r + k], m);
            const float t = T[(int64_t)i * P + j] + (i == j ? lambda : 0.f);
            const float e = m - t;
            lpart += e * e;
            const float g = 2.f * e * inv;
            if (i == j) ddi = g;
            for (int k = 0; k < r; k++) du[k] = fmaf(2.f * g, U[j * r + k], du[k]);
        }
        float* dos = dO + (int64_t)s * od;
        const float x = o[i];
        dos[i] = ddi * (1.f / (1.f + __expf(-x))) * inv_batch;   // softplus' = sigmoid
        for (int k = 0; k < r; k++) dos[P + i * r + k] = du[k] * u_scale * inv_batch;
    }
    for (int w = 16; w > 0; w >>= 1) lpart += __shfl_xor_sync(0xffffffffu, lpart, w);
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = lpart;
    __syncthreads();
    if (tid == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        atomicAdd(loss, t * inv * inv_batch);
    }
}

// d, U (FP64, for the solver) from the network outputs
__global__ void lr_outputs_kernel(const float* __restrict__ O, int S, int P, int r, float lambda, float u_scale,
                                  double* __restrict__ d, double* __restrict__ U)
{
    const int od = P + P * r;
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)S * od) return;
    const int s = (int)(i / od), c = (int)(i % od);
    const float x = O[i];
    if (c < P) d[(int64_t)s * P + c] = (double)(x > 20.f ? x : log1pf(__expf(x))) + (double)lambda;
    else U[(int64_t)s * P * r + (c - P)] = (double)(u_scale * x);
}

// Adam on FP32 master weights; BF16 copy for the products
__global__ void adam_kernel(float* __restrict__ w, __nv_bfloat16* __restrict__ wb, const float* __restrict__ g,
                            float* __restrict__ m1, float* __restrict__ m2, int64_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2, float wd)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] + wd * w[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float wi = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16_rn(wi);
}

__global__ void to_bf16_kernel(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb, int64_t n)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

// metric (FP32) from the complex FP64 Q blocks: out[s][i][j] = Re Q[s][i][j]
__global__ void metric_f32_kernel(const double* __restrict__ Q, int64_t count, float* __restrict__ out)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < count) out[i] = (float)Q[2 * i];
}

// ---------------------------------------------------------------------------
// PCG for (A + lambda I) x = b, A = Re of the complex P x P matrix Q (or a
// real matrix), preconditioner M = diag(d) + U U^T applied by Woodbury:
//   M^-1 y = D^-1 y - D^-1 U C^-1 U^T D^-1 y,  C = I + U^T D^-1 U  (r x r).
// r = 0 (U NULL) gives Jacobi / plain CG (d NULL: identity).  One CTA per
// system; x0 = 0; stops when ||r|| <= tol ||b|| or after max_iter.
// iters[sys] = iterations run; resid[sys] = final ||r|| / ||b||.
// ---------------------------------------------------------------------------
#define PCG_MAXP 1024
#define PCG_MAXR 32

__device__ __forceinline__ double block_sum(double v, double* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    return t;
}

__global__ void __launch_bounds__(256) pcg_kernel(const double* __restrict__ Qm, int cplx, int64_t sys_stride,
                                                  const double* __restrict__ bvec, int P, double lambda,
                                                  const double* __restrict__ dvec, const double* __restrict__ Umat, int r,
                                                  double tol, int max_iter, double* __restrict__ xout,
                                                  int32_t* __restrict__ iters, double* __restrict__ resid)
{
    extern __shared__ double sm[];
    double* x = sm;
    double* rv = x + P;
    double* z = rv + P;
    double* p = z + P;
    double* ap = p + P;
    double* dinv = ap + P;
    double* U = dinv + P;            // P x r
    double* Cf = U + P * r;          // r x r Cholesky factor of C
    double* w = Cf + r * r;          // r
    __shared__ double red[8];
    const int sys = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double* A = Qm + (int64_t)sys * sys_stride;
    const double* b = bvec + (int64_t)sys * P;
    for (int i = tid; i < P; i += blockDim.x) {
        x[i] = 0;
        rv[i] = b[i];
        dinv[i] = dvec ? 1.0 / dvec[(int64_t)sys * P + i] : 1.0;
    }
    for (int i = tid; i < P * r; i += blockDim.x) U[i] = Umat[(int64_t)sys * P * r + i];
    __syncthreads();
    if (r > 0) {
        // C = I + U^T D^-1 U, then its Cholesky factor (one thread: r <= 32)
        for (int e = tid; e < r * r; e += blockDim.x) {
            const int k = e / r, l = e % r;
            double c = (k == l) ? 1.0 : 0.0;
            for (int i = 0; i < P; i++) c += U[i * r + k] * dinv[i] * U[i * r + l];
            Cf[e] = c;
        }
        __syncthreads();
        if (tid == 0) {
            for (int j = 0; j < r; j++) {
                double s = Cf[j * r + j];
                for (int k = 0; k < j; k++) s -= Cf[j * r + k] * Cf[j * r + k];
                const double l = sqrt(s > 1e-300 ? s : 1e-300);
                Cf[j * r + j] = l;
                for (int i = j + 1; i < r; i++) {
                    double t = Cf[i * r + j];
                    for (int k = 0; k < j; k++) t -= Cf[i * r + k] * Cf[j * r + k];
                    Cf[i * r + j] = t / l;
                }
            }
        }
        __syncthreads();
    }
    // z = M^-1 rv
    auto precond = [&]() {
        for (int i = tid; i < P; i += blockDim.x) z[i] = dinv[i] * rv[i];
        __syncthreads();
        if (r > 0) {
            for (int k = warp; k < r; k += (int)(blockDim.x >> 5)) {
                double s = 0;
                for (int i = lane; i < P; i += 32) s += U[i * r + k] * z[i];
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) w[k] = s;
            }
            __syncthreads();
            if (tid == 0) {
                for (int i = 0; i < r; i++) {          // forward L y = w
                    double t = w[i];
                    for (int k = 0; k < i; k++) t -= Cf[i * r + k] * w[k];
                    w[i] = t / Cf[i * r + i];
                }
                for (int i = r - 1; i >= 0; i--) {     // backward L^T s = y
                    double t = w[i];
                    for (int k = i + 1; k < r; k++) t -= Cf[k * r + i] * w[k];
                    w[i] = t / Cf[i * r + i];
                }
            }
            __syncthreads();
            for (int i = tid; i < P; i += blockDim.x) {
                double t = 0;
                for (int k = 0; k < r; k++) t += U[i * r + k] * w[k];
                z[i] -= dinv[i] * t;
            }
            __syncthreads();
        }
    };
    double bn = 0;
    for (int i = tid; i < P; i += blockDim.x) bn += b[i] * b[i];
    bn = sqrt(block_sum(bn, red));
    if (bn == 0) {
        if (tid == 0) { iters[sys] = 0; resid[sys] = 0; }
        for (int i = tid; i < P; i += blockDim.x) xout[(int64_t)sys * P + i] = 0;
        return;
    }
    precond();
    for (int i = tid; i < P; i += blockDim.x) p[i] = z[i];
    double rz = 0;
    for (int i = tid; i < P; i += blockDim.x) rz += rv[i] * z[i];
    rz = block_sum(rz, red);
    int it = 0;
    double rn = 1.0;
    for (; it < max_iter; it++) {
        __syncthreads();
        // ap = (A + lambda I) p, one warp per row
        for (int i = warp; i < P; i += (int)(blockDim.x >> 5)) {
            double s = 0;
            for (int j = lane; j < P; j += 32) s += (cplx ? A[2 * ((int64_t)i * P + j)] : A[(int64_t)i * P + j]) * p[j];
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) ap[i] = s + lambda * p[i];
        }
        __syncthreads();
        double pap = 0;
        for (int i = tid; i < P; i += blockDim.x) pap += p[i] * ap[i];
        pap = block_sum(pap, red);
        if (!(pap > 0)) break;
        const double alpha = rz / pap;
        double rr = 0;
        for (int i = tid; i < P; i += blockDim.x) {
            x[i] += alpha * p[i];
            rv[i] -= alpha * ap[i];
            rr += rv[i] * rv[i];
        }
        rr = block_sum(rr, red);
        rn = sqrt(rr) / bn;
        if (rn <= tol) { it++; break; }
        precond();
        double rzn = 0;
        for (int i = tid; i < P; i += blockDim.x) rzn += rv[i] * z[i];
        rzn = block_sum(rzn, red);
        const double beta = rzn / rz;
        rz = rzn;
        for (int i = tid; i < P; i += blockDim.x) p[i] = z[i] + beta * p[i];
    }
    __syncthreads();
    for (int i = tid; i < P; i += blockDim.x) xout[(int64_t)sys * P + i] = x[i];
    if (tid == 0) { iters[sys] = it; resid[sys] = rn; }
}

// theta -= eta x
__global__ void axpy_kernel(double* __restrict__ theta, const double* __restrict__ x, double eta, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) theta[i] -= eta * x[i];
}

extern "C" {

int qgt_dev_lr_features(const double* theta, const int32_t* idx, int32_t S, int32_t P, float* X, void* s)
{
    int64_t n = (int64_t)S * P;
    if (n <= 0) return 0;
    features_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)s>>>(theta, idx, S, P, X);
    return qgt_dev_last_error();
}

/* Y[M x N] = act(X[M x K] W^T + b), W row-major N x K (BF16); act: 0 none, 1 silu (Z = pre-activation) */
int qgt_dev_lr_linear(int32_t M, int32_t N, int32_t K, const float* X, const void* Wbf16, const float* b, float* Y,
                      int32_t act, float* Z, void* s)
{
    return gemm<float, __nv_bfloat16>(M, N, K, X, K, 1, (const __nv_bfloat16*)Wbf16, 1, K, Y, N, b, act, Z, 0,
                                      (cudaStream_t)s);
}

/* dX[M x K] = dY[M x N] W (W: N x K BF16) */
int qgt_dev_lr_linear_dx(int32_t M, int32_t N, int32_t K, const float* dY, const void* Wbf16, float* dX, void* s)
{
    return gemm<float, __nv_bfloat16>(M, K, N, dY, N, 1, (const __nv_bfloat16*)Wbf16, K, 1, dX, K, NULL, 0, NULL, 0,
                                      (cudaStream_t)s);
}

/* dW[N x K] = dY^T X, db[N] = column sums of dY */
int qgt_dev_lr_linear_dw(int32_t M, int32_t N, int32_t K, const float* dY, const float* X, float* dW, float* db,
                         void* s)
{
    int rc = gemm<float, float>(N, K, M, dY, 1, N, X, K, 1, dW, K, NULL, 0, NULL, 0, (cudaStream_t)s);
    if (rc) return rc;
    colsum_kernel<<<(N + 255) / 256, 256, 0, (cudaStream_t)s>>>(dY, M, N, db);
    return qgt_dev_last_error();
}

int qgt_dev_lr_silu_back(const float* Z, float* dH, int64_t n, void* s)
{
    if (n <= 0) return 0;
    silu_back_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)s>>>(Z, dH, n);
    return qgt_dev_last_error();
}

int qgt_dev_lr_loss(const float* O, const float* metric, const int32_t* idx, int32_t S, int32_t P, int32_t r,
                    float lambda, float u_scale, float* dO, float* loss, void* s)
{
    if (r > 32 || P > 4096) return qgt_set_error(-1, "learned preconditioner: P %d / rank %d too large", P, r);
    size_t smem = sizeof(float) * ((size_t)P * r + P);
    if (smem > 48 * 1024) return qgt_set_error(-1, "learned preconditioner: P x rank too large for the loss kernel");
    lr_loss_kernel<<<S, 256, smem, (cudaStream_t)s>>>(O, metric, idx, P, r, lambda, u_scale, dO, loss, 1.0f / (float)S);
    return qgt_dev_last_error();
}

int qgt_dev_lr_outputs(const float* O, int32_t S, int32_t P, int32_t r, float lambda, float u_scale, double* d,
                       double* U, void* s)
{
    int64_t n = (int64_t)S * (P + P * r);
    lr_outputs_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)s>>>(O, S, P, r, lambda, u_scale, d, U);
    return qgt_dev_last_error();
}

int qgt_dev_lr_adam(float* w, void* wbf16, const float* g, float* m1, float* m2, int64_t n, float lr, float b1,
                    float b2, float eps, int32_t step, float wd, void* s)
{
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)s>>>(w, (__nv_bfloat16*)wbf16, g, m1, m2, n, lr, b1,
                                                                          b2, eps, c1, c2, wd);
    return qgt_dev_last_error();
}

int qgt_dev_lr_to_bf16(const float* w, void* wb, int64_t n, void* s)
{
    to_bf16_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)s>>>(w, (__nv_bfloat16*)wb, n);
    return qgt_dev_last_error();
}

int qgt_dev_metric_f32(const double* Q, int64_t count, float* out, void* s)
{
    if (count <= 0) return 0;
    metric_f32_kernel<<<(unsigned)((count + 255) / 256), 256, 0, (cudaStream_t)s>>>(Q, count, out);
    return qgt_dev_last_error();
}

int qgt_dev_pcg(const double* Q, int32_t cplx, int64_t sys_stride, const double* b, int32_t P, double lambda,
                const double* d, const double* U, int32_t r, double tol, int32_t max_iter, double* x, int32_t* iters,
                double* resid, int32_t nsys, void* s)
{
    if (P < 1 || P > PCG_MAXP || r < 0 || r > PCG_MAXR || nsys < 1 || (r > 0 && !U))
        return qgt_set_error(-1, "pcg: P %d (max %d), rank %d (max %d), %d systems", P, PCG_MAXP, r, PCG_MAXR, nsys);
    size_t smem = sizeof(double) * ((size_t)6 * P + (size_t)P * r + (size_t)r * r + r + 1);
    if (smem > 200 * 1024) return qgt_set_error(-1, "pcg: P x rank too large for shared memory");
    static int attr = 0;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(pcg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return qgt_set_error(-6, "pcg: %s", cudaGetErrorString(e));
        attr = 1;
    }
    pcg_kernel<<<nsys, 256, smem, (cudaStream_t)s>>>(Q, cplx, sys_stride, b, P, lambda, d, U, r, tol, max_iter, x, iters,
                                                     resid);
    return qgt_dev_last_error();
}

int qgt_dev_axpy_update(double* theta, const double* x, double eta, int32_t n, void* s)
{
    axpy_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)s>>>(theta, x, eta, n);
    return qgt_dev_last_error();
}

}  // extern "C"
