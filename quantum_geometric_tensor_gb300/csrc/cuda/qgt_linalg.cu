// qgt_linalg.cu -- the dense complex linear algebra behind the reference's
// natural-gradient and metric entry points, on the GPU in FP64.
//
//   singular values   one-sided (Hestenes) Jacobi on the columns of G: every
//                     round rotates Pp/2 disjoint column pairs (round-robin
//                     "circle" order, one CTA per pair) until a sweep rotates
//                     nothing.  The columns of W = G V end up orthogonal,
//                     sigma_j = |w_j|, U_j = w_j / sigma_j.  Replaces the
//                     LAPACK cgesvd behind compute_complex_matrix_condition_number
//                     and compute_pseudoinverse_natural_gradient
//                     (src/quantum_geometric/core/quantum_geometric_gradient.c:2733-2884).
//   LU solve          (G + lambda I) x = g by LU with partial pivoting and the
//                     reference's singularity rule (|pivot|^2 < 1e-10 fails,
//                     src/quantum_geometric/core/matrix_operations.c:55-173):
//                     one launch per column, rows addressed through a
//                     permutation (no physical swaps), multipliers kept in a
//                     separate matrix so that no CTA reads what another
//                     writes within a launch.
//   reference CG      compute_natural_gradient_cpu's conjugate gradients
//                     (src/quantum_geometric/hybrid/classical_optimization_engine.c:543-611):
//                     x0 = 0, at most 100 iterations, stop when |p^T A p| < 1e-15
//                     or |r| < 1e-8.
//   outer metric      geometric_compute_metric's Fubini-Study branch
//                     (src/quantum_geometric/core/quantum_geometric_metric.c:85-189):
//                     M_ij = delta_ij - conj(psi_i) psi_j, complex64.
// These entry points take and return host buffers; each call owns its device
// buffers and stream.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#include "../qgt_internal.h"

#define LA_MAXP 8192
#define LA_THREADS 256

static int la_fail(cudaError_t e, const char* what)
{
    return qgt_set_error(e == cudaErrorMemoryAllocation ? -2 : -6, "%s: %s", what, cudaGetErrorString(e));
}

// sum of v over the block (blockDim.x a multiple of 32, <= 1024); every thread gets the total
__device__ __forceinline__ double la_block_sum(double v, double* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    return t;
}

// ---------------------------------------------------------------------------
// Fubini-Study outer metric: out[i][j] = delta_ij - conj(psi_i) psi_j (complex64 products, as the
// reference computes them in ComplexFloat)
// ---------------------------------------------------------------------------
__global__ void fs_outer_kernel(const float2* __restrict__ psi, int64_t dim, float2* __restrict__ out)
{
    for (int64_t i = blockIdx.y; i < dim; i += gridDim.y) {
        const float2 a = psi[i];
        for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < dim; j += (int64_t)gridDim.x * blockDim.x) {
            const float2 b = psi[j];
            const float re = a.x * b.x + a.y * b.y, im = a.x * b.y - a.y * b.x;
            out[i * dim + j] = make_float2((i == j ? 1.0f : 0.0f) - re, -im);
        }
    }
}

extern "C" int qgt_dev_fs_metric(const float* psi, int64_t dim, float* out)
{
    if (!psi || !out || dim <= 0 || dim > ((int64_t)1 << 16))
        return qgt_set_error(-1, "fs metric: dimension %lld out of range (1 .. 65536)", (long long)dim);
    float2 *pd = NULL, *od = NULL;
    cudaStream_t s = NULL;
    const size_t ob = (size_t)dim * (size_t)dim * sizeof(float2);
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void**)&pd, (size_t)dim * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc((void**)&od, ob);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pd, psi, (size_t)dim * sizeof(float2), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        const unsigned gx = (unsigned)((dim + 255) / 256 < 64 ? (dim + 255) / 256 : 64);
        const unsigned gy = (unsigned)(dim < 4096 ? dim : 4096);
        fs_outer_kernel<<<dim3(gx, gy), 256, 0, s>>>(pd, dim, od);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, od, ob, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(pd);
    cudaFree(od);
    if (s) cudaStreamDestroy(s);
    return e == cudaSuccess ? 0 : la_fail(e, "fs metric");
}

// ---------------------------------------------------------------------------
// one-sided Jacobi SVD.  W: P rows x Pp columns, column-major (W[c P + r]); V: Pp x Pp column-major.
// Pp = P rounded up to even; the padding column is zero and never rotates.
// ---------------------------------------------------------------------------
__global__ void svd_init_kernel(const float2* __restrict__ G, int P, int Pp, double2* __restrict__ W,
                                double2* __restrict__ V)
{
    const int64_t nW = (int64_t)P * Pp, nV = (int64_t)Pp * Pp;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nW + nV; e += (int64_t)gridDim.x * blockDim.x) {
        if (e < nW) {
            const int c = (int)(e / P), r = (int)(e - (int64_t)c * P);
            const float2 g = c < P ? G[(int64_t)r * P + c] : make_float2(0.f, 0.f);
            W[e] = make_double2((double)g.x, (double)g.y);
        } else {
            const int64_t f = e - nW;
            const int c = (int)(f / Pp), r = (int)(f - (int64_t)c * Pp);
            V[f] = make_double2(r == c ? 1.0 : 0.0, 0.0);
        }
    }
}

// the column pair of CTA k in round `round` of a round-robin over Pp players (player 0 fixed)
__device__ __forceinline__ void svd_pair(int k, int round, int Pp, int* a, int* b)
{
    const int m = Pp - 1;
    const int x = (k == 0) ? 0 : ((k - 1 + round) % m) + 1;
    const int yk = Pp - 1 - k;
    const int y = ((yk - 1 + round) % m) + 1;   // yk >= Pp / 2 >= 1
    *a = x < y ? x : y;
    *b = x < y ? y : x;
}

__global__ void __launch_bounds__(LA_THREADS) svd_round_kernel(double2* __restrict__ W, double2* __restrict__ V, int P,
                                                               int Pp, int round, double tol, int* __restrict__ rotated)
{
    __shared__ double red[LA_THREADS / 32];
    int a, b;
    svd_pair(blockIdx.x, round, Pp, &a, &b);
    double2* wa = W + (int64_t)a * P;
    double2* wb = W + (int64_t)b * P;
    double al = 0, be = 0, gr = 0, gi = 0;
    for (int r = threadIdx.x; r < P; r += blockDim.x) {
        const double2 x = wa[r], y = wb[r];
        al += x.x * x.x + x.y * x.y;
        be += y.x * y.x + y.y * y.y;
        gr += x.x * y.x + x.y * y.y;   // conj(x) y
        gi += x.x * y.y - x.y * y.x;
    }
    al = la_block_sum(al, red);
    be = la_block_sum(be, red);
    gr = la_block_sum(gr, red);
    gi = la_block_sum(gi, red);
    const double g = hypot(gr, gi);
    if (!(g > 0.0) || !(g > tol * sqrt(al * be))) return;   // uniform over the block
    if (threadIdx.x == 0) *rotated = 1;
    // rotation [[c, s e^{i phi}], [-s e^{-i phi}, c]] zeroing <w_a|w_b> = g e^{i phi}
    const double zeta = (be - al) / (2.0 * g);
    const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + hypot(1.0, zeta));
    const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
    const double er = gr / g, ei = gi / g;
    auto rot = [&](double2* u, double2* v, int n) {
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
            const double2 x = u[r], y = v[r];
            const double2 ey = make_double2(er * y.x + ei * y.y, er * y.y - ei * y.x);   // e^{-i phi} y
            const double2 ex = make_double2(er * x.x - ei * x.y, er * x.y + ei * x.x);   // e^{i phi} x
            u[r] = make_double2(c * x.x - s * ey.x, c * x.y - s * ey.y);
            v[r] = make_double2(s * ex.x + c * y.x, s * ex.y + c * y.y);
        }
    };
    rot(wa, wb, P);
    rot(V + (int64_t)a * Pp, V + (int64_t)b * Pp, Pp);
}

__global__ void __launch_bounds__(LA_THREADS) svd_sigma_kernel(const double2* __restrict__ W, int P, double* __restrict__ sig)
{
    __shared__ double red[LA_THREADS / 32];
    const double2* w = W + (int64_t)blockIdx.x * P;
    double s = 0;
    for (int r = threadIdx.x; r < P; r += blockDim.x) s += w[r].x * w[r].x + w[r].y * w[r].y;
    s = la_block_sum(s, red);
    if (threadIdx.x == 0) sig[blockIdx.x] = sqrt(s);
}

// coef_j = (sigma_j > cutoff) ? <w_j|g> / sigma_j^2 : 0   (U_j^H g / sigma_j with U_j = w_j / sigma_j)
__global__ void __launch_bounds__(LA_THREADS) pinv_coef_kernel(const double2* __restrict__ W, const double* __restrict__ sig,
                                                               const double2* __restrict__ g, int P, double cutoff,
                                                               double2* __restrict__ coef)
{
    __shared__ double red[LA_THREADS / 32];
    const int j = blockIdx.x;
    const double2* w = W + (int64_t)j * P;
    double re = 0, im = 0;
    for (int r = threadIdx.x; r < P; r += blockDim.x) {
        re += w[r].x * g[r].x + w[r].y * g[r].y;
        im += w[r].x * g[r].y - w[r].y * g[r].x;
    }
    re = la_block_sum(re, red);
    im = la_block_sum(im, red);
    if (threadIdx.x == 0) {
        const double sj = sig[j];
        const double k = (sj > cutoff) ? 1.0 / (sj * sj) : 0.0;
        coef[j] = make_double2(re * k, im * k);
    }
}

// x_i = sum_j V_ij coef_j
__global__ void pinv_apply_kernel(const double2* __restrict__ V, const double2* __restrict__ coef, int P, int Pp,
                                  double2* __restrict__ x)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    double re = 0, im = 0;
    for (int j = 0; j < P; j++) {
        const double2 v = V[(int64_t)j * Pp + i], c = coef[j];
        re += v.x * c.x - v.y * c.y;
        im += v.x * c.y + v.y * c.x;
    }
    x[i] = make_double2(re, im);
}

extern "C" int qgt_dev_svd_pinv(const float* G, int32_t P, double* sigma, const float* g, double cutoff, double* x,
                                int32_t max_sweeps, int32_t* sweeps_out)
{
    if (!G || P <= 0 || P > LA_MAXP || max_sweeps <= 0) return qgt_set_error(-1, "svd: P %d out of range (1 .. %d)", P, LA_MAXP);
    if ((g == NULL) != (x == NULL)) return qgt_set_error(-1, "svd: g and x go together");
    const int PP = P + (P & 1);   // even number of columns (odd P: one zero padding column)
    cudaStream_t s = NULL;
    float2* Gd = NULL;
    double2 *W = NULL, *V = NULL, *gd = NULL, *coef = NULL, *xd = NULL;
    double* sig = NULL;
    int* flag = NULL;
    int* flag_h = NULL;
    int sweeps = 0;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void**)&Gd, sizeof(float2) * (size_t)P * P);
    if (e == cudaSuccess) e = cudaMalloc((void**)&W, sizeof(double2) * (size_t)P * PP);
    if (e == cudaSuccess) e = cudaMalloc((void**)&V, sizeof(double2) * (size_t)PP * PP);
    if (e == cudaSuccess) e = cudaMalloc((void**)&sig, sizeof(double) * (size_t)PP);
    if (e == cudaSuccess) e = cudaMalloc((void**)&flag, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&flag_h, sizeof(int));
    if (e == cudaSuccess && g) e = cudaMalloc((void**)&gd, sizeof(double2) * (size_t)P);
    if (e == cudaSuccess && g) e = cudaMalloc((void**)&coef, sizeof(double2) * (size_t)P);
    if (e == cudaSuccess && g) e = cudaMalloc((void**)&xd, sizeof(double2) * (size_t)P);
    if (e == cudaSuccess) e = cudaMemcpyAsync(Gd, G, sizeof(float2) * (size_t)P * P, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        svd_init_kernel<<<256, 256, 0, s>>>(Gd, P, PP, W, V);
        e = cudaGetLastError();
    }
    // sweeps of PP - 1 rounds until one rotates nothing (tolerance 1e-15 of sqrt(|w_a|^2 |w_b|^2))
    for (int sw = 0; e == cudaSuccess && sw < max_sweeps; sw++) {
        e = cudaMemsetAsync(flag, 0, sizeof(int), s);
        for (int r = 0; e == cudaSuccess && r < PP - 1; r++) {
            svd_round_kernel<<<PP / 2, LA_THREADS, 0, s>>>(W, V, P, PP, r, 1e-15, flag);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(flag_h, flag, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        sweeps = sw + 1;
        if (e == cudaSuccess && *flag_h == 0) break;
    }
    if (e == cudaSuccess) {
        svd_sigma_kernel<<<P, LA_THREADS, 0, s>>>(W, P, sig);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && g) {
        // g as complex128
        double* gh = (double*)malloc(sizeof(double) * 2 * (size_t)P);
        if (!gh) e = cudaErrorMemoryAllocation;
        else {
            for (int i = 0; i < 2 * P; i++) gh[i] = (double)g[i];
            e = cudaMemcpyAsync(gd, gh, sizeof(double2) * (size_t)P, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            free(gh);
        }
        if (e == cudaSuccess) {
            pinv_coef_kernel<<<P, LA_THREADS, 0, s>>>(W, sig, gd, P, cutoff, coef);
            pinv_apply_kernel<<<(P + 255) / 256, 256, 0, s>>>(V, coef, P, PP, xd);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(x, xd, sizeof(double2) * (size_t)P, cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess && sigma) e = cudaMemcpyAsync(sigma, sig, sizeof(double) * (size_t)P, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    const int converged = (e == cudaSuccess) && flag_h && *flag_h == 0;
    cudaFree(Gd); cudaFree(W); cudaFree(V); cudaFree(sig); cudaFree(flag); cudaFree(gd); cudaFree(coef); cudaFree(xd);
    if (flag_h) cudaFreeHost(flag_h);
    if (s) cudaStreamDestroy(s);
    if (e != cudaSuccess) return la_fail(e, "svd");
    if (sweeps_out) *sweeps_out = sweeps;
    if (!converged) return qgt_set_error(-901, "svd: Jacobi sweeps did not converge in %d sweeps", max_sweeps);
    return 0;
}

// ---------------------------------------------------------------------------
// LU with partial pivoting of A = G + lambda I (complex128, row-major, physical rows fixed; perm maps
// position -> physical row), the reference's pivot rule: the first row of largest |a|^2 in position
// order; |a|^2 < 1e-10 is singular.
// ---------------------------------------------------------------------------
__global__ void lu_init_kernel(const float2* __restrict__ G, int P, double lambda, double2* __restrict__ A,
                               int* __restrict__ perm, int* __restrict__ fail)
{
    const int64_t n = (int64_t)P * P;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(e / P), c = (int)(e - (int64_t)r * P);
        const float2 g = G[e];
        A[e] = make_double2((double)g.x + (r == c ? lambda : 0.0), (double)g.y);
        if (c == 0) perm[r] = r;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *fail = 0;
}

__global__ void __launch_bounds__(LA_THREADS) lu_step_kernel(double2* __restrict__ A, double2* __restrict__ Lm,
                                                             const int* __restrict__ pin, int* __restrict__ pout, int k,
                                                             int P, int* __restrict__ fail)
{
    __shared__ double bv[LA_THREADS / 32];
    __shared__ int bi[LA_THREADS / 32];
    if (*fail) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // pivot: largest |a_ik|^2 over positions i >= k, the first one on ties (every CTA computes it)
    double best = -1.0;
    int bpos = P;
    for (int i = k + threadIdx.x; i < P; i += blockDim.x) {
        const double2 v = A[(int64_t)pin[i] * P + k];
        const double m = v.x * v.x + v.y * v.y;
        if (m > best) { best = m; bpos = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int op = __shfl_xor_sync(0xffffffffu, bpos, o);
        if (ov > best || (ov == best && op < bpos)) { best = ov; bpos = op; }
    }
    if (lane == 0) { bv[warp] = best; bi[warp] = bpos; }
    __syncthreads();
    best = bv[0];
    bpos = bi[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++)
        if (bv[w] > best || (bv[w] == best && bi[w] < bpos)) { best = bv[w]; bpos = bi[w]; }
    if (!(best >= 1e-10)) {   // singular (or not finite)
        if (blockIdx.x == 0 && threadIdx.x == 0) *fail = 1;
        return;
    }
    const int p = bpos;
    if (blockIdx.x == 0)
        for (int i = threadIdx.x; i < P; i += blockDim.x) pout[i] = (i == k) ? pin[p] : ((i == p) ? pin[k] : pin[i]);
    const int r = pin[p];
    const double2 d = A[(int64_t)r * P + k];
    const double inv = 1.0 / (d.x * d.x + d.y * d.y);
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int i = k + 1 + blockIdx.x * (int)(blockDim.x >> 5) + warp; i < P; i += nw) {
        const int ri = (i == p) ? pin[k] : pin[i];
        const double2 a = A[(int64_t)ri * P + k];
        const double2 l = make_double2((a.x * d.x + a.y * d.y) * inv, (a.y * d.x - a.x * d.y) * inv);   // a / d
        if (lane == 0) Lm[(int64_t)ri * P + k] = l;
        for (int j = k + 1 + lane; j < P; j += 32) {
            const double2 u = A[(int64_t)r * P + j];
            double2 w = A[(int64_t)ri * P + j];
            w.x -= l.x * u.x - l.y * u.y;
            w.y -= l.x * u.y + l.y * u.x;
            A[(int64_t)ri * P + j] = w;
        }
    }
}

// forward (unit lower, multipliers Lm) and backward (upper part of A) substitution; perm = final
// permutation.  A last pivot of exactly zero (or not finite) is reported as singular: the reference
// leaves it unchecked and divides by it.
__global__ void __launch_bounds__(LA_THREADS) lu_solve_kernel(const double2* __restrict__ A, const double2* __restrict__ Lm,
                                                              const int* __restrict__ perm, const float2* __restrict__ b,
                                                              int P, double2* __restrict__ x, int* __restrict__ fail)
{
    __shared__ int bad;
    if (*fail) return;
    if (threadIdx.x == 0) {
        const double2 d = A[(int64_t)perm[P - 1] * P + P - 1];
        const double m = d.x * d.x + d.y * d.y;
        bad = !(m > 0.0) || !isfinite(m);
        if (bad) *fail = 1;
    }
    __syncthreads();
    if (bad) return;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const float2 v = b[perm[i]];
        x[i] = make_double2((double)v.x, (double)v.y);
    }
    __syncthreads();
    for (int i = 0; i < P; i++) {
        const double2 yi = x[i];
        for (int l = i + 1 + threadIdx.x; l < P; l += blockDim.x) {
            const double2 m = Lm[(int64_t)perm[l] * P + i];
            double2 w = x[l];
            w.x -= m.x * yi.x - m.y * yi.y;
            w.y -= m.x * yi.y + m.y * yi.x;
            x[l] = w;
        }
        __syncthreads();
    }
    for (int i = P - 1; i >= 0; i--) {
        if (threadIdx.x == 0) {
            const double2 d = A[(int64_t)perm[i] * P + i], v = x[i];
            const double inv = 1.0 / (d.x * d.x + d.y * d.y);
            x[i] = make_double2((v.x * d.x + v.y * d.y) * inv, (v.y * d.x - v.x * d.y) * inv);
        }
        __syncthreads();
        const double2 xi = x[i];
        for (int l = threadIdx.x; l < i; l += blockDim.x) {
            const double2 u = A[(int64_t)perm[l] * P + i];
            double2 w = x[l];
            w.x -= u.x * xi.x - u.y * xi.y;
            w.y -= u.x * xi.y + u.y * xi.x;
            x[l] = w;
        }
        __syncthreads();
    }
}

extern "C" int qgt_dev_lu_solve(const float* G, int32_t P, double lambda, const float* g, double* x, int32_t* singular)
{
    if (!G || !g || !x || P <= 0 || P > LA_MAXP) return qgt_set_error(-1, "lu solve: P %d out of range (1 .. %d)", P, LA_MAXP);
    cudaStream_t s = NULL;
    float2 *Gd = NULL, *gd = NULL;
    double2 *A = NULL, *Lm = NULL, *xd = NULL;
    int *perm = NULL, *fail = NULL, *fail_h = NULL;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void**)&Gd, sizeof(float2) * (size_t)P * P);
    if (e == cudaSuccess) e = cudaMalloc((void**)&gd, sizeof(float2) * (size_t)P);
    if (e == cudaSuccess) e = cudaMalloc((void**)&A, sizeof(double2) * (size_t)P * P);
    if (e == cudaSuccess) e = cudaMalloc((void**)&Lm, sizeof(double2) * (size_t)P * P);
    if (e == cudaSuccess) e = cudaMalloc((void**)&xd, sizeof(double2) * (size_t)P);
    if (e == cudaSuccess) e = cudaMalloc((void**)&perm, sizeof(int) * 2 * (size_t)P);
    if (e == cudaSuccess) e = cudaMalloc((void**)&fail, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&fail_h, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpyAsync(Gd, G, sizeof(float2) * (size_t)P * P, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(gd, g, sizeof(float2) * (size_t)P, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        lu_init_kernel<<<256, 256, 0, s>>>(Gd, P, lambda, A, perm, fail);
        e = cudaGetLastError();
    }
    int cur = 0;   // perm + cur P holds the permutation of the current step
    for (int k = 0; e == cudaSuccess && k < P - 1; k++) {
        const int rows = P - k - 1, warps = LA_THREADS / 32;
        int nb = (rows + warps - 1) / warps;
        if (nb > 4 * 152) nb = 4 * 152;
        lu_step_kernel<<<nb, LA_THREADS, 0, s>>>(A, Lm, perm + (size_t)cur * P, perm + (size_t)(cur ^ 1) * P, k, P, fail);
        e = cudaGetLastError();
        cur ^= 1;
    }
    if (e == cudaSuccess) {
        lu_solve_kernel<<<1, LA_THREADS, 0, s>>>(A, Lm, perm + (size_t)cur * P, gd, P, xd, fail);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(fail_h, fail, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(x, xd, sizeof(double2) * (size_t)P, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    const int sing = (e == cudaSuccess) ? *fail_h : 1;
    cudaFree(Gd); cudaFree(gd); cudaFree(A); cudaFree(Lm); cudaFree(xd); cudaFree(perm); cudaFree(fail);
    if (fail_h) cudaFreeHost(fail_h);
    if (s) cudaStreamDestroy(s);
    if (e != cudaSuccess) return la_fail(e, "lu solve");
    if (singular) *singular = sing;
    return 0;
}

// ---------------------------------------------------------------------------
// the reference's CG on F x = g (one CTA; F real row-major)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(LA_THREADS) ref_cg_kernel(const double* __restrict__ F, const double* __restrict__ g,
                                                            int P, double* __restrict__ x, double* __restrict__ work)
{
    __shared__ double red[LA_THREADS / 32];
    double* r = work;
    double* p = work + P;
    double* ap = work + 2 * (size_t)P;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    double rs = 0;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        x[i] = 0.0;
        r[i] = g[i];
        p[i] = g[i];
        rs += g[i] * g[i];
    }
    double rsold = la_block_sum(rs, red);
    for (int it = 0; it < 100; it++) {
        __syncthreads();
        for (int i = warp; i < P; i += nwarp) {
            double s = 0;
            for (int j = lane; j < P; j += 32) s += F[(int64_t)i * P + j] * p[j];
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) ap[i] = s;
        }
        __syncthreads();
        double pap = 0;
        for (int i = threadIdx.x; i < P; i += blockDim.x) pap += p[i] * ap[i];
        pap = la_block_sum(pap, red);
        if (fabs(pap) < 1e-15) break;
        const double alpha = rsold / pap;
        double rn = 0;
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            x[i] += alpha * p[i];
            r[i] -= alpha * ap[i];
            rn += r[i] * r[i];
        }
        const double rsnew = la_block_sum(rn, red);
        if (sqrt(rsnew) < 1e-8) break;
        const double beta = rsnew / rsold;
        for (int i = threadIdx.x; i < P; i += blockDim.x) p[i] = r[i] + beta * p[i];
        rsold = rsnew;
    }
}

extern "C" int qgt_dev_ref_cg(const double* F, const double* g, int32_t P, double* x)
{
    if (!F || !g || !x || P <= 0 || P > LA_MAXP) return qgt_set_error(-1, "cg: P %d out of range (1 .. %d)", P, LA_MAXP);
    cudaStream_t s = NULL;
    double *Fd = NULL, *gd = NULL, *xd = NULL, *wd = NULL;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void**)&Fd, sizeof(double) * (size_t)P * P);
    if (e == cudaSuccess) e = cudaMalloc((void**)&gd, sizeof(double) * (size_t)P);
    if (e == cudaSuccess) e = cudaMalloc((void**)&xd, sizeof(double) * (size_t)P);
    if (e == cudaSuccess) e = cudaMalloc((void**)&wd, sizeof(double) * 3 * (size_t)P);
    if (e == cudaSuccess) e = cudaMemcpyAsync(Fd, F, sizeof(double) * (size_t)P * P, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(gd, g, sizeof(double) * (size_t)P, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        ref_cg_kernel<<<1, LA_THREADS, 0, s>>>(Fd, gd, P, xd, wd);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(x, xd, sizeof(double) * (size_t)P, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(Fd); cudaFree(gd); cudaFree(xd); cudaFree(wd);
    if (s) cudaStreamDestroy(s);
    return e == cudaSuccess ? 0 : la_fail(e, "cg");
}
