// qgt_device.cu -- device context, memory, streams and graphs, and the small
// FP64 kernels of a step: gate-coefficient preparation, the TFIM H|psi>,
// the renormalised projector (Gram -> QGT, energy, gradient) and the FP64
// Cholesky natural-gradient solve.
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdio.h>

#include "../qgt_internal.h"
#include "qgt_gb300.h"

#define QGT_OK 0
#define QGT_EINVAL (-1)
#define QGT_ENOMEM (-2)
#define QGT_EHW (-6)
#define QGT_ENOTPD (-34)

static int cuda_fail(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return QGT_OK;
    int code = (e == cudaErrorMemoryAllocation) ? QGT_ENOMEM : QGT_EHW;
    return qgt_set_error(code, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return cuda_fail(e_, what); } while (0)

extern "C" {

int qgt_dev_set_device(int device) { CK(cudaSetDevice(device), "cudaSetDevice"); return QGT_OK; }

int qgt_dev_malloc(void** p, size_t bytes)
{
    *p = NULL;
    if (bytes == 0) return QGT_OK;
    CK(cudaMalloc(p, bytes), "cudaMalloc");
    return QGT_OK;
}

int qgt_dev_free(void* p) { if (p) CK(cudaFree(p), "cudaFree"); return QGT_OK; }

int qgt_dev_memcpy_h2d(void* dst, const void* src, size_t bytes, void* s)
{
    if (bytes) CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)s), "cudaMemcpyAsync H2D");
    return QGT_OK;
}

int qgt_dev_memcpy_d2h(void* dst, const void* src, size_t bytes, void* s)
{
    if (bytes) CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)s), "cudaMemcpyAsync D2H");
    return QGT_OK;
}

int qgt_dev_memcpy_d2d(void* dst, const void* src, size_t bytes, void* s)
{
    if (bytes) CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)s), "cudaMemcpyAsync D2D");
    return QGT_OK;
}

int qgt_dev_memset(void* dst, int v, size_t bytes, void* s)
{
    if (bytes) CK(cudaMemsetAsync(dst, v, bytes, (cudaStream_t)s), "cudaMemsetAsync");
    return QGT_OK;
}

int qgt_dev_stream_create(void** s)
{
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    *s = (void*)st;
    return QGT_OK;
}

int qgt_dev_stream_destroy(void* s) { if (s) CK(cudaStreamDestroy((cudaStream_t)s), "cudaStreamDestroy"); return QGT_OK; }
int qgt_dev_stream_sync(void* s) { CK(cudaStreamSynchronize((cudaStream_t)s), "cudaStreamSynchronize"); return QGT_OK; }

int qgt_dev_graph_begin(void* s)
{
    CK(cudaStreamBeginCapture((cudaStream_t)s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    return QGT_OK;
}

int qgt_dev_graph_end(void* s, void** exec)
{
    cudaGraph_t g;
    CK(cudaStreamEndCapture((cudaStream_t)s, &g), "cudaStreamEndCapture");
    cudaGraphExec_t ge;
    cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    CK(e, "cudaGraphInstantiate");
    *exec = (void*)ge;
    return QGT_OK;
}

int qgt_dev_graph_launch(void* exec, void* s) { CK(cudaGraphLaunch((cudaGraphExec_t)exec, (cudaStream_t)s), "cudaGraphLaunch"); return QGT_OK; }
int qgt_dev_graph_destroy(void* exec) { if (exec) CK(cudaGraphExecDestroy((cudaGraphExec_t)exec), "cudaGraphExecDestroy"); return QGT_OK; }

int qgt_dev_host_alloc(void** p, size_t bytes) { CK(cudaMallocHost(p, bytes ? bytes : 1), "cudaMallocHost"); return QGT_OK; }
int qgt_dev_host_free(void* p) { if (p) CK(cudaFreeHost(p), "cudaFreeHost"); return QGT_OK; }

int qgt_dev_last_error(void) { cudaError_t e = cudaGetLastError(); return cuda_fail(e, "kernel launch"); }

const char* qgt_dev_error_string(void) { return cudaGetErrorString(cudaPeekAtLastError()); }

}  // extern "C"

// ---------------------------------------------------------------------------
// gate coefficients (FP64, from theta, on the device)
// 2x2 row-major matrices of a2: RX = [[c,-is],[-is,c]], RY = [[c,-s],[s,c]],
// RZ = diag(e^{-ia/2}, e^{ia/2}); fixed gates as in
// hybrid/quantum_classical_algorithms.c:228-276.
// ---------------------------------------------------------------------------
__global__ void prepare_kernel(const qgt_dev_coef_desc_t* d, int ncoef, const double* theta, double* coef,
                               int theta_stride, int coef_stride)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncoef) return;
    theta += (int64_t)blockIdx.y * theta_stride;   // parameter point
    coef += (int64_t)8 * blockIdx.y * coef_stride;
    qgt_dev_coef_desc_t g = d[c];
    const int inv = (g.type & QGT_COEF_INVERSE) != 0;   // the gate's inverse (backward transport)
    g.type &= ~QGT_COEF_INVERSE;
    double a = g.param >= 0 ? theta[g.param] : g.angle;
    if (inv) a = -a;
    double m[8] = {1, 0, 0, 0, 0, 0, 1, 0};
    double cs, sn;
    sincos(0.5 * a, &sn, &cs);
    const double r = 0.70710678118654752440;
    switch (g.type) {
    case QGT_GATE_RX: m[0] = cs; m[1] = 0; m[2] = 0; m[3] = -sn; m[4] = 0; m[5] = -sn; m[6] = cs; m[7] = 0; break;
    case QGT_GATE_RY: m[0] = cs; m[1] = 0; m[2] = -sn; m[3] = 0; m[4] = sn; m[5] = 0; m[6] = cs; m[7] = 0; break;
    case QGT_GATE_RZ: m[0] = cs; m[1] = -sn; m[2] = 0; m[3] = 0; m[4] = 0; m[5] = 0; m[6] = cs; m[7] = sn; break;
    case QGT_GATE_X: m[0] = 0; m[2] = 1; m[4] = 1; m[6] = 0; break;
    case QGT_GATE_Y: m[0] = 0; m[2] = 0; m[3] = -1; m[4] = 0; m[5] = 1; m[6] = 0; break;
    case QGT_GATE_Z: m[6] = -1; break;
    case QGT_GATE_H: m[0] = r; m[2] = r; m[4] = r; m[6] = -r; break;
    case QGT_GATE_S: m[6] = 0; m[7] = inv ? -1 : 1; break;
    case QGT_GATE_T: m[6] = r; m[7] = inv ? -r : r; break;
    default: break;
    }
    for (int i = 0; i < 8; i++) coef[8 * c + i] = m[i];
}

// ---------------------------------------------------------------------------
// Pauli sum: (H psi)_i = sum_k c_k i^ny_k (-1)^popc((i ^ x_k) & z_k) psi_{i ^ x_k}, scaled.
// Terms are staged in shared memory; psi stays L2-resident across the terms.
// ---------------------------------------------------------------------------
template <typename T, typename R>
__global__ void pauli_kernel(const T* __restrict__ psi, T* __restrict__ out, int64_t N,
                             const qgt_dev_pauli_term_t* __restrict__ terms, int nterms, double inv,
                             uint32_t* rowmax, int64_t point_stride, int32_t rowmax_stride)
{
    extern __shared__ qgt_dev_pauli_term_t st[];
    for (int k = threadIdx.x; k < nterms; k += blockDim.x) st[k] = terms[k];
    __syncthreads();
    psi += blockIdx.y * point_stride;   // parameter point
    out += blockIdx.y * point_stride;
    if (rowmax) rowmax += (int64_t)blockIdx.y * rowmax_stride;
    float vmax = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        double ar = 0, ai = 0;
        for (int k = 0; k < nterms; k++) {
            const uint64_t j = (uint64_t)i ^ st[k].x;
            const T v = psi[j];
            double c = st[k].c;
            if (__popcll(j & st[k].z) & 1) c = -c;
            switch (st[k].ny & 3) {   // c i^ny
            case 0: ar += c * (double)v.x; ai += c * (double)v.y; break;
            case 1: ar -= c * (double)v.y; ai += c * (double)v.x; break;
            case 2: ar -= c * (double)v.x; ai -= c * (double)v.y; break;
            default: ar += c * (double)v.y; ai -= c * (double)v.x; break;
            }
        }
        T o;
        o.x = (R)(ar * inv);
        o.y = (R)(ai * inv);
        out[i] = o;
        vmax = fmaxf(vmax, sqrtf((float)(o.x * o.x + o.y * o.y)));
    }
    if (rowmax) {
        __shared__ float red[32];
        for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = vmax;
        __syncthreads();
        if (threadIdx.x == 0) {
            float m = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = fmaxf(m, red[w]);
            atomicMax(rowmax, __float_as_uint(m));
        }
    }
}

// ---------------------------------------------------------------------------
// TFIM ring: (H psi)_i = -J zz(i) psi_i - h sum_q psi_{i ^ 2^q}, scaled
// ---------------------------------------------------------------------------
template <typename T, typename R>
__global__ void tfim_kernel(const T* __restrict__ psi, T* __restrict__ out, int n, R J, R h, R inv,
                            void* split, int64_t sld, int64_t pstride, int32_t srow, float sscale, int bf16,
                            uint32_t* rowmax, int64_t point_stride, int32_t rowmax_stride)
{
    int64_t N = (int64_t)1 << n;
    psi += blockIdx.y * point_stride;   // parameter point
    out += blockIdx.y * point_stride;
    if (rowmax) rowmax += (int64_t)blockIdx.y * rowmax_stride;
    float vmax = 0.f;
    int nb = n >= 3 ? n : n - 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        int zz = 0;
        for (int b = 0; b < nb; b++) {
            int qa = b, qb = (b + 1) % n;
            zz += (((i >> qa) ^ (i >> qb)) & 1) ? -1 : 1;
        }
        T v = psi[i];
        R ar = -J * (R)zz * v.x, ai = -J * (R)zz * v.y;
        for (int q = 0; q < n; q++) {
            T w = psi[i ^ ((int64_t)1 << q)];
            ar -= h * w.x;
            ai -= h * w.y;
        }
        T o;
        o.x = ar * inv;
        o.y = ai * inv;
        out[i] = o;
        vmax = fmaxf(vmax, sqrtf((float)(o.x * o.x + o.y * o.y)));
        if (split) {
            float xr = (float)o.x * sscale, xi = (float)o.y * sscale;
            int64_t at = (int64_t)srow * sld + i;
            if (bf16) {
                __nv_bfloat16* s = (__nv_bfloat16*)split;
                __nv_bfloat16 rh = __float2bfloat16_rn(xr), ih = __float2bfloat16_rn(xi);
                s[at] = rh;
                s[pstride + at] = __float2bfloat16_rn(xr - __bfloat162float(rh));
                s[2 * pstride + at] = ih;
                s[3 * pstride + at] = __float2bfloat16_rn(xi - __bfloat162float(ih));
            } else {
                __half* s = (__half*)split;
                __half rh = __float2half_rn(xr), ih = __float2half_rn(xi);
                s[at] = rh;
                s[pstride + at] = __float2half_rn(xr - __half2float(rh));
                s[2 * pstride + at] = ih;
                s[3 * pstride + at] = __float2half_rn(xi - __half2float(ih));
            }
        }
    }
    if (rowmax) {
        __shared__ float red[32];
        for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = vmax;
        __syncthreads();
        if (threadIdx.x == 0) {
            float m = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = fmaxf(m, red[w]);
            atomicMax(rowmax, __float_as_uint(m));
        }
    }
}

// ---------------------------------------------------------------------------
// renormalised projector: s = <psi|psi>, v_p = sum_{a in p} <d_a|psi>,
// B_pq = sum <d_a|d_b>, Q = B/s - v_p conj(v_q)/s^2.
// HG_ij = <V_i|V_j>, rows: 0 psi, 1 H psi / hscale, 2 + a slot a.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 hg(const double* HG, int rows, int i, int j)
{
    return make_double2(HG[2 * ((int64_t)i * rows + j)], HG[2 * ((int64_t)i * rows + j) + 1]);
}

// HG entry with the meet-in-the-middle scale correction: row r carries the
// extra amplitude scale rho[row_group[r]] of the complex64 gates it crossed twice
__device__ __forceinline__ double2 hgs(const qgt_dev_post_args_t& a, int i, int j, const double* rho)
{
    double2 v = hg(a.HG, a.rows, i, j);
    if (rho) {
        const int gi = a.row_group[i], gj = a.row_group[j];
        const double f = (gi >= 0 ? 1.0 / rho[gi] : 1.0) * (gj >= 0 ? 1.0 / rho[gj] : 1.0);
        v.x *= f;
        v.y *= f;
    }
    return v;
}

__global__ void post_qgt_kernel(qgt_dev_post_args_t a)
{
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int P = a.P;
    if (idx >= (int64_t)P * P) return;
    a.HG += (int64_t)2 * blockIdx.y * a.rows * a.rows;   // parameter point
    a.Q += (int64_t)2 * blockIdx.y * P * P;
    int p = (int)(idx / P), q = (int)(idx % P);
    const double* ir = a.rho ? a.rho + (int64_t)blockIdx.y * a.ngroups : NULL;
    double s = a.HG[0];
    double2 B = make_double2(0, 0), vp = make_double2(0, 0), vq = make_double2(0, 0);
    for (int x = a.param_ptr[p]; x < a.param_ptr[p + 1]; x++) {
        int sa = a.param_slots[x];
        double2 t = hgs(a, sa + 2, 0, ir);
        vp.x += t.x; vp.y += t.y;
        for (int y = a.param_ptr[q]; y < a.param_ptr[q + 1]; y++) {
            double2 u = hgs(a, sa + 2, a.param_slots[y] + 2, ir);
            B.x += u.x; B.y += u.y;
        }
    }
    for (int y = a.param_ptr[q]; y < a.param_ptr[q + 1]; y++) {
        double2 t = hgs(a, a.param_slots[y] + 2, 0, ir);
        vq.x += t.x; vq.y += t.y;
    }
    // v_p conj(v_q)
    double pr = vp.x * vq.x + vp.y * vq.y;
    double pi = vp.y * vq.x - vp.x * vq.y;
    double is = 1.0 / s, is2 = is * is;
    a.Q[2 * idx] = B.x * is - pr * is2;
    a.Q[2 * idx + 1] = B.y * is - pi * is2;
}

__global__ void post_grad_kernel(qgt_dev_post_args_t a)
{
    a.HG += (int64_t)2 * blockIdx.y * a.rows * a.rows;   // parameter point
    a.grad += (int64_t)blockIdx.y * a.P;
    if (a.energy) a.energy += blockIdx.y;
    const double* ir = a.rho ? a.rho + (int64_t)blockIdx.y * a.ngroups : NULL;
    double s = a.HG[0];
    double E = a.hscale * hgs(a, 0, 1, ir).x / s;
    if (threadIdx.x == 0 && blockIdx.x == 0 && a.energy) a.energy[0] = E;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.P; p += gridDim.x * blockDim.x) {
        double g = 0, v = 0;
        for (int x = a.param_ptr[p]; x < a.param_ptr[p + 1]; x++) {
            int sa = a.param_slots[x];
            g += hgs(a, sa + 2, 1, ir).x;
            v += hgs(a, sa + 2, 0, ir).x;
        }
        // d/dtheta <psi|H|psi>/<psi|psi> = 2 Re<d psi|H psi>/s - 2 E Re<d psi|psi>/s
        a.grad[p] = 2.0 * a.hscale * g / s - 2.0 * E * v / s;
    }
}

// ---------------------------------------------------------------------------
// FP64 Cholesky of (A + lambda I), lambda x10 retries, then two triangular
// solves (learning/quantum_pipeline_impl.c:1601-1682 restated in double on
// the GPU).  One CTA; the trailing update of each column is spread over the
// block.  work: P x P doubles.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) cholesky_kernel(const double* A, int cplx, const double* b, int P,
                                                        double lambda, double* L, double* x, double* status)
{
    // one system per CTA (batched solves: system blockIdx.x)
    A += (int64_t)blockIdx.x * P * P * (cplx ? 2 : 1);
    b += (int64_t)blockIdx.x * P;
    L += (int64_t)blockIdx.x * P * P;
    x += (int64_t)blockIdx.x * P;
    status += 2 * blockIdx.x;
    __shared__ int fail;
    __shared__ double red[32];
    double lam = lambda;
    for (int attempt = 0; attempt < 12; attempt++) {
        for (int64_t i = threadIdx.x; i < (int64_t)P * P; i += blockDim.x) {
            int r = (int)(i / P), c = (int)(i % P);
            double v = cplx ? A[2 * i] : A[i];
            L[i] = (r == c) ? v + lam : v;
        }
        if (threadIdx.x == 0) fail = 0;
        __syncthreads();
        for (int j = 0; j < P; j++) {
            double d = L[(int64_t)j * P + j];
            if (d <= 0.0 || !(d == d)) {
                if (threadIdx.x == 0) fail = 1;
            }
            __syncthreads();
            if (fail) break;
            double ljj = sqrt(d);
            for (int i = j + 1 + threadIdx.x; i < P; i += blockDim.x) L[(int64_t)i * P + j] /= ljj;
            __syncthreads();
            if (threadIdx.x == 0) L[(int64_t)j * P + j] = ljj;
            // trailing lower triangle: L[i][k] -= L[i][j] L[k][j], j < k <= i
            int m = P - j - 1;
            int64_t cnt = (int64_t)m * (m + 1) / 2;
            for (int64_t t = threadIdx.x; t < cnt; t += blockDim.x) {
                // t -> (ii, kk) with 0 <= kk <= ii < m
                int ii = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
                while ((int64_t)ii * (ii + 1) / 2 > t) ii--;
                while ((int64_t)(ii + 1) * (ii + 2) / 2 <= t) ii++;
                int kk = (int)(t - (int64_t)ii * (ii + 1) / 2);
                int i = j + 1 + ii, k = j + 1 + kk;
                L[(int64_t)i * P + k] -= L[(int64_t)i * P + j] * L[(int64_t)k * P + j];
            }
            __syncthreads();
        }
        __syncthreads();
        if (!fail) {
            // forward: L y = b (y in x), backward: L^T x = y
            for (int i = 0; i < P; i++) {
                double part = 0;
                for (int k = threadIdx.x; k < i; k += blockDim.x) part += L[(int64_t)i * P + k] * x[k];
                for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
                if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
                __syncthreads();
                if (threadIdx.x == 0) {
                    double s = 0;
                    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
                    x[i] = (b[i] - s) / L[(int64_t)i * P + i];
                }
                __syncthreads();
            }
            for (int i = P - 1; i >= 0; i--) {
                double part = 0;
                for (int k = i + 1 + threadIdx.x; k < P; k += blockDim.x) part += L[(int64_t)k * P + i] * x[k];
                for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
                if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
                __syncthreads();
                if (threadIdx.x == 0) {
                    double s = 0;
                    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
                    x[i] = (x[i] - s) / L[(int64_t)i * P + i];
                }
                __syncthreads();
            }
            if (threadIdx.x == 0) { status[0] = 0.0; status[1] = lam; }
            return;
        }
        lam *= 10.0;
        __syncthreads();
    }
    if (threadIdx.x == 0) { status[0] = (double)QGT_ENOTPD; status[1] = lam; }
}

extern "C" {

int qgt_dev_prepare(const qgt_dev_coef_desc_t* d, int32_t ncoef, const double* theta, double* coef, int32_t npoints,
                    int32_t theta_stride, int32_t coef_stride, void* s)
{
    if (ncoef <= 0) return QGT_OK;
    if (npoints < 1 || npoints > 65535) return qgt_set_error(QGT_EINVAL, "prepare: %d points", npoints);
    prepare_kernel<<<dim3((ncoef + 127) / 128, npoints), 128, 0, (cudaStream_t)s>>>(d, ncoef, theta, coef, theta_stride,
                                                                                      coef_stride);
    return qgt_dev_last_error();
}

int qgt_dev_tfim(const void* psi, void* out, int32_t n, double J, double h, double inv, int fp64,
                 void* split, int64_t sld, int64_t pstride, int32_t srow, float sscale, int32_t bf16,
                 uint32_t* rowmax, int32_t npoints, int64_t point_stride, int32_t rowmax_stride, void* s)
{
    int64_t N = (int64_t)1 << n;
    if (npoints < 1 || npoints > 65535 || (split && npoints > 1)) return qgt_set_error(QGT_EINVAL, "tfim: %d points", npoints);
    int64_t want = (152 * 16 + npoints - 1) / npoints;
    int blocks = (int)((N + 255) / 256);
    if (blocks > want) blocks = (int)want;
    dim3 grid((unsigned)blocks, (unsigned)npoints);
    if (fp64)
        tfim_kernel<double2, double><<<grid, 256, 0, (cudaStream_t)s>>>((const double2*)psi, (double2*)out, n, J, h,
                                                                          inv, NULL, 0, 0, 0, 0.f, 0, NULL, point_stride,
                                                                          0);
    else
        tfim_kernel<float2, float><<<grid, 256, 0, (cudaStream_t)s>>>((const float2*)psi, (float2*)out, n, (float)J,
                                                                        (float)h, (float)inv, split, sld, pstride, srow,
                                                                        sscale, bf16, rowmax, point_stride,
                                                                        rowmax_stride);
    return qgt_dev_last_error();
}

int qgt_dev_pauli(const void* psi, void* out, int32_t n, const qgt_dev_pauli_term_t* terms, int32_t nterms,
                  double inv, int fp64, uint32_t* rowmax, int32_t npoints, int64_t point_stride, int32_t rowmax_stride,
                  void* s)
{
    int64_t N = (int64_t)1 << n;
    if (npoints < 1 || npoints > 65535 || nterms < 0) return qgt_set_error(QGT_EINVAL, "pauli: %d points", npoints);
    int64_t want = (152 * 16 + npoints - 1) / npoints;
    int blocks = (int)((N + 255) / 256);
    if (blocks > want) blocks = (int)want;
    dim3 grid((unsigned)blocks, (unsigned)npoints);
    size_t smem = sizeof(qgt_dev_pauli_term_t) * (size_t)nterms;
    if (smem > 48 * 1024) return qgt_set_error(QGT_EINVAL, "pauli: %d terms exceed shared memory", nterms);
    if (fp64)
        pauli_kernel<double2, double><<<grid, 256, smem, (cudaStream_t)s>>>((const double2*)psi, (double2*)out, N, terms,
                                                                          nterms, inv, NULL, point_stride, 0);
    else
        pauli_kernel<float2, float><<<grid, 256, smem, (cudaStream_t)s>>>((const float2*)psi, (float2*)out, N, terms,
                                                                        nterms, inv, rowmax, point_stride, rowmax_stride);
    return qgt_dev_last_error();
}

int qgt_dev_post(const qgt_dev_post_args_t* a, void* s)
{
    int64_t PP = (int64_t)a->P * a->P;
    const int np = a->npoints > 0 ? a->npoints : 1;
    if (np > 65535) return qgt_set_error(QGT_EINVAL, "post: %d points", np);
    post_qgt_kernel<<<dim3((unsigned)((PP + 255) / 256), np), 256, 0, (cudaStream_t)s>>>(*a);
    int rc = qgt_dev_last_error();
    if (rc) return rc;
    if (a->has_h) {
        post_grad_kernel<<<dim3((a->P + 255) / 256, np), 256, 0, (cudaStream_t)s>>>(*a);
        rc = qgt_dev_last_error();
    }
    return rc;
}

int qgt_dev_cholesky(const double* A, int cplx, const double* b, int32_t P, double lambda, double* work, double* x,
                     double* status, void* s)
{
    if (P <= 0) return qgt_set_error(QGT_EINVAL, "cholesky: P must be positive");
    cholesky_kernel<<<1, 1024, 0, (cudaStream_t)s>>>(A, cplx, b, P, lambda, work, x, status);
    return qgt_dev_last_error();
}

int qgt_dev_cholesky_batch(const double* A, int cplx, const double* b, int32_t P, double lambda, double* work,
                           double* x, double* status, int32_t nsys, void* s)
{
    if (P <= 0 || nsys < 1 || nsys > 0x7fffffff) return qgt_set_error(QGT_EINVAL, "cholesky: bad batch");
    cholesky_kernel<<<nsys, 1024, 0, (cudaStream_t)s>>>(A, cplx, b, P, lambda, work, x, status);
    return qgt_dev_last_error();
}

}  // extern "C"

// ---------------------------------------------------------------------------
// host-supplied states -> Gram operands: complex128 rows are rounded to
// complex64 (the precision a mixed plan evolves in) and split into the four
// half-precision planes, or kept as complex128 for the FP64 Gram.
// ---------------------------------------------------------------------------
__global__ void split_rows_kernel(const double2* __restrict__ X, int rows, int64_t N, void* split, int64_t sld,
                                  int64_t pstride, int row0, float scale, int bf16)
{
    int64_t total = (int64_t)rows * N;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int r = (int)(t / N);
        int64_t i = t % N;
        double2 v = X[t];
        float xr = (float)v.x * scale, xi = (float)v.y * scale;
        int64_t at = (int64_t)(row0 + r) * sld + i;
        if (bf16) {
            __nv_bfloat16* s = (__nv_bfloat16*)split;
            __nv_bfloat16 rh = __float2bfloat16_rn(xr), ih = __float2bfloat16_rn(xi);
            s[at] = rh;
            s[pstride + at] = __float2bfloat16_rn(xr - __bfloat162float(rh));
            s[2 * pstride + at] = ih;
            s[3 * pstride + at] = __float2bfloat16_rn(xi - __bfloat162float(ih));
        } else {
            __half* s = (__half*)split;
            __half rh = __float2half_rn(xr), ih = __float2half_rn(xi);
            s[at] = rh;
            s[pstride + at] = __float2half_rn(xr - __half2float(rh));
            s[2 * pstride + at] = ih;
            s[3 * pstride + at] = __float2half_rn(xi - __half2float(ih));
        }
    }
}

extern "C" int qgt_dev_split_rows(const double* X, int32_t rows, int64_t N, void* split, int64_t sld, int64_t pstride,
                                  int32_t row0, float scale, int32_t bf16, void* s)
{
    int64_t total = (int64_t)rows * N;
    if (total <= 0) return QGT_OK;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 32) blocks = 152 * 32;
    split_rows_kernel<<<blocks, 256, 0, (cudaStream_t)s>>>((const double2*)X, rows, N, split, sld, pstride, row0, scale,
                                                           bf16);
    return qgt_dev_last_error();
}

// out = sum_k c_k V[row0 + k]  (complex128 rows, real coefficients)
__global__ void combine_rows_kernel(const double2* __restrict__ V, int64_t N, int row0, const double* __restrict__ c,
                                    int K, double2* __restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        double re = 0, im = 0;
        for (int k = 0; k < K; k++) {
            double2 v = V[(int64_t)(row0 + k) * N + i];
            re += c[k] * v.x;
            im += c[k] * v.y;
        }
        out[i] = make_double2(re, im);
    }
}

extern "C" int qgt_dev_combine_rows(const void* V, int64_t N, int32_t row0, const double* c, int32_t K, void* out,
                                    void* s)
{
    int blocks = (int)((N + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    combine_rows_kernel<<<blocks, 256, 0, (cudaStream_t)s>>>((const double2*)V, N, row0, c, K, (double2*)out);
    return qgt_dev_last_error();
}

__global__ void c128_to_c64_kernel(const double* __restrict__ X, int64_t count, float* __restrict__ Y)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        Y[i] = (float)X[i];
}

extern "C" int qgt_dev_c128_to_c64(const double* X, int64_t count, float* Y, void* s)
{
    int blocks = (int)((count + 255) / 256);
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (count > 0) c128_to_c64_kernel<<<blocks, 256, 0, (cudaStream_t)s>>>(X, count, Y);
    return qgt_dev_last_error();
}

extern "C" {
int qgt_dev_event_create(void** ev)
{
    cudaEvent_t e;
    CK(cudaEventCreate(&e), "cudaEventCreate");
    *ev = (void*)e;
    return QGT_OK;
}
int qgt_dev_event_destroy(void* ev) { if (ev) CK(cudaEventDestroy((cudaEvent_t)ev), "cudaEventDestroy"); return QGT_OK; }
int qgt_dev_event_record(void* ev, void* s) { CK(cudaEventRecord((cudaEvent_t)ev, (cudaStream_t)s), "cudaEventRecord"); return QGT_OK; }
int qgt_dev_event_sync(void* ev) { CK(cudaEventSynchronize((cudaEvent_t)ev), "cudaEventSynchronize"); return QGT_OK; }
int qgt_dev_stream_wait_event(void* s, void* ev)
{
    CK(cudaStreamWaitEvent((cudaStream_t)s, (cudaEvent_t)ev, 0), "cudaStreamWaitEvent");
    return QGT_OK;
}
int qgt_dev_event_elapsed(void* a, void* b, float* ms)
{
    CK(cudaEventSynchronize((cudaEvent_t)b), "cudaEventSynchronize");
    CK(cudaEventElapsedTime(ms, (cudaEvent_t)a, (cudaEvent_t)b), "cudaEventElapsedTime");
    return QGT_OK;
}
}

// ---------------------------------------------------------------------------
// complex64 gate coefficients with exact rotation angles.
// Every per-vector scale a gate applies is harmless (each vector of a step
// carries the product of all gates' scales and Q = B/s - v v^H / s^2 is
// invariant under it); only the rotation ANGLE of a rounded FP32 matrix is
// an error, and it is coherent across all vectors.  For RX/RZ the warp
// searches 512 radii r in [1 - 2^-15, 1 + 2^-15] for the FP32 pair
// (fl(r cos a/2), fl(r sin a/2)) closest to the exact ray: angle error
// ~1e-10 instead of ~6e-8.  RY takes the tangent form below (angle error at
// most 3e-8 rad, from rounding t).  Diagonal fixed gates get equal-modulus
// entries.
// One warp per coefficient; 8 floats per coefficient (2x2 complex, row-major).
// ---------------------------------------------------------------------------
__global__ void prepare32_kernel(const qgt_dev_coef_desc_t* d, int ncoef, const double* theta, float* coef,
                                 int theta_stride, int coef_stride)
{
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= ncoef) return;
    theta += (int64_t)blockIdx.y * theta_stride;   // parameter point
    coef += (int64_t)8 * blockIdx.y * coef_stride;
    qgt_dev_coef_desc_t g = d[c];
    const int inv = (g.type & QGT_COEF_INVERSE) != 0;   // the gate's inverse (backward transport)
    g.type &= ~QGT_COEF_INVERSE;
    float m[8] = {1.f, 0.f, 0.f, 0.f, 0.f, 0.f, 1.f, 0.f};
    if (g.type == QGT_GATE_RY) {
        // tangent form: RY = c [[1, -t], [t, 1]] (t = s / c, |t| <= 1) or
        // |s| [[k, -g], [g, k]] (k = c / |s|, g = sign s); the pass kernels
        // apply these scaled rotations with one multiply-add per component,
        // and the scale (the column norm) is divided out by the pass
        // renormalisation.  Both scales (c and |s|) are even in the angle, so
        // a gate and its inverse (backward transport) carry the same sign and
        // a vector that crosses both keeps its sign.
        double a = g.param >= 0 ? theta[g.param] : g.angle;
        if (inv) a = -a;
        double s0, c0;
        sincos(0.5 * a, &s0, &c0);
        if (fabs(c0) >= fabs(s0)) {
            const float t = (float)(s0 / c0);
            m[0] = 1.f; m[2] = -t; m[4] = t; m[6] = 1.f;
        } else {
            const float k = (float)(c0 / fabs(s0)), g = s0 > 0 ? 1.f : -1.f;
            m[0] = k; m[2] = -g; m[4] = g; m[6] = k;
        }
    } else if (g.type == QGT_GATE_RX || g.type == QGT_GATE_RZ) {
        double a = g.param >= 0 ? theta[g.param] : g.angle;
        if (inv) a = -a;
        double s0, c0;
        sincos(0.5 * a, &s0, &c0);
        double best = 1e300;
        float bc = (float)c0, bs = (float)s0;
        for (int i = 0; i < 16; i++) {
            int k = lane + 32 * i - 256;
            double r = 1.0 + (double)k * 5.9604644775390625e-08;  // 2^-24
            float cf = (float)(r * c0), sf = (float)(r * s0);
            double e = fabs((double)sf * c0 - (double)cf * s0);
            if (e < best) { best = e; bc = cf; bs = sf; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            double ob = __shfl_xor_sync(0xffffffffu, best, o);
            float oc = __shfl_xor_sync(0xffffffffu, bc, o), os = __shfl_xor_sync(0xffffffffu, bs, o);
            if (ob < best || (ob == best && oc < bc)) { best = ob; bc = oc; bs = os; }
        }
        if (g.type == QGT_GATE_RX) { m[0] = bc; m[1] = 0; m[2] = 0; m[3] = -bs; m[4] = 0; m[5] = -bs; m[6] = bc; m[7] = 0; }
        else { m[0] = bc; m[1] = -bs; m[2] = 0; m[3] = 0; m[4] = 0; m[5] = 0; m[6] = bc; m[7] = bs; }
    } else {
        const float r = 0.70710678118654752440f;
        switch (g.type) {
        case QGT_GATE_X: m[0] = 0; m[2] = 1; m[4] = 1; m[6] = 0; break;
        case QGT_GATE_Y: m[0] = 0; m[3] = -1; m[5] = 1; m[6] = 0; break;
        case QGT_GATE_Z: m[6] = -1; break;
        case QGT_GATE_H: m[0] = r; m[2] = r; m[4] = r; m[6] = -r; break;
        case QGT_GATE_S: m[6] = 0; m[7] = inv ? -1.f : 1.f; break;
        case QGT_GATE_T: m[0] = (float)sqrt(2.0 * (double)r * (double)r); m[6] = r; m[7] = inv ? -r : r; break;
        default: break;
        }
    }
    if (lane < 8) coef[8 * c + lane] = m[lane];
}

// Pass renormalisation: for each pass (blockIdx.x) of each point
// (blockIdx.y), G = prod over the pass's coefficient entries of their scales
// |column 0| (FP64), and the pass's designated entry (its last single-qubit
// gate, ren[pass] >= 0) is multiplied by 1 / G, so that every vector leaves
// the pass with the norm it entered with.  Every vector of a pass runs the
// whole pass program, so all of them take the same factor.  One warp per
// pass; runs after prepare32_kernel and before scale_product_kernel (which
// then sees the applied scales).
__global__ void renorm_kernel(float* __restrict__ coef, int coef_stride, const int32_t* __restrict__ ptr,
                              const int32_t* __restrict__ src, const int32_t* __restrict__ ren)
{
    const int k = blockIdx.x, lane = threadIdx.x;
    coef += (int64_t)8 * blockIdx.y * coef_stride;
    const int d = ren[k];
    if (d < 0) return;
    double lg = 0;
    for (int i = ptr[k] + lane; i < ptr[k + 1]; i += 32) {
        const float* m = coef + 8 * src[i];
        const double r2 = (double)m[0] * m[0] + (double)m[1] * m[1] + (double)m[4] * m[4] + (double)m[5] * m[5];
        lg += 0.5 * log(r2);
    }
    for (int o = 16; o > 0; o >>= 1) lg += __shfl_xor_sync(0xffffffffu, lg, o);
    const float f = (float)exp(-lg);
    __syncwarp();
    if (lane < 8) coef[8 * d + lane] *= f;
}

extern "C" int qgt_dev_renorm_passes(float* coef32, int32_t coef_stride, const int32_t* ptr, const int32_t* src,
                                     const int32_t* ren, int32_t npasses, int32_t npoints, void* s)
{
    if (npasses <= 0) return 0;
    if (npoints < 1 || npoints > 65535) return qgt_set_error(QGT_EINVAL, "renorm: bad point count");
    renorm_kernel<<<dim3((unsigned)npasses, (unsigned)npoints), 32, 0, (cudaStream_t)s>>>(coef32, coef_stride, ptr, src, ren);
    return qgt_dev_last_error();
}

// rho[point][m] = prod over groups 0..m of the amplitude scales r = |column 0|
// of the groups' complex64 coefficient entries (FP64 from the exact FP32 values)
__global__ void scale_product_kernel(const float* __restrict__ coef, int coef_stride, const int32_t* __restrict__ ptr,
                                     const int32_t* __restrict__ src, int ngroups, double* __restrict__ rho)
{
    __shared__ double red[32];
    __shared__ double acc;
    coef += (int64_t)8 * blockIdx.x * coef_stride;
    if (threadIdx.x == 0) acc = 0;
    for (int g = 0; g < ngroups; g++) {
        double lg = 0;
        for (int i = ptr[g] + threadIdx.x; i < ptr[g + 1]; i += blockDim.x) {
            const float* m = coef + 8 * src[i];
            const double r2 = (double)m[0] * m[0] + (double)m[1] * m[1] + (double)m[4] * m[4] + (double)m[5] * m[5];
            lg += 0.5 * log(r2);
        }
        for (int o = 16; o > 0; o >>= 1) lg += __shfl_xor_sync(0xffffffffu, lg, o);
        __syncthreads();
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lg;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) acc += red[w];
            rho[(int64_t)blockIdx.x * ngroups + g] = exp(acc);
        }
    }
}

extern "C" int qgt_dev_scale_product(const float* coef32, int32_t coef_stride, const int32_t* ptr, const int32_t* src,
                                     int32_t ngroups, double* rho, int32_t npoints, void* s)
{
    if (npoints < 1 || ngroups < 0) return qgt_set_error(QGT_EINVAL, "scale product: bad arguments");
    if (ngroups == 0) return 0;
    scale_product_kernel<<<npoints, 256, 0, (cudaStream_t)s>>>(coef32, coef_stride, ptr, src, ngroups, rho);
    return qgt_dev_last_error();
}

// combined phase entries of diagonal runs (products formed in FP64)
__global__ void combine_diag_kernel(double* __restrict__ coef, float* __restrict__ coef32, int stride, int base,
                                    const int32_t* __restrict__ ptr, const int32_t* __restrict__ src, int ncomb)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ncomb) return;
    const int64_t off = (int64_t)8 * blockIdx.y * stride;
    for (int t = 0; t < 2; t++) {
        double a0r = 1, a0i = 0, a1r = 1, a1i = 0;
        if (t == 0 && !coef) continue;
        if (t == 1 && !coef32) continue;
        for (int i = ptr[k]; i < ptr[k + 1]; i++) {
            const int64_t e = off + (int64_t)8 * src[i];
            const double p0r = t ? coef32[e] : coef[e], p0i = t ? coef32[e + 1] : coef[e + 1];
            const double p1r = t ? coef32[e + 6] : coef[e + 6], p1i = t ? coef32[e + 7] : coef[e + 7];
            double x = a0r * p0r - a0i * p0i;
            a0i = a0r * p0i + a0i * p0r;
            a0r = x;
            x = a1r * p1r - a1i * p1i;
            a1i = a1r * p1i + a1i * p1r;
            a1r = x;
        }
        const int64_t d = off + (int64_t)8 * (base + k);
        const double m[8] = {a0r, a0i, 0, 0, 0, 0, a1r, a1i};
        for (int i = 0; i < 8; i++) {
            if (t) coef32[d + i] = (float)m[i];
            else coef[d + i] = m[i];
        }
    }
}

extern "C" int qgt_dev_combine_diag(double* coef, float* coef32, int32_t stride, int32_t base, const int32_t* ptr,
                                    const int32_t* src, int32_t ncomb, int32_t npoints, void* s)
{
    if (ncomb <= 0) return 0;
    if (npoints < 1 || npoints > 65535) return qgt_set_error(QGT_EINVAL, "combine: %d points", npoints);
    combine_diag_kernel<<<dim3((ncomb + 127) / 128, npoints), 128, 0, (cudaStream_t)s>>>(coef, coef32, stride, base, ptr,
                                                                                           src, ncomb);
    return qgt_dev_last_error();
}

extern "C" int qgt_dev_prepare32(const qgt_dev_coef_desc_t* d, int32_t ncoef, const double* theta, float* coef,
                                 int32_t npoints, int32_t theta_stride, int32_t coef_stride, void* s)
{
    if (ncoef <= 0) return QGT_OK;
    if (npoints < 1 || npoints > 65535) return qgt_set_error(QGT_EINVAL, "prepare32: %d points", npoints);
    prepare32_kernel<<<dim3((ncoef + 7) / 8, npoints), 256, 0, (cudaStream_t)s>>>(d, ncoef, theta, coef, theta_stride,
                                                                                    coef_stride);
    return qgt_dev_last_error();
}
