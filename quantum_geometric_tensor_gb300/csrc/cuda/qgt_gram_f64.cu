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
                                                       int64_t kchunk, double2* __restrict__ part, int64_t point_stride)
{
    V += blockIdx.z * point_stride;   // parameter point
    part += (int64_t)blockIdx.z * gridDim.y * gridDim.x * (GT * GT);
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
    part += (int64_t)blockIdx.y * nsplit * ntp * (GT * GT);
    HG += (int64_t)blockIdx.y * rows * rows;
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
                                int32_t npoints, int64_t point_stride, void* stream)
{
    if (npoints < 1 || npoints > 65535) return qgt_set_error(-1, "gram_f64: %d points", npoints);
    int nt = (rows + GT - 1) / GT;
    int ntp = nt * (nt + 1) / 2;
    int64_t kchunk = (N + nsplit - 1) / nsplit;
    kchunk = (kchunk + KT - 1) / KT * KT;
    int ns = (int)((N + kchunk - 1) / kchunk);
    cudaStream_t s = (cudaStream_t)stream;
    gram_f64_kernel<<<dim3(ntp, ns, npoints), 256, 0, s>>>((const double2*)V, N, rows, nt, kchunk, (double2*)part,
                                                           point_stride);
    int rc = qgt_dev_last_error();
    if (rc) return rc;
    int64_t cnt = (int64_t)rows * rows;
    gram_f64_reduce_kernel<<<dim3((unsigned)((cnt + 255) / 256), npoints), 256, 0, s>>>((const double2*)part, rows, nt,
                                                                                        ntp, ns, (double2*)HG);
    return qgt_dev_last_error();
}

// ---------------------------------------------------------------------------
// Small Gram: rows <= 8 (a few vectors per point, e.g. psi and two derivative
// slots of a Berry-curvature point).  Memory-bound: every thread reads its
// amplitudes of all rows once and keeps the rows (rows + 1) / 2 sums in FP64
// registers (complex128 rows: FP64 products; complex64 rows: FP32 sums of
// short blocks, gram_small32_kernel below).  Block sums go
// to part[point][split][pair]; a second kernel adds the splits and writes the
// Hermitian HG of each point.
// ---------------------------------------------------------------------------
template <typename T, int ROWS>
__global__ void __launch_bounds__(256) gram_small_kernel(const T* __restrict__ V, int64_t N, int64_t point_stride,
                                                         int skip, double2* __restrict__ part)
{
    constexpr int NP = ROWS * (ROWS + 1) / 2;
    __shared__ double2 red[8][NP];
    V += blockIdx.y * point_stride;
    double2 acc[NP];
#pragma unroll
    for (int p = 0; p < NP; p++) acc[p] = make_double2(0, 0);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x) {
        double xr[ROWS], xi[ROWS];
#pragma unroll
        for (int r = 0; r < ROWS; r++) {
            T v = V[(int64_t)(r + (r > 0 ? skip : 0)) * N + k];
            xr[r] = (double)v.x;
            xi[r] = (double)v.y;
        }
        int p = 0;
#pragma unroll
        for (int i = 0; i < ROWS; i++)
#pragma unroll
            for (int j = i; j < ROWS; j++, p++) {
                // conj(x_i) x_j
                acc[p].x += xr[i] * xr[j] + xi[i] * xi[j];
                acc[p].y += xr[i] * xi[j] - xi[i] * xr[j];
            }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int p = 0; p < NP; p++) {
        for (int o = 16; o > 0; o >>= 1) {
            acc[p].x += __shfl_xor_sync(0xffffffffu, acc[p].x, o);
            acc[p].y += __shfl_xor_sync(0xffffffffu, acc[p].y, o);
        }
        if (lane == 0) red[warp][p] = acc[p];
    }
    __syncthreads();
    if (threadIdx.x < NP) {
        double2 s = make_double2(0, 0);
        for (int w = 0; w < 8; w++) { s.x += red[w][threadIdx.x].x; s.y += red[w][threadIdx.x].y; }
        part[((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * NP + threadIdx.x] = s;
    }
}

// complex64 rows: the products and sums of SB consecutive grid-stride
// amplitudes of a thread run in FP32 (FMA), and each block sum is added to an
// FP64 accumulator.  FP64 work drops SB-fold (GB300 issues about one FP64 FMA
// per 64 FP32 FMAs), which leaves the kernel bound by HBM; the rounding of a
// 32-term FP32 block adds about 2^-24 sqrt(32 / N) to an entry of unit
// vectors, far below the complex64 amplitudes' own error.
template <int ROWS, int SB>
__global__ void __launch_bounds__(256) gram_small32_kernel(const float2* __restrict__ V, int64_t N, int64_t point_stride,
                                                           int skip, double2* __restrict__ part)
{
    constexpr int NP = ROWS * (ROWS + 1) / 2;
    __shared__ double2 red[8][NP];
    V += blockIdx.y * point_stride;
    double2 acc[NP];
#pragma unroll
    for (int p = 0; p < NP; p++) acc[p] = make_double2(0, 0);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k0 < N; k0 += SB * stride) {
        float2 sb[NP];
#pragma unroll
        for (int p = 0; p < NP; p++) sb[p] = make_float2(0.f, 0.f);
        constexpr int UN = ROWS <= 4 ? 4 : 1;   /* loads in flight vs registers of the sums */
#pragma unroll UN
        for (int t = 0; t < SB; t++) {
            const int64_t k = k0 + t * stride;
            if (k < N) {
                float2 x[ROWS];
#pragma unroll
                for (int r = 0; r < ROWS; r++) x[r] = V[(int64_t)(r + (r > 0 ? skip : 0)) * N + k];
                int p = 0;
#pragma unroll
                for (int i = 0; i < ROWS; i++)
#pragma unroll
                    for (int j = i; j < ROWS; j++, p++) {
                        sb[p].x = fmaf(x[i].x, x[j].x, fmaf(x[i].y, x[j].y, sb[p].x));
                        sb[p].y = fmaf(x[i].x, x[j].y, fmaf(-x[i].y, x[j].x, sb[p].y));
                    }
            }
        }
#pragma unroll
        for (int p = 0; p < NP; p++) {
            acc[p].x += (double)sb[p].x;
            acc[p].y += (double)sb[p].y;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int p = 0; p < NP; p++) {
        for (int o = 16; o > 0; o >>= 1) {
            acc[p].x += __shfl_xor_sync(0xffffffffu, acc[p].x, o);
            acc[p].y += __shfl_xor_sync(0xffffffffu, acc[p].y, o);
        }
        if (lane == 0) red[warp][p] = acc[p];
    }
    __syncthreads();
    if (threadIdx.x < NP) {
        double2 s = make_double2(0, 0);
        for (int w = 0; w < 8; w++) { s.x += red[w][threadIdx.x].x; s.y += red[w][threadIdx.x].y; }
        part[((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * NP + threadIdx.x] = s;
    }
}

// HG (rows x rows) of each point from the splits' sums over the rows read
// (row 1 skipped when skip = 1: its entries are written as zeros)
__global__ void gram_small_reduce_kernel(const double2* __restrict__ part, int rows, int skip, int nsplit,
                                         double2* __restrict__ HG)
{
    const int rr = rows - skip;   // rows read
    const int np = rr * (rr + 1) / 2;
    HG += (int64_t)blockIdx.x * rows * rows;
    if (skip)
        for (int t = threadIdx.x; t < rows; t += blockDim.x) {
            HG[rows + t] = make_double2(0, 0);
            HG[(int64_t)t * rows + 1] = make_double2(0, 0);
        }
    const int p = threadIdx.x;
    if (p >= np) return;
    part += (int64_t)blockIdx.x * nsplit * np;
    int i = 0, rem = p;
    while (rem >= rr - i) { rem -= rr - i; i++; }
    int j = i + rem;
    double2 s = make_double2(0, 0);
    for (int sp = 0; sp < nsplit; sp++) { s.x += part[(int64_t)sp * np + p].x; s.y += part[(int64_t)sp * np + p].y; }
    if (i > 0) i += skip;
    if (j > 0) j += skip;
    HG[(int64_t)i * rows + j] = s;
    HG[(int64_t)j * rows + i] = make_double2(s.x, -s.y);
}

template <typename T>
static void gram_small_launch(const void* V, int64_t N, int rows, int skip, int nsplit, double2* part, int npoints,
                              int64_t ps, cudaStream_t s)
{
    dim3 g((unsigned)nsplit, (unsigned)npoints);
    const T* v = (const T*)V;
    switch (rows) {
    case 1: gram_small_kernel<T, 1><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 2: gram_small_kernel<T, 2><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 3: gram_small_kernel<T, 3><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 4: gram_small_kernel<T, 4><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 5: gram_small_kernel<T, 5><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 6: gram_small_kernel<T, 6><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 7: gram_small_kernel<T, 7><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    default: gram_small_kernel<T, 8><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    }
}

static void gram_small32_launch(const void* V, int64_t N, int rows, int skip, int nsplit, double2* part, int npoints,
                                int64_t ps, cudaStream_t s)
{
    dim3 g((unsigned)nsplit, (unsigned)npoints);
    const float2* v = (const float2*)V;
    switch (rows) {
    case 1: gram_small32_kernel<1, 32><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 2: gram_small32_kernel<2, 32><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 3: gram_small32_kernel<3, 32><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 4: gram_small32_kernel<4, 32><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 5: gram_small32_kernel<5, 32><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 6: gram_small32_kernel<6, 32><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    case 7: gram_small32_kernel<7, 32><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    default: gram_small32_kernel<8, 32><<<g, 256, 0, s>>>(v, N, ps, skip, part); break;
    }
}

extern "C" int qgt_dev_gram_small(const void* V, int64_t N, int32_t rows, int32_t skip_row1, int32_t fp64, double* part,
                                  int32_t nsplit, double* HG, int32_t npoints, int64_t point_stride, void* stream)
{
    if (rows < 1 || rows > 8 || nsplit < 1 || nsplit > 65535 || npoints < 1 || npoints > 65535 ||
        (skip_row1 != 0 && skip_row1 != 1) || (skip_row1 && rows < 2))
        return qgt_set_error(-1, "gram_small: %d rows (skip %d), %d splits, %d points", rows, skip_row1, nsplit,
                             npoints);
    cudaStream_t s = (cudaStream_t)stream;
    const int rr = rows - skip_row1;
    if (fp64) gram_small_launch<double2>(V, N, rr, skip_row1, nsplit, (double2*)part, npoints, point_stride, s);
    else gram_small32_launch(V, N, rr, skip_row1, nsplit, (double2*)part, npoints, point_stride, s);
    int rc = qgt_dev_last_error();
    if (rc) return rc;
    gram_small_reduce_kernel<<<npoints, 64, 0, s>>>((const double2*)part, rows, skip_row1, nsplit, (double2*)HG);
    return qgt_dev_last_error();
}

// ---------------------------------------------------------------------------
// Overlaps <V + a_off[k] | V + b_off[k]> of rows of N amplitudes (offsets in
// amplitudes), FP64 sums (complex64 rows: FP32 sums of 32-term blocks added in
// FP64): Berry phases around loops and plaquette links on
// parameter lattices.  Pair k is split over nchunk CTAs (block k * nchunk + c
// sums the amplitudes [c len, (c + 1) len)); part[k * nchunk + c] receives
// the partial sums, which the caller adds in a fixed order.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) overlap_kernel(const T* __restrict__ V, int64_t N, int64_t len,
                                                      int32_t nchunk, const int64_t* __restrict__ a_off,
                                                      const int64_t* __restrict__ b_off, double2* __restrict__ part)
{
    __shared__ double2 red[8];
    const int64_t k = blockIdx.x / nchunk, c = blockIdx.x % nchunk;
    const T* a = V + a_off[k];
    const T* b = V + b_off[k];
    const int64_t lo = c * len, hi = lo + len < N ? lo + len : N;
    double re = 0, im = 0;
    if constexpr (sizeof(T) == 16) {
        for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
            const T x = a[i], y = b[i];
            re += (double)x.x * y.x + (double)x.y * y.y;
            im += (double)x.x * y.y - (double)x.y * y.x;
        }
    } else {
        // complex64: FP32 sums of 32 consecutive strided terms, added in FP64 (as in gram_small32_kernel)
        for (int64_t i0 = lo + threadIdx.x; i0 < hi; i0 += 32 * (int64_t)blockDim.x) {
            float sr = 0.f, si = 0.f;
#pragma unroll 8
            for (int t = 0; t < 32; t++) {
                const int64_t i = i0 + t * (int64_t)blockDim.x;
                if (i < hi) {
                    const T x = a[i], y = b[i];
                    sr = fmaf(x.x, y.x, fmaf(x.y, y.y, sr));
                    si = fmaf(x.x, y.y, fmaf(-x.y, y.x, si));
                }
            }
            re += (double)sr;
            im += (double)si;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_double2(re, im);
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 t = make_double2(0, 0);
        for (int w = 0; w < 8; w++) { t.x += red[w].x; t.y += red[w].y; }
        part[blockIdx.x] = t;
    }
}

extern "C" int qgt_dev_overlaps(const void* V, int32_t fp64, int64_t N, const int64_t* a_off, const int64_t* b_off,
                                int32_t n, int32_t nchunk, double* part, void* stream)
{
    if (n <= 0) return 0;
    if (N <= 0 || nchunk <= 0 || (int64_t)n * nchunk > 0x7fffffff)
        return qgt_set_error(-1, "overlaps: %d pairs x %d chunks outside the grid", n, nchunk);
    const int64_t len = (N + nchunk - 1) / nchunk;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned grid = (unsigned)((int64_t)n * nchunk);
    if (fp64) overlap_kernel<double2><<<grid, 256, 0, s>>>((const double2*)V, N, len, nchunk, a_off, b_off, (double2*)part);
    else overlap_kernel<float2><<<grid, 256, 0, s>>>((const float2*)V, N, len, nchunk, a_off, b_off, (double2*)part);
    return qgt_dev_last_error();
}

// ---------------------------------------------------------------------------
// Closed-form Berry map.  With theta_a and theta_b each driving one rotation
// R(t) = cos(t/2) I - i sin(t/2) G (G^2 = I), the circuit's state is
//     psi(ta, tb) = sum_{r,s in {0,1}} c_r(ta) c_s(tb) v_rs,  c(t) = (cos(t/2), -i sin(t/2)),
// v_rs the circuit with G_a^r, G_b^s in place of the two rotations; so every
// inner product among psi, d_a psi, d_b psi is a bilinear form in the 4 x 4
// Gram K = <v|v>, and the whole G x G lattice of Omega_ab = Im Q_ab follows
// from K.  The four v_rs come from the states at (ta, tb) in {0, pi}^2:
//     psi(0,0) = v_00, psi(pi,0) = -i v_10, psi(0,pi) = -i v_01, psi(pi,pi) = -v_11.
// part holds, per circuit, the partial sums of the 10 overlaps <psi_i|psi_j>
// (i <= j, in the order (0,0) (0,1) (0,2) (0,3) (1,1) (1,2) (1,3) (2,2) (2,3)
// (3,3)) over nchunk ranges; maps[circuit][x][y] = Omega at
// (2 pi x / G, 2 pi y / G).  One CTA per circuit.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) berry_closed_kernel(const double2* __restrict__ part, int nchunk, int G,
                                                           double* __restrict__ maps)
{
    __shared__ double Kr[4][4], Ki[4][4];
    const int m = blockIdx.x;
    if (threadIdx.x < 10) {
        const int pr = threadIdx.x;
        const int ii[10] = {0, 0, 0, 0, 1, 1, 1, 2, 2, 3}, jj[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};
        const double2* pp = part + ((int64_t)m * 10 + pr) * nchunk;
        double re = 0, im = 0;
        for (int c = 0; c < nchunk; c++) { re += pp[c].x; im += pp[c].y; }
        // <v_i|v_j> = conj(f_i) f_j <psi_i|psi_j> with v_i = f_i psi_i, f = (1, i, i, -1)
        const double fr[4] = {1, 0, 0, -1}, fi[4] = {0, 1, 1, 0};
        const int i = ii[pr], j = jj[pr];
        const double ar = fr[i] * fr[j] + fi[i] * fi[j], ai = fr[i] * fi[j] - fi[i] * fr[j];   // conj(f_i) f_j
        const double kr = ar * re - ai * im, ki = ar * im + ai * re;
        Kr[i][j] = kr; Ki[i][j] = ki;
        Kr[j][i] = kr; Ki[j][i] = -ki;
    }
    __syncthreads();
    const double step = 6.283185307179586476925 / (double)G;
    for (int t = threadIdx.x; t < G * G; t += blockDim.x) {
        const int x = t / G, y = t % G;
        double sa, ca, sb, cb;
        sincos(0.5 * step * x, &sa, &ca);
        sincos(0.5 * step * y, &sb, &cb);
        // coefficient vectors over (r, s), index r + 2 s: c = (cos, -i sin), c' = (-sin / 2, -i cos / 2)
        const double car[2] = {ca, 0}, cai[2] = {0, -sa}, dar[2] = {-0.5 * sa, 0}, dai[2] = {0, -0.5 * ca};
        const double cbr[2] = {cb, 0}, cbi[2] = {0, -sb}, dbr[2] = {-0.5 * sb, 0}, dbi[2] = {0, -0.5 * cb};
        double pr_[4], pi_[4], qr[4], qi[4], wr[4], wi[4];   // psi, d_a psi, d_b psi coefficients
        for (int k = 0; k < 4; k++) {
            const int r = k & 1, s = k >> 1;
            pr_[k] = car[r] * cbr[s] - cai[r] * cbi[s];
            pi_[k] = car[r] * cbi[s] + cai[r] * cbr[s];
            qr[k] = dar[r] * cbr[s] - dai[r] * cbi[s];
            qi[k] = dar[r] * cbi[s] + dai[r] * cbr[s];
            wr[k] = car[r] * dbr[s] - cai[r] * dbi[s];
            wi[k] = car[r] * dbi[s] + cai[r] * dbr[s];
        }
        // x^H K y
        auto form = [&](const double* xr, const double* xi, const double* yr, const double* yi, double* outr, double* outi) {
            double sr = 0, si = 0;
            for (int i = 0; i < 4; i++) {
                double tr = 0, ti = 0;   // (K y)_i
                for (int j = 0; j < 4; j++) {
                    tr += Kr[i][j] * yr[j] - Ki[i][j] * yi[j];
                    ti += Kr[i][j] * yi[j] + Ki[i][j] * yr[j];
                }
                sr += xr[i] * tr + xi[i] * ti;   // conj(x_i) (K y)_i
                si += xr[i] * ti - xi[i] * tr;
            }
            *outr = sr;
            *outi = si;
        };
        double sn, sni, Ar, Ai, Br, Bi, Cr, Ci;
        form(pr_, pi_, pr_, pi_, &sn, &sni);
        form(qr, qi, wr, wi, &Ar, &Ai);     // <d_a psi|d_b psi>
        form(qr, qi, pr_, pi_, &Br, &Bi);   // <d_a psi|psi>
        form(pr_, pi_, wr, wi, &Cr, &Ci);   // <psi|d_b psi>
        const double inv = 1.0 / sn;
        // Im(A / s - B C / s^2)
        maps[(int64_t)m * G * G + t] = Ai * inv - (Br * Ci + Bi * Cr) * inv * inv;
    }
}

extern "C" int qgt_dev_berry_closed(const double* part, int32_t nchunk, int32_t ncirc, int32_t G, double* maps,
                                    void* stream)
{
    if (ncirc <= 0) return 0;
    if (G < 1 || G > 1024 || nchunk < 1) return qgt_set_error(-1, "berry closed form: grid %d, %d chunks", G, nchunk);
    berry_closed_kernel<<<ncirc, 256, 0, (cudaStream_t)stream>>>((const double2*)part, nchunk, G, maps);
    return qgt_dev_last_error();
}
