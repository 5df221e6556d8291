// qgt_pass.cu -- tile passes: the gate application hot path.
//
// A pass holds a set S of t qubits ("tile bits", always including qubits
// 0..4 so that every tile is a union of 256-byte or larger contiguous
// segments).  One CTA loads the 2^t amplitudes of one tile of one vector into
// shared memory, applies every op of the pass in order (dense 1-qubit gates on
// tile bits, phases / CZ on any qubit, CNOT with the target in the tile) and
// stores the tile back.  Qubits outside S are constant over the tile, so
// diagonal gates and controls on them reduce to per-tile constants.
//
// Derivative states (a4, exact generator insertion): an entry may insert
// (-i/2) G right after one op -- the derivative of exp(-i a G/2) -- so the
// derivative vectors branch from psi inside the pass that holds their gate
// and are then transported by every later pass (in place).
//
// The last pass of a mixed-precision plan also writes the split
// half-precision operands of the tensor-core Gram.
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "../qgt_internal.h"

template <typename R> struct vec2t;
template <> struct vec2t<float> { typedef float2 T; };
template <> struct vec2t<double> { typedef double2 T; };

template <typename T, typename R>
__device__ __forceinline__ T cfma2(R ar, R ai, T x, R br, R bi, T y)
{
    // (ar + i ai) x + (br + i bi) y
    T o;
    o.x = ar * x.x - ai * x.y + br * y.x - bi * y.y;
    o.y = ar * x.y + ai * x.x + br * y.y + bi * y.x;
    return o;
}

template <typename T, typename R>
__device__ __forceinline__ T cscale(T x, R br, R bi)
{
    T o;
    o.x = br * x.x - bi * x.y;
    o.y = br * x.y + bi * x.x;
    return o;
}

// bit value of qubit (local bit lb when in the tile, else from the tile base)
__device__ __forceinline__ int qbit(int l, int lb, int q, uint64_t base)
{
    return lb >= 0 ? (l >> lb) & 1 : (int)((base >> q) & 1);
}

// Gate coefficients are FP64 on the device.  In the complex64 path each one
// is applied as a float-float pair hi + lo (hi = fl(m), lo = fl(m - hi)), so
// the matrix the kernel applies is the FP64 matrix to ~2^-48: rounding the
// matrices to FP32 would instead shift every rotation angle by ~6e-8 rad, an
// error that is coherent across all vectors and shows up directly in Q.
template <typename R>
struct coefpair {
    R h, l;
};

template <typename R>
__device__ __forceinline__ coefpair<R> split_coef(double m)
{
    coefpair<R> c;
    c.h = (R)m;
    c.l = (R)(m - (double)c.h);
    return c;
}

// (a + i b) x + (c + i d) y with float-float coefficients (R = float) or plain FP64
template <typename T, typename R>
__device__ __forceinline__ T cfma2p(const coefpair<R>* m, T x, T y)
{
    T o;
    o.x = m[0].h * x.x - m[1].h * x.y + m[2].h * y.x - m[3].h * y.y;
    o.y = m[0].h * x.y + m[1].h * x.x + m[2].h * y.y + m[3].h * y.x;
    if (sizeof(R) == 4) {
        o.x += m[0].l * x.x - m[1].l * x.y + m[2].l * y.x - m[3].l * y.y;
        o.y += m[0].l * x.y + m[1].l * x.x + m[2].l * y.y + m[3].l * y.x;
    }
    return o;
}

template <typename T, typename R>
__device__ __forceinline__ T cscalep(T x, const coefpair<R>* p)
{
    T o;
    o.x = p[0].h * x.x - p[1].h * x.y;
    o.y = p[0].h * x.y + p[1].h * x.x;
    if (sizeof(R) == 4) {
        o.x += p[0].l * x.x - p[1].l * x.y;
        o.y += p[0].l * x.y + p[1].l * x.x;
    }
    return o;
}

template <typename R>
__device__ void apply_op(const qgt_dev_op_t& op, const double* __restrict__ coef, typename vec2t<R>::T* tile, int TS,
                         uint64_t base)
{
    typedef typename vec2t<R>::T T;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (op.kind == QOP_1Q) {
        const double* m = coef + 8 * op.coef;
        coefpair<R> r0[4], r1[4];
        for (int i = 0; i < 4; i++) { r0[i] = split_coef<R>(__ldg(m + i)); r1[i] = split_coef<R>(__ldg(m + 4 + i)); }
        const int b = op.lb;
        for (int p = tid; p < TS / 2; p += nt) {
            int i0 = ((p >> b) << (b + 1)) | (p & ((1 << b) - 1));
            int i1 = i0 | (1 << b);
            T a0 = tile[i0], a1 = tile[i1];
            tile[i0] = cfma2p<T, R>(r0, a0, a1);
            tile[i1] = cfma2p<T, R>(r1, a0, a1);
        }
    } else if (op.kind == QOP_PHASE) {
        const double* m = coef + 8 * op.coef;
        coefpair<R> p0[2] = {split_coef<R>(__ldg(m + 0)), split_coef<R>(__ldg(m + 1))};
        coefpair<R> p1[2] = {split_coef<R>(__ldg(m + 6)), split_coef<R>(__ldg(m + 7))};
        if (op.lb >= 0) {
            for (int l = tid; l < TS; l += nt) {
                int bit = (l >> op.lb) & 1;
                tile[l] = cscalep<T, R>(tile[l], bit ? p1 : p0);
            }
        } else {
            int bit = (int)((base >> op.q) & 1);
            const coefpair<R>* pp = bit ? p1 : p0;
            if (!(pp[0].h == (R)1 && pp[0].l == (R)0 && pp[1].h == (R)0 && pp[1].l == (R)0))
                for (int l = tid; l < TS; l += nt) tile[l] = cscalep<T, R>(tile[l], pp);
        }
    } else if (op.kind == QOP_CZ) {
        if (op.lb < 0 && op.lb2 < 0) {
            if (((base >> op.q) & 1) && ((base >> op.q2) & 1))
                for (int l = tid; l < TS; l += nt) { T v = tile[l]; v.x = -v.x; v.y = -v.y; tile[l] = v; }
        } else {
            for (int l = tid; l < TS; l += nt) {
                if (qbit(l, op.lb, op.q, base) & qbit(l, op.lb2, op.q2, base)) {
                    T v = tile[l]; v.x = -v.x; v.y = -v.y; tile[l] = v;
                }
            }
        }
    } else if (op.kind == QOP_CNOT) {
        const int b = op.lb;
        if (op.lb2 < 0 && !((base >> op.q2) & 1)) return;  // control outside the tile and 0
        for (int p = tid; p < TS / 2; p += nt) {
            int i0 = ((p >> b) << (b + 1)) | (p & ((1 << b) - 1));
            if (op.lb2 >= 0 && !((i0 >> op.lb2) & 1)) continue;
            int i1 = i0 | (1 << b);
            T t0 = tile[i0];
            tile[i0] = tile[i1];
            tile[i1] = t0;
        }
    } else if (op.kind == QOP_SWAP) {
        const int a = op.lb, b = op.lb2;
        for (int l = tid; l < TS; l += nt) {
            if (((l >> a) & 1) && !((l >> b) & 1)) {
                int j = l ^ (1 << a) ^ (1 << b);
                T t0 = tile[l];
                tile[l] = tile[j];
                tile[j] = t0;
            }
        }
    }
}

// (-i/2) G after the op of a parameterised rotation (exact: swaps, signs, x0.5)
template <typename R>
__device__ void apply_generator(const qgt_dev_op_t& op, typename vec2t<R>::T* tile, int TS, uint64_t base)
{
    typedef typename vec2t<R>::T T;
    const int tid = threadIdx.x, nt = blockDim.x;
    const R h = (R)0.5;
    if (op.gen == QGEN_X || op.gen == QGEN_Y) {
        const int b = op.lb;
        for (int p = tid; p < TS / 2; p += nt) {
            int i0 = ((p >> b) << (b + 1)) | (p & ((1 << b) - 1));
            int i1 = i0 | (1 << b);
            T a0 = tile[i0], a1 = tile[i1], o0, o1;
            if (op.gen == QGEN_X) {  // (-i/2) [[0,1],[1,0]]: o0 = -i a1 / 2
                o0.x = h * a1.y; o0.y = -h * a1.x;
                o1.x = h * a0.y; o1.y = -h * a0.x;
            } else {                 // (-i/2) [[0,-i],[i,0]] = [[0,-1/2],[1/2,0]]
                o0.x = -h * a1.x; o0.y = -h * a1.y;
                o1.x = h * a0.x; o1.y = h * a0.y;
            }
            tile[i0] = o0;
            tile[i1] = o1;
        }
    } else if (op.gen == QGEN_Z) {  // diag(-i/2, +i/2)
        for (int l = tid; l < TS; l += nt) {
            int bit = qbit(l, op.lb, op.q, base);
            T v = tile[l], o;
            R sg = bit ? h : -h;  // multiply by i*sg
            o.x = -sg * v.y;
            o.y = sg * v.x;
            tile[l] = o;
        }
    }
}

__device__ __forceinline__ uint64_t scatter_local(int l, int t, const int8_t* l2p)
{
    uint64_t ph = 0;
    for (int b = 0; b < t; b++) ph |= (uint64_t)((l >> b) & 1) << l2p[b];
    return ph;
}

template <typename R>
__global__ void __launch_bounds__(QGT_PASS_THREADS) pass_kernel(const qgt_dev_pass_args_t a)
{
    typedef typename vec2t<R>::T T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* tile = reinterpret_cast<T*>(smem_raw);
    __shared__ int8_t l2p[16];
    const int t = a.tile_bits, TS = 1 << t;
    if (threadIdx.x < 16) l2p[threadIdx.x] = a.local_to_phys[threadIdx.x];
    const qgt_dev_entry_t e = a.entries[blockIdx.y];
    const int pt = blockIdx.z;
    const double* coef = a.coef + (int64_t)8 * pt * a.coef_stride;
    // physical base of this tile: scatter blockIdx.x over the qubits outside S
    uint64_t base = 0;
    {
        uint32_t rest = blockIdx.x;
        for (int q = 0; q < a.n; q++)
            if (!((a.tile_mask >> q) & 1)) { base |= (uint64_t)(rest & 1u) << q; rest >>= 1; }
    }
    __syncthreads();
    const T* src = reinterpret_cast<const T*>(a.V) + pt * a.point_stride + (int64_t)e.src_row * a.N;
    for (int l = threadIdx.x; l < TS; l += blockDim.x) {
        uint64_t ph = base | scatter_local(l, t, l2p);
        T v;
        if (e.flags & QENT_SRC_ZERO) { v.x = (ph == 0) ? (R)1 : (R)0; v.y = (R)0; }
        else v = src[ph];
        tile[l] = v;
    }
    __syncthreads();
    for (int j = 0; j < a.nops; j++) {
        qgt_dev_op_t op = a.ops[j];
        apply_op<R>(op, coef, tile, TS, base);
        __syncthreads();
        if (j == e.spawn_op) {
            apply_generator<R>(op, tile, TS, base);
            __syncthreads();
        }
    }
    T* dst = reinterpret_cast<T*>(a.V) + pt * a.point_stride + (int64_t)e.dst_row * a.N;
    float vmax = 0.f;
    for (int l = threadIdx.x; l < TS; l += blockDim.x) {
        uint64_t ph = base | scatter_local(l, t, l2p);
        T v = tile[l];
        if (e.flags & QENT_STORE_V) dst[ph] = v;
        if (e.flags & QENT_ROWMAX) vmax = fmaxf(vmax, sqrtf((float)(v.x * v.x + v.y * v.y)));
        if (e.flags & QENT_STORE_SPLIT) {
            float xr = (float)v.x * a.split_scale, xi = (float)v.y * a.split_scale;
            int64_t at = (int64_t)e.split_row * a.split_ld + (int64_t)ph;
            const int64_t ps = a.split_plane_stride;
            if (a.split_bf16) {
                __nv_bfloat16* s = reinterpret_cast<__nv_bfloat16*>(a.split);
                __nv_bfloat16 rh = __float2bfloat16_rn(xr), ih = __float2bfloat16_rn(xi);
                s[at] = rh;
                s[ps + at] = __float2bfloat16_rn(xr - __bfloat162float(rh));
                s[2 * ps + at] = ih;
                s[3 * ps + at] = __float2bfloat16_rn(xi - __bfloat162float(ih));
            } else {
                __half* s = reinterpret_cast<__half*>(a.split);
                __half rh = __float2half_rn(xr), ih = __float2half_rn(xi);
                s[at] = rh;
                s[ps + at] = __float2half_rn(xr - __half2float(rh));
                s[2 * ps + at] = ih;
                s[3 * ps + at] = __float2half_rn(xi - __half2float(ih));
            }
        }
    }
    if (e.flags & QENT_ROWMAX) {
        // block max -> one atomicMax per CTA (non-negative floats order like their bit patterns)
        __shared__ float red[QGT_PASS_THREADS / 32];
        for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = vmax;
        __syncthreads();
        if (threadIdx.x == 0) {
            float m = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = fmaxf(m, red[w]);
            atomicMax(a.rowmax + (int64_t)pt * a.rowmax_stride + e.dst_row, __float_as_uint(m));
        }
    }
}

extern "C" int qgt_dev_pass(const qgt_dev_pass_args_t* a, int fp64, void* stream)
{
    if (a->nentries <= 0) return 0;
    int TS = 1 << a->tile_bits;
    int64_t ntiles = (int64_t)1 << (a->n - a->tile_bits);
    const int np = a->npoints > 0 ? a->npoints : 1;
    if (a->nentries > 65535 || ntiles > 0x7fffffff || np > 65535)
        return qgt_set_error(-1, "pass: %d entries / %lld tiles / %d points exceed the grid", a->nentries,
                             (long long)ntiles, np);
    dim3 grid((unsigned)ntiles, (unsigned)a->nentries, (unsigned)np);
    size_t smem = (size_t)TS * (fp64 ? sizeof(double2) : sizeof(float2));
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    // the attribute is set once per process, outside any stream capture (the
    // first launch of every plan runs eagerly)
    static int attr_set[2] = {0, 0};
    const int maxsmem = 1 << 16;
    if (!attr_set[fp64 ? 1 : 0]) {
        e = fp64 ? cudaFuncSetAttribute(pass_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsmem)
                 : cudaFuncSetAttribute(pass_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsmem);
        if (e == cudaSuccess) attr_set[fp64 ? 1 : 0] = 1;
    }
    if (smem > (size_t)maxsmem) return qgt_set_error(-1, "pass: tile of %d amplitudes exceeds shared memory", TS);
    if (e == cudaSuccess) {
        if (fp64) pass_kernel<double><<<grid, QGT_PASS_THREADS, smem, s>>>(*a);
        else pass_kernel<float><<<grid, QGT_PASS_THREADS, smem, s>>>(*a);
    }
    if (e != cudaSuccess) return qgt_set_error(-6, "pass: %s", cudaGetErrorString(e));
    return qgt_dev_last_error();
}
