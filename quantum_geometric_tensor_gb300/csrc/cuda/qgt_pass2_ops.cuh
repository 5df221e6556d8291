// qgt_pass2_ops.cuh -- the gate arithmetic of the register-resident tile passes: butterflies on
// register bits, warp-shuffle gates on lane bits, phases, CNOTs and the exact generator insertions.
// Shared by the program interpreter (qgt_pass2.cu) and the straight-line pass kernels that the
// host generates per pass program and compiles at plan creation (qgt_jit.c, qgt_jit_rt.cu), so
// that both paths do the same arithmetic.  Needs float2 / double2, uint32_t, uint64_t and the
// QGEN_* generator codes.
#ifndef QGT_PASS2_OPS_CUH
#define QGT_PASS2_OPS_CUH

template <typename R> struct v2of;
template <> struct v2of<float> { typedef float2 T; };
template <> struct v2of<double> { typedef double2 T; };

// role-encoded bit: 0..4 lane bit, 8 + i reg bit i, 16 + w warp bit w, 32 outside the tile (physical qubit q)
#define RL_REG 8
#define RL_WARP 16
#define RL_OUT 32

template <typename T, typename R>
struct Cf {
    R m[8];
};

template <typename R>
__device__ __forceinline__ void load_coef(const void* tab, int idx, R* m)
{
    const R* t = reinterpret_cast<const R*>(tab) + 8 * idx;
#pragma unroll
    for (int i = 0; i < 8; i++) m[i] = __ldg(t + i);
}

template <typename T, typename R>
__device__ __forceinline__ T cm(R ar, R ai, T x)
{
    T o;
    o.x = ar * x.x - ai * x.y;
    o.y = ar * x.y + ai * x.x;
    return o;
}

template <typename T, typename R>
__device__ __forceinline__ T cmad2(const R* m, T x, T y)  // (m0 + i m1) x + (m2 + i m3) y
{
    T o;
    o.x = m[0] * x.x - m[1] * x.y + m[2] * y.x - m[3] * y.y;
    o.y = m[0] * x.y + m[1] * x.x + m[2] * y.y + m[3] * y.x;
    return o;
}

template <typename T, typename R>
__device__ __forceinline__ T rmad2(R a, T x, R b, T y)  // real a x + b y
{
    T o;
    o.x = a * x.x + b * y.x;
    o.y = a * x.y + b * y.y;
    return o;
}

// complex64: packed FP32x2 arithmetic (one instruction per two lanes of a
// complex number); per component the same rounding as fmaf
template <>
__device__ __forceinline__ float2 rmad2<float2, float>(float a, float2 x, float b, float2 y)
{
    return __ffma2_rn(make_float2(a, a), x, __fmul2_rn(make_float2(b, b), y));
}

template <>
__device__ __forceinline__ float2 cmad2<float2, float>(const float* m, float2 x, float2 y)
{
    // (m0 + i m1) x + (m2 + i m3) y with i z = (-z.y, z.x)
    const float2 xs = make_float2(-x.y, x.x), ys = make_float2(-y.y, y.x);
    float2 o = __fmul2_rn(make_float2(m[3], m[3]), ys);
    o = __ffma2_rn(make_float2(m[2], m[2]), y, o);
    o = __ffma2_rn(make_float2(m[1], m[1]), xs, o);
    return __ffma2_rn(make_float2(m[0], m[0]), x, o);
}

// real a x + y
template <typename T, typename R>
__device__ __forceinline__ T fma_s(R a, T x, T y)
{
    T o;
    o.x = a * x.x + y.x;
    o.y = a * x.y + y.y;
    return o;
}
template <>
__device__ __forceinline__ float2 fma_s<float2, float>(float a, float2 x, float2 y)
{
    return __ffma2_rn(make_float2(a, a), x, y);
}

// (pr + i pi) x
template <typename T, typename R>
__device__ __forceinline__ T cmul_s(R pr, R pi, T x)
{
    T o;
    o.x = pr * x.x - pi * x.y;
    o.y = pr * x.y + pi * x.x;
    return o;
}
template <>
__device__ __forceinline__ float2 cmul_s<float2, float>(float pr, float pi, float2 x)
{
    return __ffma2_rn(make_float2(pr, pr), x, __fmul2_rn(make_float2(pi, pi), make_float2(-x.y, x.x)));
}

template <typename T>
__device__ __forceinline__ T shfl_x(T v, int mask);
template <>
__device__ __forceinline__ float2 shfl_x<float2>(float2 v, int mask)
{
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, mask), __shfl_xor_sync(0xffffffffu, v.y, mask));
}
template <>
__device__ __forceinline__ double2 shfl_x<double2>(double2 v, int mask)
{
    return make_double2(__shfl_xor_sync(0xffffffffu, v.x, mask), __shfl_xor_sync(0xffffffffu, v.y, mask));
}

// ---- butterflies on a register bit ----
template <int RI, int NR, bool real, typename T, typename R>
__device__ __forceinline__ void u_reg(T* v, const R* m)
{
#pragma unroll
    for (int j = 0; j < NR; j++) {
        if (j & (1 << RI)) continue;
        const int k = j | (1 << RI);
        T a0 = v[j], a1 = v[k];
        if (real) {
            v[j] = rmad2<T, R>(m[0], a0, m[2], a1);
            v[k] = rmad2<T, R>(m[4], a0, m[6], a1);
        } else {
            v[j] = cmad2<T, R>(m, a0, a1);
            v[k] = cmad2<T, R>(m + 4, a0, a1);
        }
    }
}

// tangent-form rotation [[1, m2], [m4, 1]]: one multiply-add per component
template <int RI, int NR, typename T, typename R>
__device__ __forceinline__ void tan_reg(T* v, R m2, R m4)
{
#pragma unroll
    for (int j = 0; j < NR; j++) {
        if (j & (1 << RI)) continue;
        const int k = j | (1 << RI);
        const T a0 = v[j], a1 = v[k];
        v[j] = fma_s<T, R>(m2, a1, a0);
        v[k] = fma_s<T, R>(m4, a0, a1);
    }
}

// cotangent form [[m0, -SG], [SG, m6]], SG = +1 or -1
template <int RI, int NR, int SG, typename T, typename R>
__device__ __forceinline__ void cot_reg(T* v, R m0, R m6)
{
#pragma unroll
    for (int j = 0; j < NR; j++) {
        if (j & (1 << RI)) continue;
        const int k = j | (1 << RI);
        const T a0 = v[j], a1 = v[k];
        T n;
        if (SG > 0) {
            n.x = -a1.x;
            n.y = -a1.y;
            v[j] = fma_s<T, R>(m0, a0, n);
            v[k] = fma_s<T, R>(m6, a1, a0);
        } else {
            n.x = -a0.x;
            n.y = -a0.y;
            v[j] = fma_s<T, R>(m0, a0, a1);
            v[k] = fma_s<T, R>(m6, a1, n);
        }
    }
}

template <int RI, int NR, typename T, typename R>
__device__ __forceinline__ void phase_reg(T* v, const R* m)
{
#pragma unroll
    for (int j = 0; j < NR; j++) v[j] = (j & (1 << RI)) ? cm<T, R>(m[6], m[7], v[j]) : cm<T, R>(m[0], m[1], v[j]);
}

// CNOT with reg target RI, control given by a per-register predicate mask (bit j of cmask)
template <int RI, int NR, typename T>
__device__ __forceinline__ void cnot_reg(T* v, uint32_t cmask)
{
#pragma unroll
    for (int j = 0; j < NR; j++) {
        if (j & (1 << RI)) continue;
        const int k = j | (1 << RI);
        if ((cmask >> j) & 1u) { T t = v[j]; v[j] = v[k]; v[k] = t; }
    }
}

// (-i/2) X or (-i/2) Y on reg bit RI (exact)
template <int RI, int NR, typename T, typename R>
__device__ __forceinline__ void gen_reg(T* v, int gen)
{
    const R h = (R)0.5;
#pragma unroll
    for (int j = 0; j < NR; j++) {
        if (j & (1 << RI)) continue;
        const int k = j | (1 << RI);
        T a0 = v[j], a1 = v[k], o0, o1;
        if (gen == QGEN_X) { o0.x = h * a1.y; o0.y = -h * a1.x; o1.x = h * a0.y; o1.y = -h * a0.x; }
        else { o0.x = -h * a1.x; o0.y = -h * a1.y; o1.x = h * a0.x; o1.y = h * a0.y; }
        v[j] = o0;
        v[k] = o1;
    }
}

#define RB_SWITCH(ri, CALL)                         \
    switch (ri) {                                   \
    case 0: CALL(0); break;                         \
    case 1: CALL(1); break;                         \
    case 2: CALL(2); break;                         \
    case 3: CALL(3); break;                         \
    default: if (RB > 4) { CALL(4 % RB); } break;   \
    }

// one single-qubit gate on register bit RI; real rotations in tangent form
// [[1, -t], [t, 1]] or [[k, -g], [g, k]] (g = +-1) take the one-multiply-add
// paths (the form is uniform per CTA: one coefficient table per point)
template <int RI, int NR, typename T, typename R>
__device__ __forceinline__ void gate_reg(T* v, const R* m, bool real)
{
    const bool tanf = real && m[0] == (R)1 && m[6] == (R)1;
    const bool cotf = real && !tanf && m[2] == -m[4] && (m[4] == (R)1 || m[4] == (R)-1);
    if (tanf) tan_reg<RI, NR, T, R>(v, m[2], m[4]);
    else if (cotf && m[4] > (R)0) cot_reg<RI, NR, 1, T, R>(v, m[0], m[6]);
    else if (cotf) cot_reg<RI, NR, -1, T, R>(v, m[0], m[6]);
    else if (real) u_reg<RI, NR, true, T, R>(v, m);
    else u_reg<RI, NR, false, T, R>(v, m);
}

// the same on lane bit b: v' = c_self v + c_partner w (w = the partner lane's
// amplitude); row 1 of the matrix for the upper lane, row 0 for the lower one
template <int NR, typename T, typename R>
__device__ __forceinline__ void gate_lane(T* v, const R* m, bool real, int b, int lane)
{
    const bool tanf = real && m[0] == (R)1 && m[6] == (R)1;
    const bool cotf = real && !tanf && m[2] == -m[4] && (m[4] == (R)1 || m[4] == (R)-1);
    const int hi = (lane >> b) & 1;
    const R cs0 = hi ? m[6] : m[0], cs1 = hi ? m[7] : m[1];
    const R cp0 = hi ? m[4] : m[2], cp1 = hi ? m[5] : m[3];
    if (tanf) {
        // own + c w
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const T w = shfl_x<T>(v[j], 1 << b);
            v[j] = fma_s<T, R>(cp0, w, v[j]);
        }
    } else if (cotf) {
        // k own + c w with c = -g (lower lane) or +g (upper lane)
#pragma unroll
        for (int j = 0; j < NR; j++) {
            T w = shfl_x<T>(v[j], 1 << b);
            w.x *= cp0;
            w.y *= cp0;
            v[j] = fma_s<T, R>(cs0, v[j], w);
        }
    } else if (real) {
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const T w = shfl_x<T>(v[j], 1 << b);
            v[j] = rmad2<T, R>(cs0, v[j], cp0, w);
        }
    } else {
        const R mm[4] = {cs0, cs1, cp0, cp1};
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const T w = shfl_x<T>(v[j], 1 << b);
            v[j] = cmad2<T, R>(mm, v[j], w);
        }
    }
}

// m (2x2 complex, row-major (re, im) pairs) <- (-i/2) G m for the generator G of a rotation: the
// coefficients of a gate whose derivative vector is spawned there (G commutes with the rotation)
__device__ __forceinline__ void fold_gen(float* m, int gen)
{
    float t[8];
    if (gen == QGEN_Y) {   // (-i/2) Y = [[0, -1/2], [1/2, 0]]
        for (int i = 0; i < 4; i++) { t[i] = -0.5f * m[4 + i]; t[4 + i] = 0.5f * m[i]; }
    } else if (gen == QGEN_X) {   // (-i/2) X = [[0, -i/2], [-i/2, 0]]; -i/2 (a + ib) = b/2 - i a/2
        for (int i = 0; i < 2; i++) {
            t[2 * i] = 0.5f * m[5 + 2 * i];
            t[2 * i + 1] = -0.5f * m[4 + 2 * i];
            t[4 + 2 * i] = 0.5f * m[1 + 2 * i];
            t[5 + 2 * i] = -0.5f * m[2 * i];
        }
    } else {   // (-i/2) Z = diag(-i/2, i/2)
        for (int i = 0; i < 2; i++) {
            t[2 * i] = 0.5f * m[1 + 2 * i];
            t[2 * i + 1] = -0.5f * m[2 * i];
            t[4 + 2 * i] = -0.5f * m[5 + 2 * i];
            t[5 + 2 * i] = 0.5f * m[4 + 2 * i];
        }
    }
    for (int i = 0; i < 8; i++) m[i] = t[i];
}

// bit value of a non-register role for this thread
__device__ __forceinline__ int role_bit(int role, int q, int lane, int warp, uint64_t base)
{
    if (role < RL_REG) return (lane >> role) & 1;
    if (role < RL_OUT) return (warp >> (role - RL_WARP)) & 1;
    return (int)((base >> q) & 1);
}

// per-register mask of "bit is 1" for any role: reg -> pattern over j; other -> all or nothing
template <int NR>
__device__ __forceinline__ uint32_t role_mask(int role, int q, int lane, int warp, uint64_t base)
{
    const uint32_t all = (NR == 32) ? 0xffffffffu : ((1u << NR) - 1u);
    if (role >= RL_REG && role < RL_WARP) {
        const int ri = role - RL_REG;
        uint32_t m = 0;
#pragma unroll
        for (int j = 0; j < NR; j++) m |= (uint32_t)((j >> ri) & 1) << j;
        return m;
    }
    return role_bit(role, q, lane, warp, base) ? all : 0u;
}

// (-i/2) G of a rotation on role `ra` (physical qubit q) for a derivative spawned there, through the
// gate paths with the exact generator matrices (-i/2) X, (-i/2) Y, (-i/2) Z (entries 0, +-1/2)
template <int NR, int RB, typename T, typename R>
__device__ __forceinline__ void spawn_gen_op(T* v, int gen, int ra, int q, int lane, int warp, uint64_t base)
{
    const R h = (R)0.5;
    R gm[8] = {(R)0, (R)0, (R)0, (R)0, (R)0, (R)0, (R)0, (R)0};
    if (gen == QGEN_X) { gm[3] = -h; gm[5] = -h; }
    else if (gen == QGEN_Y) { gm[2] = -h; gm[4] = h; }
    else { gm[1] = -h; gm[7] = h; }
    const bool reg = ra >= RL_REG && ra < RL_WARP;
    if (gen == QGEN_Z) {
        if (reg) {
            const int ri = ra - RL_REG;
#define G_CALL(I) phase_reg<I, NR, T, R>(v, gm)
            RB_SWITCH(ri, G_CALL)
#undef G_CALL
        } else {
            const int bit = role_bit(ra, q, lane, warp, base);
            const R pr = bit ? gm[6] : gm[0], pi = bit ? gm[7] : gm[1];
#pragma unroll
            for (int j = 0; j < NR; j++) v[j] = cm<T, R>(pr, pi, v[j]);
        }
    } else if (reg) {
        const int ri = ra - RL_REG;
        if (gen == QGEN_Y) {
#define G_CALL(I) u_reg<I, NR, true, T, R>(v, gm)
            RB_SWITCH(ri, G_CALL)
#undef G_CALL
        } else {
#define G_CALL(I) u_reg<I, NR, false, T, R>(v, gm)
            RB_SWITCH(ri, G_CALL)
#undef G_CALL
        }
    } else {
        const int b = ra, hi = (lane >> b) & 1;
        const R cs0 = hi ? gm[6] : gm[0], cs1 = hi ? gm[7] : gm[1];
        const R cp0 = hi ? gm[4] : gm[2], cp1 = hi ? gm[5] : gm[3];
        const R mm[4] = {cs0, cs1, cp0, cp1};
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const T w = shfl_x<T>(v[j], 1 << b);
            v[j] = cmad2<T, R>(mm, v[j], w);
        }
    }
}

// a diagonal run's combined phase: c = cr + i ci (thread factor) times, per register bit i, the
// factor f0_i (bit 0) or f1_i (bit 1), times the static sign sgn over the register index; formed
// as two tables over register bits 0..2 (with c) and 3..RB-1, then one product per amplitude
template <int NR, int RB, typename T, typename R>
__device__ __forceinline__ void diag_run_apply(T* v, R cr, R ci, const R* f0r, const R* f0i, const R* f1r,
                                               const R* f1i, uint32_t sgn)
{
    constexpr int LB = 3, HB = RB - 3;
    R tlr[1 << LB], tli[1 << LB], thr[1 << HB], thi[1 << HB];
    tlr[0] = cr;
    tli[0] = ci;
#pragma unroll
    for (int i = 0; i < LB; i++)
#pragma unroll
        for (int j = 0; j < (1 << i); j++) {
            const R ar = tlr[j], ai = tli[j];
            tlr[j + (1 << i)] = ar * f1r[i] - ai * f1i[i];
            tli[j + (1 << i)] = ar * f1i[i] + ai * f1r[i];
            tlr[j] = ar * f0r[i] - ai * f0i[i];
            tli[j] = ar * f0i[i] + ai * f0r[i];
        }
    thr[0] = (R)1;
    thi[0] = (R)0;
#pragma unroll
    for (int i = 0; i < HB; i++)
#pragma unroll
        for (int j = 0; j < (1 << i); j++) {
            const R ar = thr[j], ai = thi[j];
            thr[j + (1 << i)] = ar * f1r[LB + i] - ai * f1i[LB + i];
            thi[j + (1 << i)] = ar * f1i[LB + i] + ai * f1r[LB + i];
            thr[j] = ar * f0r[LB + i] - ai * f0i[LB + i];
            thi[j] = ar * f0i[LB + i] + ai * f0r[LB + i];
        }
#pragma unroll
    for (int j = 0; j < NR; j++) {
        const R hr = thr[j >> LB], hi2 = thi[j >> LB], lr = tlr[j & ((1 << LB) - 1)], li = tli[j & ((1 << LB) - 1)];
        R pr = lr * hr - li * hi2, pi = lr * hi2 + li * hr;
        if ((sgn >> j) & 1u) { pr = -pr; pi = -pi; }
        v[j] = cmul_s<T, R>(pr, pi, v[j]);
    }
}

// (-i/2) Z on a qubit whose "bit is 1" mask over the register index is mk (a derivative spawned
// by a rotation inside a diagonal run, applied after the run)
template <int NR, typename T, typename R>
__device__ __forceinline__ void zgen_apply(T* v, uint32_t mk)
{
    const R h = (R)0.5;
#pragma unroll
    for (int j = 0; j < NR; j++) {
        const R sg = ((mk >> j) & 1u) ? h : -h;
        T o;
        o.x = -sg * v[j].y;
        o.y = sg * v[j].x;
        v[j] = o;
    }
}

#endif
