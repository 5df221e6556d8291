// qgt_pass2.cu -- register-resident tile passes (the gate-application hot path).
//
// A full tile (2^12, 2^13 or 2^14 complex64, or 2^12 complex128 amplitudes) is held in the
// registers of one CTA of 2^WB warps (256 or 512 threads): each thread owns NR = 2^RB amplitudes
// (RB = 5 for complex64 tiles of 13 or 14 bits, 4 for 12-bit tiles and complex128).  The tile's local bits play three
// roles:
//   lane bits  0..4   (always; physical qubits 0..4, so every global access of
//                      a warp is 32 consecutive amplitudes)
//   reg bits   RB bits chosen per segment (index into the thread's registers)
//   warp bits  the remaining WB = 3 or 4 bits (the warp index)
// A pass is compiled on the host into a program of segments.  Within a
// segment every non-diagonal gate acts on a reg bit (in-register butterfly,
// statically indexed) or a lane bit (warp shuffle); diagonal gates act on any
// bit.  Between segments the tile is re-laid out through shared memory
// (conflict-free: lanes always index consecutive amplitudes).
//
// Gate coefficients come from the complex64 table with exact rotation angles
// (prepare32_kernel).  Derivative slots branch from psi by an exact (-i/2) G
// inserted after their gate; later passes transport them in place.
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "../qgt_internal.h"

#include "qgt_pass2_ops.cuh"

// CKPT: the launch's entries also store their state before every Q2_SEG op whose slot is >= 0 (the
// checkpoint writers of a pass; spawns then run the program from that segment on)
template <typename R, int RB, int WB, bool CKPT>
__global__ void __launch_bounds__(32 << WB, (WB >= 4) ? 1 : ((sizeof(R) == 4 && RB == 4) ? 3 : 2))
    pass2_kernel(const qgt_dev_pass2_args_t a)
{
    typedef typename v2of<R>::T T;
    constexpr int NR = 1 << RB;
    extern __shared__ __align__(16) unsigned char p2_smem[];
    T* tile = reinterpret_cast<T*>(p2_smem);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // the pass program and each op's coefficients, staged once per CTA
    qgt_dev_op2_t* sops = reinterpret_cast<qgt_dev_op2_t*>(p2_smem + ((size_t)sizeof(T) << (5 + RB + WB)));
    R* scoef = reinterpret_cast<R*>(sops + a.nops);
    // this CTA's vector entry runs the pass program from its start op (a Q2_SEG; a derivative
    // spawned after a checkpoint starts at its segment); ops keep their program indices
    const qgt_dev_entry_t e = a.entries[blockIdx.y];
    const int start = e.start_op;

    // per SEG op: its layout's local bits [0, 16) and their physical qubits [16, 32)
    int8_t* sseg = reinterpret_cast<int8_t*>(scoef + 8 * a.nops);
    // generator matrices (-i/2) X, (-i/2) Y, (-i/2) Z (2 x 2 complex, row-major)
    __shared__ R sgen[24];
    // physical offset of the tile's local bits 5 .. tile_bits - 1 (checkpoint stores)
    __shared__ uint32_t supper[1 << (RB + WB)];
    uint64_t base = 0;
    {
        uint32_t rest = blockIdx.x;
        for (int q = 0; q < a.n; q++)
            if (!((a.tile_mask >> q) & 1)) { base |= (uint64_t)(rest & 1u) << q; rest >>= 1; }
    }
    // layout of the current segment: local index contributions of reg bits and of this thread
    int lreg[RB];
    uint32_t preg[RB];   // n <= 30: physical indices fit in 32 bits
    int lthr = 0;
    uint32_t pthr = 0;
    auto set_layout_from = [&](const int8_t* L) {   // 16 local bits, then their physical qubits
        const int8_t* Pq = L + 16;
        lthr = lane;
        pthr = (uint32_t)base | (uint32_t)lane;  // local bits 0..4 are physical qubits 0..4
#pragma unroll
        for (int w = 0; w < WB; w++) {
            const int lb = L[8 + w];
            if ((warp >> w) & 1) { lthr |= 1 << lb; pthr |= 1u << Pq[8 + w]; }
        }
#pragma unroll
        for (int i = 0; i < RB; i++) { lreg[i] = 1 << L[i]; preg[i] = 1u << Pq[i]; }
    };
    auto set_layout = [&](int at) { set_layout_from(sseg + 32 * at); };   // the SEG op at program index `at`
    auto lidx = [&](int j) {
        int l = lthr;
#pragma unroll
        for (int i = 0; i < RB; i++) if ((j >> i) & 1) l |= lreg[i];
        return l;
    };
    auto pidx = [&](int j) {
        uint32_t p = pthr;
#pragma unroll
        for (int i = 0; i < RB; i++) if ((j >> i) & 1) p |= preg[i];
        return p;
    };

    // the tile loads go out first, from the entry's own copy of its starting layout; the program
    // is staged into shared memory while they are in flight
    T v[NR];
    set_layout_from(e.lay);
    {
        const T* src = reinterpret_cast<const T*>(a.V) + blockIdx.z * a.point_stride + (int64_t)e.src_row * a.N;
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t ph = pidx(j);
            if (e.flags & QENT_SRC_ZERO) { v[j].x = (ph == 0) ? (R)1 : (R)0; v[j].y = (R)0; }
            else v[j] = src[ph];
        }
    }
    {
        if (threadIdx.x < (1 << (a.tile_bits - 5))) {
            uint32_t o = 0;
            for (int b = 5; b < a.tile_bits; b++)
                if ((threadIdx.x >> (b - 5)) & 1) o |= 1u << a.local_to_phys[b];
            supper[threadIdx.x] = o;
        }
        if (threadIdx.x < 24) {
            const int g = threadIdx.x >> 3, k = threadIdx.x & 7;
            const R h = (R)0.5;
            R x = (R)0;
            if (g == 0 && (k == 3 || k == 5)) x = -h;              // X: -i/2 off the diagonal
            if (g == 1) x = (k == 2) ? -h : ((k == 4) ? h : (R)0);  // Y: [[0, -1/2], [1/2, 0]]
            if (g == 2) x = (k == 1) ? -h : ((k == 7) ? h : (R)0);  // Z: diag(-i/2, i/2)
            sgen[threadIdx.x] = x;
        }
        const R* ctab = ((sizeof(R) == 4) ? reinterpret_cast<const R*>(a.coef32) : reinterpret_cast<const R*>(a.coef)) +
                        (int64_t)8 * blockIdx.z * a.coef_stride;
        for (int i = start + threadIdx.x; i < a.nops; i += blockDim.x) sops[i] = a.ops[i];
        for (int i = 8 * start + threadIdx.x; i < 8 * a.nops; i += blockDim.x) {
            const int c = a.ops[i >> 3].coef;
            scoef[i] = c >= 0 ? ctab[8 * c + (i & 7)] : (((i & 7) == 0 || (i & 7) == 6) ? (R)1 : (R)0);   // identity
        }
        for (int i = 32 * start + threadIdx.x; i < 32 * a.nops; i += blockDim.x) {
            const qgt_dev_op2_t o = a.ops[i >> 5];
            if (o.kind != Q2_SEG) continue;
            const int8_t lb = a.segs[16 * o.seg + (i & 15)];
            sseg[i] = (i & 16) ? ((lb >= 0 && lb < 16) ? a.local_to_phys[lb] : (int8_t)0) : lb;
        }
        if (start > 0 && threadIdx.x < 32) {
            // the starting segment's layout also in slot 0 (the initial layout of every entry)
            const int8_t lb = a.segs[16 * a.ops[start].seg + (threadIdx.x & 15)];
            sseg[threadIdx.x] = (threadIdx.x & 16) ? ((lb >= 0 && lb < 16) ? a.local_to_phys[lb] : (int8_t)0) : lb;
        }
        __syncthreads();
    }
    // (-i/2) G of the rotation op `so` on the current vector (a derivative spawned there), through
    // the gate paths with the generator matrices (-i/2) X, (-i/2) Y, (-i/2) Z (exact: entries 0, +-1/2)
    auto spawn_gen = [&](const qgt_dev_op2_t& so) {
        const R* gm = sgen + 8 * (so.gen - QGEN_X);
        const bool reg = so.ra >= RL_REG && so.ra < RL_WARP;
        if (so.gen == QGEN_Z) {
            if (reg) {
                const int ri = so.ra - RL_REG;
#define G_CALL(I) phase_reg<I, NR, T, R>(v, gm)
                RB_SWITCH(ri, G_CALL)
#undef G_CALL
            } else {
                const int bit = role_bit(so.ra, so.q, lane, warp, base);
                const R pr = bit ? gm[6] : gm[0], pi = bit ? gm[7] : gm[1];
#pragma unroll
                for (int j = 0; j < NR; j++) v[j] = cm<T, R>(pr, pi, v[j]);
            }
        } else if (reg) {
            const int ri = so.ra - RL_REG;
            if (so.gen == QGEN_Y) {
#define G_CALL(I) u_reg<I, NR, true, T, R>(v, gm)
                RB_SWITCH(ri, G_CALL)
#undef G_CALL
            } else {
#define G_CALL(I) u_reg<I, NR, false, T, R>(v, gm)
                RB_SWITCH(ri, G_CALL)
#undef G_CALL
            }
        } else {
            const int b = so.ra, hi = (lane >> b) & 1;
            const R cs0 = hi ? gm[6] : gm[0], cs1 = hi ? gm[7] : gm[1];
            const R cp0 = hi ? gm[4] : gm[2], cp1 = hi ? gm[5] : gm[3];
            const R mm[4] = {cs0, cs1, cp0, cp1};
#pragma unroll
            for (int j = 0; j < NR; j++) {
                const T w = shfl_x<T>(v[j], 1 << b);
                v[j] = cmad2<T, R>(mm, v[j], w);
            }
        }
    };
    for (int pc = start + 1; pc < a.nops; pc++) {
        const qgt_dev_op2_t op = sops[pc];
        R m[8];
        if (op.kind == Q2_SEG) {
            // re-layout through shared memory
            __syncthreads();
#pragma unroll
            for (int j = 0; j < NR; j++) tile[lidx(j)] = v[j];
            __syncthreads();
            if (CKPT && op.slot >= 0) {
                // checkpoint writer: the state before this segment (the tile in local order), for the
                // spawns that start here; warps copy 32 consecutive amplitudes (local bits 0..4 =
                // physical qubits 0..4)
                T* ck = reinterpret_cast<T*>(a.V) + blockIdx.z * a.point_stride + (int64_t)op.slot * a.N;
                for (int i = 0; i < NR; i++) {
                    const int l = threadIdx.x + (int)blockDim.x * i;
                    ck[(uint32_t)base | (uint32_t)(l & 31) | supper[l >> 5]] = tile[l];
                }
            }
            set_layout(pc);
#pragma unroll
            for (int j = 0; j < NR; j++) v[j] = tile[lidx(j)];
            continue;
        }
        if (op.kind == Q2_DIAG) {
            // combined phase of the run: c (thread factor) x prod_i f_i(reg bit i) x sign(static mask)
            const int cnt = op.seg, nt = op.ra, nz = op.rb;
            const int r0 = pc + 1, t0 = r0 + RB, z0 = t0 + nt;
            R cr = (R)1, ci = (R)0;
            for (int u = t0; u < z0; u++) {
                const qgt_dev_op2_t so = sops[u];
                const R* c8 = scoef + 8 * u;
                const int bit = role_bit(so.ra, so.q, lane, warp, base);
                const R pr = bit ? c8[6] : c8[0], pi = bit ? c8[7] : c8[1];
                const R t = cr * pr - ci * pi;
                ci = cr * pi + ci * pr;
                cr = t;
            }
            uint32_t par = 0;
            for (int u = z0; u < z0 + nz; u++) {
                const qgt_dev_op2_t so = sops[u];
                par ^= (pthr >> so.q) & (uint32_t)__popc(pthr & (uint32_t)so.slot);
            }
            if (par & 1u) { cr = -cr; ci = -ci; }
            // register-bit factors (|0>, |1>), the |1> factor negated by an odd CZ parity with the thread bits
            R f0r[RB], f0i[RB], f1r[RB], f1i[RB];
#pragma unroll
            for (int i = 0; i < RB; i++) {
                const R* c8 = scoef + 8 * (r0 + i);
                const R sg = (__popc(pthr & (uint32_t)sops[r0 + i].slot) & 1) ? (R)-1 : (R)1;
                f0r[i] = c8[0];
                f0i[i] = c8[1];
                f1r[i] = sg * c8[6];
                f1i[i] = sg * c8[7];
            }
            // tables over register bits 0..2 (with c) and 3..RB-1, then one product per amplitude
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
            const uint32_t sgn = (uint32_t)op.slot;
#pragma unroll
            for (int j = 0; j < NR; j++) {
                const R hr = thr[j >> LB], hi2 = thi[j >> LB], lr = tlr[j & ((1 << LB) - 1)], li = tli[j & ((1 << LB) - 1)];
                R pr = lr * hr - li * hi2, pi = lr * hi2 + li * hr;
                if ((sgn >> j) & 1u) { pr = -pr; pi = -pi; }
                v[j] = cmul_s<T, R>(pr, pi, v[j]);
            }
            if (e.spawn_op > pc && e.spawn_op <= pc + cnt) {
                // (-i/2) Z of the spawning rotation, after the run (diagonal ops commute)
                const qgt_dev_op2_t so = sops[e.spawn_op];
                const uint32_t mk = role_mask<NR>(so.ra, so.q, lane, warp, base);
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
            pc += cnt;
            continue;
        }
        if (op.kind == Q2_UM) {
            // commuting single-qubit gates on distinct bits: `ra` lane gates, then one gate per
            // register bit set in `rb`, ascending; a derivative spawned at any of them is
            // applied after the block (its generator commutes with the other gates)
            const int cnt = op.seg, nl = op.ra;
            const uint32_t rmask = op.rb;
            for (int u = pc + 1; u <= pc + nl; u++) {
                const R* mm = scoef + 8 * u;
                gate_lane<NR, T, R>(v, mm, sops[u].kind == Q2_UR, sops[u].ra, lane);
            }
            int at = pc + 1 + nl;
#pragma unroll
            for (int i = 0; i < RB; i++) {
                if ((rmask >> i) & 1u) {
                    const R* mm = scoef + 8 * at;
                    const bool real = sops[at].kind == Q2_UR;
#define U_CALL(I) gate_reg<I, NR, T, R>(v, mm, real)
                    RB_SWITCH(i, U_CALL)
#undef U_CALL
                    at++;
                }
            }
            if (e.spawn_op > pc && e.spawn_op <= pc + cnt) spawn_gen(sops[e.spawn_op]);
            pc += cnt;
            continue;
        }
        if (op.kind == Q2_U || op.kind == Q2_UR) {
#pragma unroll
            for (int i = 0; i < 8; i++) m[i] = scoef[8 * pc + i];
            const bool real = op.kind == Q2_UR;
            if (op.ra >= RL_REG) {
                const int ri = op.ra - RL_REG;
#define U_CALL(I) gate_reg<I, NR, T, R>(v, m, real)
                RB_SWITCH(ri, U_CALL)
#undef U_CALL
            } else {
                gate_lane<NR, T, R>(v, m, real, op.ra, lane);
            }
        } else if (op.kind == Q2_PHASE) {
#pragma unroll
            for (int i = 0; i < 8; i++) m[i] = scoef[8 * pc + i];
            if (op.ra >= RL_REG && op.ra < RL_WARP) {
                const int ri = op.ra - RL_REG;
#define P_CALL(I) phase_reg<I, NR, T, R>(v, m)
                RB_SWITCH(ri, P_CALL)
#undef P_CALL
            } else {
                const int bit = role_bit(op.ra, op.q, lane, warp, base);
                const R pr = bit ? m[6] : m[0], pi = bit ? m[7] : m[1];
                if (!(pr == (R)1 && pi == (R)0)) {
#pragma unroll
                    for (int j = 0; j < NR; j++) v[j] = cm<T, R>(pr, pi, v[j]);
                }
            }
        } else if (op.kind == Q2_CZ) {
            const uint32_t mk = role_mask<NR>(op.ra, op.q, lane, warp, base) & role_mask<NR>(op.rb, op.q2, lane, warp, base);
            if (mk) {
#pragma unroll
                for (int j = 0; j < NR; j++)
                    if ((mk >> j) & 1u) { v[j].x = -v[j].x; v[j].y = -v[j].y; }
            }
        } else if (op.kind == Q2_CNOT) {
            const uint32_t cmask = role_mask<NR>(op.rb, op.q2, lane, warp, base);
            if (op.ra >= RL_REG) {
                const int ri = op.ra - RL_REG;
#define C_CALL(I) cnot_reg<I, NR, T>(v, cmask)
                RB_SWITCH(ri, C_CALL)
#undef C_CALL
            } else {
                const int b = op.ra;
#pragma unroll
                for (int j = 0; j < NR; j++) {
                    T w = shfl_x<T>(v[j], 1 << b);
                    if ((cmask >> j) & 1u) v[j] = w;
                }
            }
        }
        if (pc == e.spawn_op) spawn_gen(op);
    }
    // store
    T* dst = reinterpret_cast<T*>(a.V) + blockIdx.z * a.point_stride + (int64_t)e.dst_row * a.N;
    float vmax = 0.f;
#pragma unroll
    for (int j = 0; j < NR; j++) {
        const uint32_t ph = pidx(j);
        if (e.flags & QENT_STORE_V) dst[ph] = v[j];
        if (e.flags & QENT_ROWMAX) vmax = fmaxf(vmax, sqrtf((float)(v[j].x * v[j].x + v[j].y * v[j].y)));
        if (e.flags & QENT_STORE_SPLIT) {
            float xr = (float)v[j].x * a.split_scale, xi = (float)v[j].y * a.split_scale;
            int64_t at = (int64_t)e.split_row * a.split_ld + (int64_t)ph;
            const int64_t ps = a.split_plane_stride;
            __nv_bfloat16* s = reinterpret_cast<__nv_bfloat16*>(a.split);
            __nv_bfloat16 rh = __float2bfloat16_rn(xr), ih = __float2bfloat16_rn(xi);
            s[at] = rh;
            s[ps + at] = __float2bfloat16_rn(xr - __bfloat162float(rh));
            s[2 * ps + at] = ih;
            s[3 * ps + at] = __float2bfloat16_rn(xi - __bfloat162float(ih));
        }
    }
    if (e.flags & QENT_ROWMAX) {
        __shared__ float red[1 << WB];
        for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        if (lane == 0) red[warp] = vmax;
        __syncthreads();
        if (threadIdx.x == 0) {
            float mx = 0.f;
            for (int w = 0; w < (1 << WB); w++) mx = fmaxf(mx, red[w]);
            atomicMax(a.rowmax + (int64_t)blockIdx.z * a.rowmax_stride + e.dst_row, __float_as_uint(mx));
        }
    }
}

template <typename R, int RB, int WB>
static int pass2_launch(const qgt_dev_pass2_args_t* a, dim3 grid, size_t smem, size_t smax, cudaStream_t stream)
{
    static int attr = 0;   // per instantiation: the dynamic shared-memory limit is raised once
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(pass2_kernel<R, RB, WB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smax);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(pass2_kernel<R, RB, WB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smax);
        if (e != cudaSuccess) return qgt_set_error(-6, "pass2: %s", cudaGetErrorString(e));
        attr = 1;
    }
    if (a->ckpt) pass2_kernel<R, RB, WB, true><<<grid, 32 << WB, smem, stream>>>(*a);
    else pass2_kernel<R, RB, WB, false><<<grid, 32 << WB, smem, stream>>>(*a);
    return qgt_dev_last_error();
}

extern "C" int qgt_dev_pass2(const qgt_dev_pass2_args_t* a, int fp64, void* stream)
{
    if (a->nentries <= 0) return 0;
    // tiles: complex128 12 bits (4 register, 3 warp bits); complex64 12 bits (4 register, 3 warp
    // bits: 12-qubit circuits), 13 bits (5 register, 3 warp bits, 2 CTAs per SM) or 14 bits
    // (5 register, 4 warp bits: 512 threads, 1 CTA per SM)
    const bool ok = fp64 ? a->tile_bits == QGT_TILE_MAX_F64
                         : (a->tile_bits == QGT_TILE_MAX_F64 || a->tile_bits == QGT_TILE_MAX_F32 ||
                            a->tile_bits == QGT_TILE_WIDE_F32);
    if (!ok) return qgt_set_error(-1, "pass2: tile of %d bits not supported", a->tile_bits);
    int64_t ntiles = (int64_t)1 << (a->n - a->tile_bits);
    const int np = a->npoints > 0 ? a->npoints : 1;
    if (a->nentries > 65535 || ntiles > 0x7fffffff || np > 65535) return qgt_set_error(-1, "pass2: grid too large");
    dim3 grid((unsigned)ntiles, (unsigned)a->nentries, (unsigned)np);
    const bool wide = !fp64 && a->tile_bits == QGT_TILE_WIDE_F32;
    size_t smem = ((size_t)1 << (a->tile_bits + (fp64 ? 4 : 3))) +                       /* the tile */
                  (size_t)a->nops * (sizeof(qgt_dev_op2_t) + 8 * (fp64 ? sizeof(double) : sizeof(float)) + 32);
    const size_t smax = wide ? 200 * 1024 : 112 * 1024;
    if (smem > smax) return qgt_set_error(-1, "pass2: program of %d ops too large", a->nops);
    cudaStream_t s = (cudaStream_t)stream;
    if (fp64) return pass2_launch<double, 4, 3>(a, grid, smem, smax, s);
    if (wide) return pass2_launch<float, 5, 4>(a, grid, smem, smax, s);
    if (a->tile_bits == QGT_TILE_MAX_F64) return pass2_launch<float, 4, 3>(a, grid, smem, smax, s);
    return pass2_launch<float, 5, 3>(a, grid, smem, smax, s);
}
