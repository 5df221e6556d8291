/*
 * qgt_jit.c -- straight-line CUDA source for one register-resident pass
 * program.
 *
 * The pass interpreter (qgt_pass2.cu) reads each op of a pass program from
 * shared memory and dispatches on it; at 20 qubits its warps spend a large
 * part of their cycles waiting for instructions after those dispatches.  A
 * plan can instead turn each pass program into its own kernel: every op
 * becomes inline code with its register bit, lane bit, coefficient index and
 * layout constants fixed, every layout change becomes stores and loads at
 * immediate offsets, and an entry enters the code at its starting segment.
 * The arithmetic is the interpreter's (the same gate routines of
 * qgt_pass2_ops.cuh), so both paths give the same amplitudes.  The source is
 * compiled at plan creation (qgt_jit_rt.cu) for sm_103a.
 *
 * Generated kernel (RB register bits, WB warp bits, 2^(5+RB+WB) amplitudes
 * per tile):
 *   args   V (float2 rows), N, entries (int32 words of qgt_dev_entry_t),
 *          coef32, rowmax, coef_stride, point_stride, rowmax_stride
 *   grid   (tiles, entries, points), 32 << WB threads, 8 << tile_bits bytes
 *          of dynamic shared memory (the re-layout tile)
 */
#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../qgt_internal.h"

#define RL_REG_ 8
#define RL_WARP_ 16
#define RL_OUT_ 32

typedef struct {
    char* s;
    size_t n, cap;
    int err;
} sbuf_t;

static void sb_printf(sbuf_t* b, const char* fmt, ...)
{
    if (b->err) return;
    for (;;) {
        va_list ap;
        va_start(ap, fmt);
        int k = vsnprintf(b->s + b->n, b->cap - b->n, fmt, ap);
        va_end(ap);
        if (k < 0) { b->err = 1; return; }
        if ((size_t)k < b->cap - b->n) { b->n += (size_t)k; return; }
        size_t nc = b->cap * 2 + (size_t)k + 1024;
        char* ns = (char*)realloc(b->s, nc);
        if (!ns) { b->err = 1; return; }
        b->s = ns;
        b->cap = nc;
    }
}

/* role -> expression of this thread's bit value (lane, warp or outside qubit) */
static void role_bit_expr(sbuf_t* b, int role, int q)
{
    if (role < RL_REG_) sb_printf(b, "((lane >> %d) & 1)", role);
    else if (role < RL_OUT_) sb_printf(b, "((warp >> %d) & 1)", role - RL_WARP_);
    else sb_printf(b, "(int)((base >> %d) & 1ull)", q);
}

/* The coefficient entries a pass reads, one shared-memory slot per op that reads one: the kernel
 * copies them from the point's coefficient table into shared memory once per CTA (coalesced), and
 * the ops read their 8 floats from there (a broadcast load) instead of from global memory just
 * before use.  A slot may carry a spawn fold (see folds_spawn). */
typedef struct {
    int n, cap;
    int* coef;      /* global coefficient index of the slot */
    int* pc;        /* program index of the op (its spawn number) */
    int8_t* gen;    /* generator folded into the slot for the entry spawned at pc (QGEN_NONE: none) */
    int err;
} slots_t;

static int add_slot(slots_t* t, int coef, int pc, int gen)
{
    if (t->n == t->cap) {
        int nc = t->cap ? 2 * t->cap : 64;
        int* c = (int*)realloc(t->coef, sizeof(int) * nc);
        if (c) t->coef = c;
        int* q = (int*)realloc(t->pc, sizeof(int) * nc);
        if (q) t->pc = q;
        int8_t* g = (int8_t*)realloc(t->gen, (size_t)nc);
        if (g) t->gen = g;
        if (!c || !q || !g) { t->err = 1; return 0; }
        t->cap = nc;
    }
    t->coef[t->n] = coef;
    t->pc[t->n] = pc;
    t->gen[t->n] = (int8_t)gen;
    return t->n++;
}

/* coefficient entry c into R m[8] (identity for c < 0); fold_gen: spawn fold of this op */
static void load_coef(sbuf_t* b, slots_t* t, int c, int pc, int fold_gen)
{
    if (c < 0) sb_printf(b, "R m[8] = {1.f, 0.f, 0.f, 0.f, 0.f, 0.f, 1.f, 0.f};");
    else sb_printf(b, "R m[8]; LDS8(m, %d);", add_slot(t, c, pc, fold_gen));
}

/* layout of program layout index seg: lthr / pthr and the constant per-register offsets */
typedef struct {
    int lreg[8];          /* local bit of register bit i */
    int preg[8];          /* physical qubit of register bit i */
    int lwarp[8], pwarp[8];
} lay_t;

static void layout_of(const qgt_jit_pass_desc_t* d, int seg, lay_t* L)
{
    const int8_t* s = d->segs + 16 * seg;
    for (int i = 0; i < d->RB; i++) { L->lreg[i] = s[i]; L->preg[i] = d->l2p[s[i]]; }
    for (int w = 0; w < d->WB; w++) { L->lwarp[w] = s[8 + w]; L->pwarp[w] = d->l2p[s[8 + w]]; }
}

static unsigned lconst(const qgt_jit_pass_desc_t* d, const lay_t* L, int j)
{
    unsigned c = 0;
    for (int i = 0; i < d->RB; i++) if ((j >> i) & 1) c |= 1u << L->lreg[i];
    return c;
}

static unsigned pconst(const qgt_jit_pass_desc_t* d, const lay_t* L, int j)
{
    unsigned c = 0;
    for (int i = 0; i < d->RB; i++) if ((j >> i) & 1) c |= 1u << L->preg[i];
    return c;
}

static void emit_set_layout(sbuf_t* b, const qgt_jit_pass_desc_t* d, const lay_t* L)
{
    sb_printf(b, "    lthr = (unsigned)lane");
    for (int w = 0; w < d->WB; w++) sb_printf(b, " | ((unsigned)((warp >> %d) & 1) << %d)", w, L->lwarp[w]);
    sb_printf(b, ";\n    pthr = (unsigned)base | (unsigned)lane");
    for (int w = 0; w < d->WB; w++) sb_printf(b, " | ((unsigned)((warp >> %d) & 1) << %d)", w, L->pwarp[w]);
    sb_printf(b, ";\n");
}

static int is_start(const qgt_jit_pass_desc_t* d, int pc)
{
    for (int i = 0; i < d->nstarts; i++) if (d->starts[i] == pc) return 1;
    return 0;
}

/* (-i/2) G of the rotation o (a derivative spawned there): exact entries 0, +-1/2 */
static void emit_spawn(sbuf_t* b, const qgt_dev_op2_t* o)
{
    const int reg = o->ra >= RL_REG_ && o->ra < RL_WARP_;
    if (o->gen == QGEN_Z) {
        if (reg) {
            /* bit 0: (-i/2) z = (y/2, -x/2); bit 1: (+i/2) z = (-y/2, x/2) */
            unsigned mk = 0;
            for (int j = 0; j < 32; j++) mk |= (unsigned)((j >> (o->ra - RL_REG_)) & 1) << j;
            sb_printf(b, "zgen_apply<NR, T, R>(v, %uu);", mk);
        } else {
            sb_printf(b, "{ const unsigned mk = ");
            role_bit_expr(b, o->ra, o->q);
            sb_printf(b, " ? 0xffffffffu : 0u; zgen_apply<NR, T, R>(v, mk); }");
        }
    } else if (reg) {
        sb_printf(b, "gen_reg<%d, NR, T, R>(v, %d);", o->ra - RL_REG_, (int)o->gen);
    } else if (o->gen == QGEN_X) {
        /* (-i/2) X: the partner lane's amplitude times -i/2 */
        sb_printf(b, "{\n#pragma unroll\n for (int j = 0; j < NR; j++) { const T w = shfl_x<T>(v[j], %d); "
                     "v[j] = make_float2(0.5f * w.y, -0.5f * w.x); } }", 1 << o->ra);
    } else {
        /* (-i/2) Y = [[0, -1/2], [1/2, 0]]: the partner times -1/2 (lower lane) or +1/2 (upper lane) */
        sb_printf(b, "{ const R sg = ((lane >> %d) & 1) ? 0.5f : -0.5f;\n#pragma unroll\n"
                     " for (int j = 0; j < NR; j++) { const T w = shfl_x<T>(v[j], %d); v[j] = make_float2(sg * w.x, sg * w.y); } }",
                  o->ra, 1 << o->ra);
    }
}

/* a derivative spawned at a rotation: the spawned vector applies (-i/2) G R in place of R (G
 * commutes with R), so the generator is folded into the gate's coefficients in the shared-memory
 * copy of the one CTA whose entry spawns there (fold_gen of qgt_pass2_ops.cuh, at staging); the
 * other CTAs apply R.  Real gates fold only Y (the product stays real); the caller applies other
 * generators after the gate. */
static int folds_spawn(const qgt_dev_op2_t* o)
{
    if (o->gen == QGEN_NONE || o->coef < 0) return 0;
    if (o->kind == Q2_UR) return o->gen == QGEN_Y;
    return o->kind == Q2_U;
}

/* a single-qubit gate: real matrices (RY, H, X) as m0 x + m2 y / m4 x + m6 y (two packed FP32x2
 * instructions per amplitude), complex ones in full.  Uniform branches to one-multiply-add paths
 * for RY's tangent and cotangent forms were measured slower (passes 4.24 -> 4.49 ms at 20 qubits):
 * the code they add per gate costs more in instruction fetch than the multiply they save.
 * pc: the op's program index (its spawn number). */
static void emit_u(sbuf_t* b, slots_t* t, const qgt_dev_op2_t* o, int pc)
{
    if (o->coef < 0) return;   /* identity */
    const int real = o->kind == Q2_UR;
    sb_printf(b, "    { ");
    load_coef(b, t, o->coef, pc, folds_spawn(o) ? o->gen : QGEN_NONE);
    if (o->ra >= RL_REG_) {
        sb_printf(b, " u_reg<%d, NR, %s, T, R>(v, m); }\n", o->ra - RL_REG_, real ? "true" : "false");
    } else if (real) {
        sb_printf(b, " const int hi = (lane >> %d) & 1; const R cs0 = hi ? m[6] : m[0], cp0 = hi ? m[4] : m[2];\n"
                     "#pragma unroll\n      for (int j = 0; j < NR; j++) { const T w = shfl_x<T>(v[j], %d); "
                     "v[j] = rmad2<T, R>(cs0, v[j], cp0, w); } }\n", o->ra, 1 << o->ra);
    } else {
        sb_printf(b, " const int hi = (lane >> %d) & 1; const R mm[4] = {hi ? m[6] : m[0], hi ? m[7] : m[1], "
                     "hi ? m[4] : m[2], hi ? m[5] : m[3]};\n#pragma unroll\n      for (int j = 0; j < NR; j++) { "
                     "const T w = shfl_x<T>(v[j], %d); v[j] = cmad2<T, R>(mm, v[j], w); } }\n", o->ra, 1 << o->ra);
    }
}

char* qgt_jit_pass_source(const qgt_jit_pass_desc_t* d)
{
    const int RB = d->RB, WB = d->WB, NR = 1 << RB;
    if (RB < 4 || RB > 5 || WB < 3 || WB > 5 || d->nops < 1 || d->prog[0].kind != Q2_SEG) {
        qgt_set_error(-1, "jit: unsupported program (RB %d, WB %d)", RB, WB);
        return NULL;
    }
    /* four parts: the kernel's head (hsb), its entry points (lsb: each loads its tile), its program
     * and store (bsb), and, once the program has registered its coefficient slots, the slot table
     * and the staging code.  The staging runs after the tile loads are issued, so that the loads'
     * latency overlaps the staging's own global reads and barriers. */
    sbuf_t hsb = {NULL, 0, 0, 0}, lsb = {NULL, 0, 0, 0}, bsb = {NULL, 0, 0, 0}, osb = {NULL, 0, 0, 0};
    sbuf_t tsb = {NULL, 0, 0, 0};   /* file-scope constant tables of the program (generator lookups) */
    sbuf_t* tb_ = &tsb;
    slots_t slots = {0, 0, NULL, NULL, NULL, 0};
    slots_t* t = &slots;
    hsb.cap = 1 << 14;
    lsb.cap = 1 << 14;
    bsb.cap = 1 << 16;
    osb.cap = 1 << 16;
    tsb.cap = 1 << 12;
    hsb.s = (char*)malloc(hsb.cap);
    lsb.s = (char*)malloc(lsb.cap);
    bsb.s = (char*)malloc(bsb.cap);
    osb.s = (char*)malloc(osb.cap);
    tsb.s = (char*)malloc(tsb.cap);
    if (!hsb.s || !lsb.s || !bsb.s || !osb.s || !tsb.s) {
        free(hsb.s);
        free(lsb.s);
        free(bsb.s);
        free(osb.s);
        free(tsb.s);
        return NULL;
    }
    hsb.s[0] = lsb.s[0] = bsb.s[0] = osb.s[0] = tsb.s[0] = 0;
    sbuf_t* b = &hsb;
    const int nthreads = 32 << WB;
    /* CTAs per SM the registers must allow: 512-thread 14-qubit tiles 1, 1024-thread 14-qubit tiles 1
     * (64 registers), 512-thread 13-qubit tiles of 16 amplitudes 2 (64 registers), 256-thread tiles
     * 2 (32 amplitudes) or 3 (16) */
    const int minb = WB == 5 ? 1 : (WB == 4 ? (RB == 4 ? 2 : 1) : (RB == 4 ? 3 : 2));
    const int es = (int)(sizeof(qgt_dev_entry_t) / 4);
    sb_printf(b, "extern \"C\" __global__ void __launch_bounds__(%d, %d) %s(float2* __restrict__ V, long long N, "
                 "const int* __restrict__ ents, const float* __restrict__ coef32, unsigned* __restrict__ rowmax, "
                 "int coef_stride, long long point_stride, int rowmax_stride)\n{\n",
              nthreads, minb, d->kname);
    sb_printf(b, "    typedef float R;\n    typedef float2 T;\n    constexpr int RB = %d, NR = %d;\n", RB, NR);
    sb_printf(b, "    extern __shared__ __align__(16) unsigned char qsm[];\n    T* tile = reinterpret_cast<T*>(qsm);\n");
    sb_printf(b, "    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;\n");
    sb_printf(b, "    const int* e = ents + %d * (int)blockIdx.y;\n", es);
    sb_printf(b, "    const int start = e[%d], spawn = e[%d], flags = e[%d];\n",
              (int)(offsetof(qgt_dev_entry_t, start_op) / 4), (int)(offsetof(qgt_dev_entry_t, spawn_op) / 4),
              (int)(offsetof(qgt_dev_entry_t, flags) / 4));
    sb_printf(b, "    (void)spawn;\n");
    /* outside qubits of the tile from blockIdx.x, lowest first */
    sb_printf(b, "    const unsigned bx = blockIdx.x;\n    const unsigned long long base = 0ull");
    {
        int k = 0;
        for (int q = 0; q < d->n; q++)
            if (!((d->tile_mask >> q) & 1u)) { sb_printf(b, " | ((unsigned long long)((bx >> %d) & 1u) << %d)", k, q); k++; }
    }
    sb_printf(b, ";\n    const float* ct = coef32 + (long long)8 * blockIdx.z * coef_stride;\n");
    sb_printf(b, "    T* const Vp = V + (long long)blockIdx.z * point_stride;\n");
    sb_printf(b, "    T v[NR];\n    unsigned lthr, pthr;\n    (void)lthr;\n");
    if (d->ckpt) {
        /* physical offset of the tile's local bits 5 .. tile_bits - 1 (checkpoint stores) */
        sb_printf(b, "    __shared__ unsigned supper[%d];\n", 1 << (RB + WB));
        sb_printf(b, "    if (threadIdx.x < %d) { unsigned o = 0;", 1 << (d->tile_bits - 5));
        for (int lb = 5; lb < d->tile_bits; lb++)
            sb_printf(b, " if ((threadIdx.x >> %d) & 1) o |= %uu;", lb - 5, 1u << d->l2p[lb]);
        sb_printf(b, " supper[threadIdx.x] = o; }\n    __syncthreads();\n");
    }
    b = &lsb;
    /* entry points: the tile loads of each start, then the coefficient staging (STG_) */
    sb_printf(b, "    switch (start) {\n");
    for (int i = 0; i < d->nstarts; i++) sb_printf(b, "    case %d: goto S_%d;\n", d->starts[i], d->starts[i]);
    sb_printf(b, "    default: return;\n    }\n");
    for (int i = 0; i < d->nstarts; i++) {
        const int a = d->starts[i];
        lay_t L;
        layout_of(d, d->prog[a].seg, &L);
        sb_printf(b, "S_%d:\n", a);
        emit_set_layout(b, d, &L);
        if (d->start_zero && d->start_zero[i]) {
            sb_printf(b, "    if (flags & %d) {\n", QENT_SRC_ZERO);
            for (int j = 0; j < NR; j++)
                sb_printf(b, "        v[%d] = make_float2((pthr + %uu) == 0u ? 1.f : 0.f, 0.f);\n", j, pconst(d, &L, j));
            sb_printf(b, "        goto STG_;\n    }\n");
        }
        sb_printf(b, "    {\n        const T* src = Vp + (long long)e[%d] * N;\n",
                  (int)(offsetof(qgt_dev_entry_t, src_row) / 4));
        for (int j = 0; j < NR; j++) sb_printf(b, "        v[%d] = src[pthr + %uu];\n", j, pconst(d, &L, j));
        sb_printf(b, "    }\n    goto STG_;\n");
    }
    b = &bsb;
    /* the program */
    lay_t cur;
    layout_of(d, d->prog[0].seg, &cur);
    sb_printf(b, "B_0:\n");
    for (int pc = 1; pc < d->nops; pc++) {
        const qgt_dev_op2_t* o = &d->prog[pc];
        if (o->kind == Q2_SEG) {
            lay_t nl;
            layout_of(d, o->seg, &nl);
            sb_printf(b, "    // op %d: re-layout to layout %d\n    __syncthreads();\n", pc, (int)o->seg);
            for (int j = 0; j < NR; j++) sb_printf(b, "    tile[lthr + %uu] = v[%d];\n", lconst(d, &cur, j), j);
            sb_printf(b, "    __syncthreads();\n");
            if (d->ckpt && o->slot >= 0) {
                sb_printf(b, "    { T* ck = Vp + (long long)%d * N;\n", o->slot);
                sb_printf(b, "      for (int i = 0; i < NR; i++) { const int l = threadIdx.x + %d * i; "
                             "ck[(unsigned)base | (unsigned)(l & 31) | supper[l >> 5]] = tile[l]; } }\n", nthreads);
            }
            emit_set_layout(b, d, &nl);
            for (int j = 0; j < NR; j++) sb_printf(b, "    v[%d] = tile[lthr + %uu];\n", j, lconst(d, &nl, j));
            cur = nl;
            if (is_start(d, pc)) sb_printf(b, "B_%d:\n", pc);
            continue;
        }
        if (o->kind == Q2_DIAG) {
            const int cnt = o->seg, nt = o->ra, nz = o->rb;
            const int r0 = pc + 1, t0 = r0 + RB, z0 = t0 + nt;
            sb_printf(b, "    { // op %d: diagonal run of %d entries\n      R cr = (R)1, ci = (R)0;\n", pc, cnt);
            for (int u = t0; u < z0; u++) {
                const qgt_dev_op2_t* so = &d->prog[u];
                if (so->coef < 0) continue;
                sb_printf(b, "      { ");
                load_coef(b, t, so->coef, u, QGEN_NONE);
                sb_printf(b, " const int bit = ");
                role_bit_expr(b, so->ra, so->q);
                sb_printf(b, "; const R pr = bit ? m[6] : m[0], pi = bit ? m[7] : m[1]; const R t = cr * pr - ci * pi; "
                             "ci = cr * pi + ci * pr; cr = t; }\n");
            }
            if (nz > 0) {
                sb_printf(b, "      unsigned par = 0u;\n");
                for (int u = z0; u < z0 + nz; u++)
                    sb_printf(b, "      par ^= (pthr >> %d) & (unsigned)__popc(pthr & %uu);\n", (int)d->prog[u].q,
                              (unsigned)d->prog[u].slot);
                sb_printf(b, "      if (par & 1u) { cr = -cr; ci = -ci; }\n");
            }
            sb_printf(b, "      R f0r[RB], f0i[RB], f1r[RB], f1i[RB];\n");
            for (int i = 0; i < RB; i++) {
                const qgt_dev_op2_t* so = &d->prog[r0 + i];
                sb_printf(b, "      { ");
                load_coef(b, t, so->coef, r0 + i, QGEN_NONE);
                if (so->slot != 0)
                    sb_printf(b, " const R sg = (__popc(pthr & %uu) & 1) ? (R)-1 : (R)1;", (unsigned)so->slot);
                else
                    sb_printf(b, " const R sg = (R)1;");
                sb_printf(b, " f0r[%d] = m[0]; f0i[%d] = m[1]; f1r[%d] = sg * m[6]; f1i[%d] = sg * m[7]; }\n", i, i, i, i);
            }
            sb_printf(b, "      diag_run_apply<NR, RB, T, R>(v, cr, ci, f0r, f0i, f1r, f1i, %uu);\n", (unsigned)o->slot);
            /* (-i/2) Z of a rotation spawned inside the run, after it: the spawning entry looks up the
             * rotation's role and qubit in a constant table over the run's op range (one code path
             * per run instead of one per rotation) */
            int zlo = -1, zhi = -1;
            for (int u = z0 + nz; u <= pc + cnt; u++)
                if (d->prog[u].kind == Q2_ZGEN) { if (zlo < 0) zlo = u; zhi = u; }
            if (zlo >= 0) {
                sb_printf(tb_, "static __constant__ int zg_%s_%d[%d] = {", d->kname, pc, 2 * (zhi - zlo + 1));
                for (int u = zlo; u <= zhi; u++) {
                    const qgt_dev_op2_t* so = &d->prog[u];
                    if (so->kind == Q2_ZGEN) sb_printf(tb_, "%s%d, %d", u > zlo ? ", " : "", (int)so->ra, (int)so->q);
                    else sb_printf(tb_, "%s-1, 0", u > zlo ? ", " : "");
                }
                sb_printf(tb_, "};\n");
                sb_printf(b, "      if ((unsigned)(spawn - %d) <= %uu) { const int zr = zg_%s_%d[2 * (spawn - %d)], "
                             "zq = zg_%s_%d[2 * (spawn - %d) + 1];\n"
                             "        if (zr >= 0) zgen_apply<NR, T, R>(v, role_mask<NR>(zr, zq, lane, warp, base)); }\n",
                          zlo, (unsigned)(zhi - zlo), d->kname, pc, zlo, d->kname, pc, zlo);
            }
            sb_printf(b, "    }\n");
            pc += cnt;
            continue;
        }
        if (o->kind == Q2_UM) {
            const int cnt = o->seg, nl = o->ra;
            const unsigned rmask = o->rb;
            sb_printf(b, "    // op %d: block of %d commuting gates\n", pc, cnt);
            for (int u = pc + 1; u <= pc + nl; u++) emit_u(b, t, &d->prog[u], u);
            int at = pc + 1 + nl;
            for (int i = 0; i < RB; i++)
                if ((rmask >> i) & 1u) {
                    qgt_dev_op2_t x = d->prog[at];
                    x.ra = (uint8_t)(RL_REG_ + i);   /* the block's i-th register op acts on register bit i */
                    emit_u(b, t, &x, at);
                    at++;
                }
            /* generators not folded into a gate: applied after the block (they commute with it) */
            int ng = 0;
            for (int u = pc + 1; u <= pc + cnt; u++) ng += d->prog[u].gen != 0 && !folds_spawn(&d->prog[u]);
            if (ng) {
                sb_printf(b, "    switch (spawn) {\n");
                for (int u = pc + 1; u <= pc + cnt; u++)
                    if (d->prog[u].gen != 0 && !folds_spawn(&d->prog[u])) {
                        sb_printf(b, "    case %d: ", u);
                        emit_spawn(b, &d->prog[u]);
                        sb_printf(b, " break;\n");
                    }
                sb_printf(b, "    default: break;\n    }\n");
            }
            pc += cnt;
            continue;
        }
        switch (o->kind) {
        case Q2_U:
        case Q2_UR:
            emit_u(b, t, o, pc);
            break;
        case Q2_PHASE:
            if (o->coef < 0) break;
            if (o->ra >= RL_REG_ && o->ra < RL_WARP_) {
                sb_printf(b, "    { ");
                load_coef(b, t, o->coef, pc, QGEN_NONE);
                sb_printf(b, " phase_reg<%d, NR, T, R>(v, m); }\n", o->ra - RL_REG_);
            } else {
                sb_printf(b, "    { ");
                load_coef(b, t, o->coef, pc, QGEN_NONE);
                sb_printf(b, " const int bit = ");
                role_bit_expr(b, o->ra, o->q);
                sb_printf(b, "; const R pr = bit ? m[6] : m[0], pi = bit ? m[7] : m[1];\n"
                             "      if (!(pr == (R)1 && pi == (R)0)) {\n#pragma unroll\n"
                             "        for (int j = 0; j < NR; j++) v[j] = cm<T, R>(pr, pi, v[j]); } }\n");
            }
            break;
        case Q2_CZ:
            sb_printf(b, "    { const unsigned mk = role_mask<NR>(%d, %d, lane, warp, base) & role_mask<NR>(%d, %d, lane, warp, base);\n"
                         "      if (mk) {\n#pragma unroll\n        for (int j = 0; j < NR; j++) if ((mk >> j) & 1u) { v[j].x = -v[j].x; v[j].y = -v[j].y; } } }\n",
                      (int)o->ra, (int)o->q, (int)o->rb, (int)o->q2);
            break;
        case Q2_CNOT:
            sb_printf(b, "    { const unsigned cmask = role_mask<NR>(%d, %d, lane, warp, base);\n", (int)o->rb, (int)o->q2);
            if (o->ra >= RL_REG_)
                sb_printf(b, "      cnot_reg<%d, NR, T>(v, cmask); }\n", o->ra - RL_REG_);
            else
                sb_printf(b, "#pragma unroll\n      for (int j = 0; j < NR; j++) { T w = shfl_x<T>(v[j], 1 << %d); "
                             "if ((cmask >> j) & 1u) v[j] = w; } }\n", (int)o->ra);
            break;
        default:
            free(hsb.s);
            free(lsb.s);
            free(bsb.s);
            free(osb.s);
            free(tsb.s);
            free(t->coef);
            free(t->pc);
            free(t->gen);
            qgt_set_error(-1, "jit: op kind %d at %d not expected outside a block", (int)o->kind, pc);
            return NULL;
        }
        if (o->gen != 0 && (o->kind == Q2_U || o->kind == Q2_UR || o->kind == Q2_PHASE) && !folds_spawn(o)) {
            sb_printf(b, "    if (spawn == %d) { ", pc);
            emit_spawn(b, o);
            sb_printf(b, " }\n");
        }
    }
    /* store */
    sb_printf(b, "    {\n      T* dst = Vp + (long long)e[%d] * N;\n", (int)(offsetof(qgt_dev_entry_t, dst_row) / 4));
    sb_printf(b, "      if (flags & %d) {\n", QENT_STORE_V);
    for (int j = 0; j < NR; j++) sb_printf(b, "        dst[pthr + %uu] = v[%d];\n", pconst(d, &cur, j), j);
    /* row maximum of |v|: the largest squared magnitude, one square root per thread (sqrtf is
     * correctly rounded, hence monotonic: the same value as the largest of the roots) */
    sb_printf(b, "      }\n      if (flags & %d) {\n        float vmax = 0.f;\n#pragma unroll\n"
                 "        for (int j = 0; j < NR; j++) vmax = fmaxf(vmax, (float)(v[j].x * v[j].x + v[j].y * v[j].y));\n"
                 "        vmax = sqrtf(vmax);\n"
                 "        for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));\n"
                 "        if (lane == 0) atomicMax(rowmax + (long long)blockIdx.z * rowmax_stride + e[%d], __float_as_uint(vmax));\n"
                 "      }\n    }\n}\n",
              QENT_ROWMAX, (int)(offsetof(qgt_dev_entry_t, dst_row) / 4));
    /* assemble: slot table and program tables, head, entry points (tile loads), staging of the
     * slots (with the spawn folds), dispatch to the start, program */
    b = &osb;
    const int ns = t->n;
    sb_printf(b, "#define LDS8(m, s) { const float4 a_ = *reinterpret_cast<const float4*>(csm + 8 * (s)); "
                 "const float4 b_ = *reinterpret_cast<const float4*>(csm + 8 * (s) + 4); "
                 "m[0] = a_.x; m[1] = a_.y; m[2] = a_.z; m[3] = a_.w; m[4] = b_.x; m[5] = b_.y; m[6] = b_.z; m[7] = b_.w; }\n");
    if (ns > 0) {
        sb_printf(b, "static __constant__ int qslot_%s[%d] = {", d->kname, ns);
        for (int i = 0; i < ns; i++) sb_printf(b, "%s%d", i ? ", " : "", t->coef[i]);
        sb_printf(b, "};\n");
    }
    sb_printf(b, "%s", tsb.s ? tsb.s : "");
    sb_printf(b, "%s", hsb.s ? hsb.s : "");
    if (ns > 0) sb_printf(b, "    __shared__ __align__(16) float csm[%d];\n", 8 * ns);
    else sb_printf(b, "    const float* csm = ct;\n    (void)csm;\n");
    sb_printf(b, "%s", lsb.s ? lsb.s : "");
    sb_printf(b, "STG_:\n");
    if (ns > 0) {
        /* the slot whose gate this entry's derivative spawns at (fs, generator fg) is written by
         * thread 0 with the generator folded in; every other slot is copied as is; one barrier */
        int nf = 0;
        for (int i = 0; i < ns; i++) nf += t->gen[i] != QGEN_NONE;
        if (nf) {
            sb_printf(b, "    int fs = -1, fg = 0;\n    switch (spawn) {\n");
            for (int i = 0; i < ns; i++)
                if (t->gen[i] != QGEN_NONE) sb_printf(b, "    case %d: fs = %d; fg = %d; break;\n", t->pc[i], i, (int)t->gen[i]);
            sb_printf(b, "    default: break;\n    }\n");
            sb_printf(b, "    for (int i = threadIdx.x; i < %d; i += %d) if ((i >> 3) != fs) csm[i] = __ldg(ct + 8 * qslot_%s[i >> 3] + (i & 7));\n",
                      8 * ns, nthreads, d->kname);
            sb_printf(b, "    if (fs >= 0 && threadIdx.x == 0) {\n      float fm[8];\n"
                         "      for (int k = 0; k < 8; k++) fm[k] = __ldg(ct + 8 * qslot_%s[fs] + k);\n"
                         "      fold_gen(fm, fg);\n      for (int k = 0; k < 8; k++) csm[8 * fs + k] = fm[k];\n    }\n",
                      d->kname);
        } else {
            sb_printf(b, "    for (int i = threadIdx.x; i < %d; i += %d) csm[i] = __ldg(ct + 8 * qslot_%s[i >> 3] + (i & 7));\n",
                      8 * ns, nthreads, d->kname);
        }
        sb_printf(b, "    __syncthreads();\n");
    }
    sb_printf(b, "    switch (start) {\n");
    for (int i = 0; i < d->nstarts; i++) sb_printf(b, "    case %d: goto B_%d;\n", d->starts[i], d->starts[i]);
    sb_printf(b, "    default: return;\n    }\n");
    sb_printf(b, "%s", bsb.s ? bsb.s : "");
    const int err = hsb.err || lsb.err || bsb.err || osb.err || tsb.err || t->err;
    free(hsb.s);
    free(lsb.s);
    free(bsb.s);
    free(tsb.s);
    free(t->coef);
    free(t->pc);
    free(t->gen);
    if (err) {
        free(osb.s);
        qgt_set_error(-2, "jit: out of memory while writing the pass source");
        return NULL;
    }
    return osb.s;
}
