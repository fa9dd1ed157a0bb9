/* The code generator: a NAND/STO program, and for verify its specification, become one CUDA
   kernel for sm_103a, compiled by NVRTC (engine.c).  This replaces the reference's x86 JIT
   (src/jit.c, src/x86.c); nothing of the x86 encoder carries over.

   Layout.  One thread evaluates one 32-bit word of lanes: lane l of word w is the assignment
   x = 32 w + l (the reference's numbering, src/enum.h:1-5, with 32 lanes per word instead of
   512 per line).  Input k of n is bit j = n-1-k of x: for j < 5 it is the constant lane pattern
   of bit j, for j >= 5 the word is all zeros or all ones from bit j-5 of w.

   The program body is straight-line C over u32 variables, one per cell plus RR.  NVVM turns the
   reassignments into SSA and ptxas keeps the live values in registers and fuses NAND chains into
   3-input LOP3 operations; a STO is a register rename and costs nothing.

   Comparison, per mode (src/enum.c:166-200):
     search  hit = AND over output bits of (target bit ? out : ~out), target folded in as a constant
     equiv   hit = OR over name-matched outputs of (a ^ b)
     verify  the right side is evaluated per lane in registers from x: the part of each input
             vector that comes from the word number is computed once per word, the lane part is a
             compile-time constant per lane (the 32 lanes are unrolled).  The 32 expected values are
             transposed into bit-sliced words with a 32x32 bit transpose (two byte-permute levels,
             three shift/select levels) and compared with the outputs word by word.
   The hit mask of each word is reduced by the kernel template: popcount for the count, a
   warp-ordered record of the first 16 hits per warp for the 16 smallest. */
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include "codegen.h"
#include "lutmap.h"

typedef struct {
    char  *s;
    size_t len, cap;
} Src;

static void emit(Src *o, const char *fmt, ...)
{
    for (;;) {
        va_list ap;
        va_start(ap, fmt);
        size_t room = o->cap - o->len;
        int k = vsnprintf(o->s ? o->s + o->len : NULL, room, fmt, ap);
        va_end(ap);
        if (k >= 0 && (size_t)k < room) {
            o->len += (size_t)k;
            return;
        }
        o->cap = o->cap ? 2 * o->cap + (size_t)k : 65536 + (size_t)k;
        o->s = tc_xrealloc(o->s, o->cap);
    }
}

/* ---- shared prelude ------------------------------------------------------------------------ */

static const char *PRELUDE =
    "typedef unsigned int u32;\n"
    "typedef unsigned long long u64;\n"
    "#define TC_ONES 0xffffffffu\n"
    "#ifndef TC_HOST_EMULATION\n"
    "#define TC_DEV __device__ __forceinline__\n"
    "#define TC_LOP3(d, a, b, c, tt) asm(\"lop3.b32 %0, %1, %2, %3, \" #tt \";\" "
    ": \"=r\"(d) : \"r\"(a), \"r\"(b), \"r\"(c))\n"
    "#else\n"
    "#define TC_DEV static inline\n"
    "#define TC_LOP3(d, a, b, c, tt) ((d) = tc_lop3_host((a), (b), (c), (tt)))\n"
    "static inline u32 tc_lop3_host(u32 a, u32 b, u32 c, u32 tt)\n{\n"
    "    u32 r = 0;\n"
    "    for (int k = 0; k < 8; k++)\n"
    "        if ((tt >> k) & 1)\n"
    "            r |= ((k & 4) ? a : ~a) & ((k & 2) ? b : ~b) & ((k & 1) ? c : ~c);\n"
    "    return r;\n}\n"
    "#endif\n"
    /* lane patterns: bit l of TC_PAT[j] is bit j of l */
    "#define TC_PAT0 0xaaaaaaaau\n#define TC_PAT1 0xccccccccu\n#define TC_PAT2 0xf0f0f0f0u\n"
    "#define TC_PAT3 0xff00ff00u\n#define TC_PAT4 0xffff0000u\n"
    /* select form of one transpose exchange: rows k and k+j, groups of 2j bits */
    "#define TC_XCH(a, b, j, m) do { u32 ta_ = ((a) >> (j)), tb_ = ((b) << (j)); "
    "(b) = ((b) & ~(m)) | (ta_ & (m)); (a) = ((a) & ~((m) << (j))) | (tb_ & ((m) << (j))); "
    "} while (0)\n"
    /* A[l] bit b -> A[b] bit l */
    "TC_DEV void tc_transpose32(u32 *A)\n{\n"
    "    for (int k = 0; k < 16; k++) { u32 x = A[k], y = A[k + 16];\n"
    "        A[k] = __byte_perm(x, y, 0x5410); A[k + 16] = __byte_perm(x, y, 0x7632); }\n"
    "    for (int k = 0; k < 32; k = ((k | 8) + 1) & ~8) { u32 x = A[k], y = A[k + 8];\n"
    "        A[k] = __byte_perm(x, y, 0x6240); A[k + 8] = __byte_perm(x, y, 0x7351); }\n"
    "    for (int k = 0; k < 32; k = ((k | 4) + 1) & ~4) TC_XCH(A[k], A[k + 4], 4, 0x0f0f0f0fu);\n"
    "    for (int k = 0; k < 32; k = ((k | 2) + 1) & ~2) TC_XCH(A[k], A[k + 2], 2, 0x33333333u);\n"
    "    for (int k = 0; k < 32; k = ((k | 1) + 1) & ~1) TC_XCH(A[k], A[k + 1], 1, 0x55555555u);\n"
    "}\n";

/* ---- the program body ---------------------------------------------------------------------- */

static void operand(Src *o, const char *pf, uint32_t a)
{
    if (a == CELL_ZERO)
        emit(o, "0u");
    else if (a == CELL_ONE)
        emit(o, "TC_ONES");
    else
        emit(o, "%s%u", pf, (unsigned)a);
}

/* Declares the cells of p (prefix pf), sets the inputs in_cells[k] from input word in<k>, and
   runs `ticks` passes. */
static void body(Src *o, const Program *p, const char *pf, const uint32_t *in_cells, size_t n,
                 unsigned ticks)
{
    emit(o, "    u32 %sr = 0u;\n", pf);
    for (uint32_t c = CELL_FIRST_FREE; c < p->ncells; c++)
        emit(o, "    u32 %s%u = 0u;\n", pf, (unsigned)c);
    for (size_t k = 0; k < n; k++)
        emit(o, "    %s%u = in%zu;\n", pf, (unsigned)in_cells[k], k);
    if (ticks > 1)
        emit(o, "#pragma unroll 1\n    for (u32 tick = 0; tick < %uu; tick++) {\n", ticks);
    for (size_t i = 0; i < p->len; i++) {
        Instr in = p->code[i];
        if (in.op == OP_NAND) {
            emit(o, "    %sr = ~(%sr & ", pf, pf);
            operand(o, pf, in.addr);
            emit(o, ");\n");
        } else if (in.addr >= CELL_FIRST_FREE) {
            emit(o, "    %s%u = %sr;\n", pf, (unsigned)in.addr, pf);
        }
    }
    if (ticks > 1)
        emit(o, "    }\n");
}

/* ---- the program body mapped onto LOP3 ----------------------------------------------------- */

typedef struct {
    TcNet *net;
    int   *order;
    int    norder;
} Mapped;

static void node_name(char *buf, size_t len, const TcNet *net, int node)
{
    const TcNode *x = tc_net_node(net, node);
    if (node == 0)
        snprintf(buf, len, "0u");
    else if (node == 1)
        snprintf(buf, len, "TC_ONES");
    else if (x->kind == TN_LEAF)
        snprintf(buf, len, "in%d", x->id);
    else
        snprintf(buf, len, "n%d", node);
}

/* Emits the chosen LUTs as lop3.b32 instructions; returns the count. */
static int emit_luts(Src *o, TcNet *net, const int *want, int nwant)
{
    int *order = tc_xmalloc(((size_t)tc_net_size(net) + 1) * sizeof *order), norder = 0;
    int luts = tc_net_map(net, want, nwant, order, &norder);
    for (int i = 0; i < norder; i++) {
        int leaves[3], nl;
        uint8_t tt;
        tc_net_lut(net, order[i], leaves, &nl, &tt);
        char a[32], b[32], c[32];
        node_name(a, sizeof a, net, leaves[0]);
        node_name(b, sizeof b, net, nl > 1 ? leaves[1] : 0);
        node_name(c, sizeof c, net, nl > 2 ? leaves[2] : 0);
        emit(o, "    u32 n%d; TC_LOP3(n%d, %s, %s, %s, 0x%02x);\n", order[i], order[i], a, b, c,
             (unsigned)tt);
    }
    free(order);
    return luts;
}

/* ---- the specification --------------------------------------------------------------------- */

/* Can the right side be computed on 32-bit words?  The low 32 bits of + - * & | ^ ~ neg and of a
   left shift by a constant depend only on the low 32 bits of the operands; a right shift or a
   shift by a computed amount does not. */
static int spec_fits_32(const TcSpec *s)
{
    if (s->width > 32)
        return 0;
    for (int i = 0; i < s->nrpn; i++) {
        if (s->rpn[i].op == TS_SHR)
            return 0;
        if (s->rpn[i].op == TS_SHL && (i == 0 || s->rpn[i - 1].op != TS_NUM))
            return 0;
    }
    return 1;
}

/* The part of input vector k that comes from the word number (y = 32 word + lane with its 5 low
   bits zero; x bit p of the assignment is y bit sigma[p]): runs of vector bits b0..b1 whose y bits
   descend (pos = P - b) come from one shift of the bit-reversed y; other bits one at a time. */
static void emit_var_high(Src *o, const TcSpec *s, int k, const int *sigma)
{
    emit(o, "    const u64 vh%d = 0ull", k);
    int w = s->var_bits[k];
    for (int b0 = 0; b0 < w;) {
        int P = sigma[s->var_pos[k][b0]] + b0, b1 = b0;
        while (b1 + 1 < w && sigma[s->var_pos[k][b1 + 1]] == P - (b1 + 1))
            b1++;
        /* bit b of the vector = bit (63 - pos) = bit (63 - P + b) of brx */
        int sh = 63 - P;
        uint64_t mask = (b1 - b0 + 1 == 64 ? ~0ull : ((1ull << (b1 - b0 + 1)) - 1)) << b0;
        if (b1 > b0 && sh >= 0)
            emit(o, " | ((brx >> %d) & 0x%llxull)", sh, (unsigned long long)mask);
        else if (b1 > b0)
            emit(o, " | ((brx << %d) & 0x%llxull)", -sh, (unsigned long long)mask);
        else
            emit(o, " | (((xw >> %d) & 1ull) << %d)", sigma[s->var_pos[k][b0]], b0);
        b0 = b1 + 1;
    }
    emit(o, ";\n");
}

/* The part of input vector k that comes from lane l (y bits 0..4). */
static uint64_t var_low(const TcSpec *s, int k, int l, const int *sigma)
{
    uint64_t v = 0;
    for (int b = 0; b < s->var_bits[k]; b++)
        if (sigma[s->var_pos[k][b]] < 5)
            v |= (uint64_t)((l >> sigma[s->var_pos[k][b]]) & 1) << b;
    return v;
}

/* RPN for lane l into e[l] (and eh[l] when the left side is wider than 32 bits).  Every item
   gets its own variable t<i>; a compile-time stack holds the item numbers. */
static void emit_lane(Src *o, const TcSpec *s, int l, int narrow, const int *sigma)
{
    const char *T = narrow ? "u32" : "u64";
    int st[TS_MAX_STACK + 2] = {0}, sp = 0;
    emit(o, "    {\n");
    for (int i = 0; i < s->nrpn; i++) {
        int op = s->rpn[i].op;
        uint64_t v = s->rpn[i].v;
        if (op == TS_NUM) {
            emit(o, "      const %s t%d = (%s)0x%llxull;\n", T, i, T, (unsigned long long)v);
            st[sp++] = i;
        } else if (op == TS_VAR) {
            emit(o, "      const %s t%d = (%s)(vh%d + 0x%llxull);\n", T, i, T, (int)v,
                 (unsigned long long)var_low(s, (int)v, l, sigma));
            st[sp++] = i;
        } else if (op == TS_NOT) {
            emit(o, "      const %s t%d = ~t%d;\n", T, i, st[sp - 1]);
            st[sp - 1] = i;
        } else if (op == TS_NEG) {
            emit(o, "      const %s t%d = (%s)0 - t%d;\n", T, i, T, st[sp - 1]);
            st[sp - 1] = i;
        } else {
            int a = st[sp - 2], b = st[sp - 1];
            switch (op) {
            case TS_ADD: emit(o, "      const %s t%d = t%d + t%d;\n", T, i, a, b); break;
            case TS_SUB: emit(o, "      const %s t%d = t%d - t%d;\n", T, i, a, b); break;
            case TS_MUL: emit(o, "      const %s t%d = t%d * t%d;\n", T, i, a, b); break;
            case TS_AND: emit(o, "      const %s t%d = t%d & t%d;\n", T, i, a, b); break;
            case TS_OR:  emit(o, "      const %s t%d = t%d | t%d;\n", T, i, a, b); break;
            case TS_XOR: emit(o, "      const %s t%d = t%d ^ t%d;\n", T, i, a, b); break;
            case TS_SHL:
                if (narrow)
                    emit(o, "      const u32 t%d = t%d < 32u ? t%d << t%d : 0u;\n", i, b, a, b);
                else
                    emit(o, "      const u64 t%d = t%d < 64ull ? t%d << t%d : 0ull;\n", i, b, a, b);
                break;
            default: /* TS_SHR, wide only */
                emit(o, "      const u64 t%d = t%d < 64ull ? t%d >> t%d : 0ull;\n", i, b, a, b);
                break;
            }
            sp--;
            st[sp - 1] = i;
        }
    }
    emit(o, "      e[%d] = (u32)t%d;\n", l, st[0]);
    if (!narrow)
        emit(o, "      eh[%d] = (u32)(t%d >> 32);\n", l, st[0]);
    emit(o, "    }\n");
}

/* ---- one enumeration kernel -------------------------------------------------------------- */

/* Where the assignment bits come from.  The kernel enumerates y = 32 word + lane: y bits 0..4 are
   the bit lane (constant patterns), 5..9 the thread's lane in its warp, 10..9+sb the 2^sb steps
   a warp takes through one stretch of a chunk of 1,024 words (sb = step_bits: 3, 4 or 5), the
   bits above that the stretch and the chunk.  Assignment x has y bit sigma[j] at its bit j
   (input k is x bit n-1-k).  Only the sb inputs on the step bits change from step to step: every
   LUT that depends on none of them is computed once per stretch (tc_outer) and kept in registers
   for its steps (tc_inner).  The identity puts x bits 10..9+sb there; when other inputs among x
   bits 0..9+sb leave more LUTs out of the steps (an array multiplier's last rows, say, whose
   inputs are the low x bits), sigma moves those onto the step bits and the x bits it displaces
   onto the lanes.  x bits 15 and up never move, so a chunk is the same set of assignments
   either way and the reference's --part shares hold. */
typedef struct {
    int      split;     /* 1: the stretch-invariant LUTs are hoisted */
    int      permuted;  /* 1: sigma is not the identity */
    int      sigma[64];
    uint64_t inner;     /* inputs (bit k) that change between steps */
    int      step_bits; /* a stretch of 2^step_bits steps shares the hoisted values */
} Layout;

#define SPLIT_MAX_FIELDS 64   /* values kept across the steps: registers */

static int popcount64(uint64_t v)
{
    int c = 0;
    for (; v; v &= v - 1)
        c++;
    return c;
}

/* LUTs of `order` that depend on no input of mask `vary`. */
static int invariant_luts(const uint64_t *sup, int norder, uint64_t vary)
{
    int c = 0;
    for (int i = 0; i < norder; i++)
        c += (sup[i] & vary) == 0;
    return c;
}

static uint64_t input_bit(size_t n, int j)  /* the input on x bit j */
{
    return 1ull << (n - 1 - (size_t)j);
}

/* Picks how many steps a stretch of words takes (2^sb, sb = 3, 4 or 5) and the sb inputs that
   change between them: for each sb, greedily the ones among x bits 0..9+sb that leave the most
   LUTs invariant (or the identity's, x bits 10..9+sb, if that is as good), then the sb whose
   estimated work per word is least: the LUTs that change per step, plus the invariant ones and
   `outer_extra` (what else runs once per stretch) spread over its 2^sb steps.  Measured on mul16
   with the spec hoisted: 2.64 ms per 2^32 at sb = 4, 2.67 at 3, 2.77 at 5; the estimate picks 4.
   force_sb (3..5) leaves the estimate out and takes that sb (the autotuner's candidates). */
static void choose_layout(Layout *L, size_t n, const uint64_t *sup, int norder, int outer_extra,
                          int force_sb)
{
    memset(L, 0, sizeof *L);
    for (int j = 0; j < 64; j++)
        L->sigma[j] = j;
    L->step_bits = 5;
    if (n < 13 || norder == 0)
        return;
    double best_cost = 0;
    uint64_t best_set = 0;
    int best_sb = 0, best_perm = 0;
    for (int sb = 5; sb >= 3; sb--) {
        const int top = 10 + sb;  /* x bits 0..top-1 may move */
        if ((int)n < top || (force_sb && sb != force_sb))
            continue;
        uint64_t id = 0, set = 0;
        for (int j = 10; j < top; j++)
            id |= input_bit(n, j);
        for (int step = 0; step < sb; step++) {
            int bj = -1, bc = -1;
            for (int j = 0; j < top; j++) {
                uint64_t m = input_bit(n, j);
                if (set & m)
                    continue;
                int c = invariant_luts(sup, norder, set | m);
                if (c > bc) {
                    bc = c;
                    bj = j;
                }
            }
            set |= input_bit(n, bj);
        }
        if (invariant_luts(sup, norder, set) <= invariant_luts(sup, norder, id))
            set = id;
        const int inv = invariant_luts(sup, norder, set);
        const double cost = (norder - inv) + (double)(inv + outer_extra) / (1 << sb);
        if (!best_sb || cost < best_cost) {
            best_cost = cost;
            best_set = set;
            best_sb = sb;
            best_perm = set != id;
        }
    }
    if (!best_sb)
        return;
    L->inner = best_set;
    L->step_bits = best_sb;
    if (!best_perm)
        return;
    /* x bits 0..9+sb: the chosen sb to y bits 10..9+sb, the rest in order to y bits 0..9 */
    int next_lane = 0, next_step = 10;
    for (int j = 0; j < 10 + best_sb; j++)
        L->sigma[j] = (best_set & input_bit(n, j)) ? next_step++ : next_lane++;
    L->permuted = 1;
}

/* Is the spec a sum of a part that depends on no step input and a part that depends on no bit-lane
   input (the x bits sigma puts on the step bits and on y bits 0..4)?  Then over a stretch's steps
   each lane's value is its value at step 0 plus a difference that is the same for all 32 lanes.  Sums,
   differences, negations and complements of such specs are such specs; a product or a left shift
   is one when neither factor has a bit-lane input while the other has a step input; a bitwise
   and, or or xor when its operands together have bit-lane or step inputs but not both. */
static int spec_separable(const TcSpec *s, const int *sigma, int step_bits, int *step_tz)
{
    /* tz: low bits known zero in the part that depends on step inputs (64: no such part) */
    int dl[TS_MAX_STACK + 2], ds[TS_MAX_STACK + 2], ok[TS_MAX_STACK + 2], tz[TS_MAX_STACK + 2];
    int sp = 0;
    for (int i = 0; i < s->nrpn; i++) {
        const int op = s->rpn[i].op;
        if (op == TS_NUM) {
            dl[sp] = ds[sp] = 0;
            tz[sp] = 64;
            ok[sp++] = 1;
        } else if (op == TS_VAR) {
            const int v = (int)s->rpn[i].v;
            dl[sp] = ds[sp] = 0;
            tz[sp] = 64;
            for (int b = 0; b < s->var_bits[v]; b++) {
                const int q = sigma[s->var_pos[v][b]];
                dl[sp] |= q < 5;
                if (q >= 10 && q < 10 + step_bits) {
                    ds[sp] = 1;
                    if (b < tz[sp])
                        tz[sp] = b;
                }
            }
            ok[sp++] = 1;
        } else if (op == TS_NOT || op == TS_NEG) {
            continue;
        } else if (op == TS_SHR || sp < 2) {
            return 0;
        } else {
            const int a = sp - 2, b = sp - 1;
            int k = ok[a] && ok[b], t = tz[a] < tz[b] ? tz[a] : tz[b];
            if (op == TS_MUL || op == TS_SHL) {
                k = k && !(dl[a] && ds[b]) && !(ds[a] && dl[b]);
                /* x * y: the step part is (step part of one) * (the other), so its low zeros are
                   at least the step part's; a left shift by a constant c adds c */
                t = ds[a] ? tz[a] : tz[b];
                if (op == TS_SHL && ds[a] && i > 0 && s->rpn[i - 1].op == TS_NUM)
                    t += (int)(s->rpn[i - 1].v < 64 ? s->rpn[i - 1].v : 64);
                if (ds[a] && ds[b])
                    t = 0;
            } else if (op == TS_AND || op == TS_OR || op == TS_XOR) {
                k = k && !((dl[a] || dl[b]) && (ds[a] || ds[b]));
                t = 0;  /* a bitwise part is not a sum: no known zeros claimed */
            }
            dl[a] |= dl[b];
            ds[a] |= ds[b];
            tz[a] = t > 64 ? 64 : t;
            ok[a] = k;
            sp--;
        }
    }
    *step_tz = sp == 1 ? tz[0] : 0;
    return sp == 1 && ok[0];
}

/* Input k as y bit q: a lane pattern for q < 5, else bit q - 5 of the word spread over all 32
   lanes (a shift up to the sign bit and an arithmetic shift down: two instructions; words fit
   32 bits up to 37 inputs). */
static void emit_input(Src *o, size_t k, size_t n, int q, const char *w32, const char *w64)
{
    if (q < 5)
        emit(o, "    const u32 in%zu = TC_PAT%d;\n", k, q);
    else if (n <= 37)
        emit(o, "    const u32 in%zu = (u32)((int)(%s << %d) >> 31);\n", k, w32, 31 - (q - 5));
    else
        emit(o, "    const u32 in%zu = 0u - (u32)((%s >> %d) & 1ull);\n", k, w64, q - 5);
}

static void emit_word_function(Src *o, const TcGenEnum *g)
{
    const Program *a = g->a;
    size_t n = a->ninputs;
    const TcSpec *s = g->spec;
    Layout L;
    memset(&L, 0, sizeof L);
    for (int j = 0; j < 64; j++)
        L.sigma[j] = j;
    L.step_bits = 5;
    Src outer = {0}, inner = {0}, fields = {0}, stores = {0}, loads = {0};
    int step_tz = 0;
    TcGenWork work = {0, 0, 1, -1};
    /* the cells compared, as (program, cell) pairs: a first */
    char (*val_a)[24] = tc_xcalloc(a->ncells + 1, sizeof *val_a);
    char (*val_b)[24] = tc_xcalloc((g->b ? g->b->ncells : 0) + 1, sizeof *val_b);
    if (g->ticks == 1 && !g->no_map) {
        TcNet *net = tc_net_new();
        int *leaf = tc_xmalloc((n + 1) * sizeof *leaf);
        for (size_t k = 0; k < n; k++)
            leaf[k] = tc_net_leaf(net, (int)k);
        int *cur_a = tc_xmalloc((a->ncells + 1) * sizeof *cur_a);
        int *cur_b = g->b ? tc_xmalloc((g->b->ncells + 1) * sizeof *cur_b) : NULL;
        tc_net_pass(net, a, a->inputs, n, leaf, cur_a);
        if (g->mode == EN_EQUIV)
            tc_net_pass(net, g->b, g->b_inputs, n, leaf, cur_b);
        int *want = tc_xmalloc(((size_t)a->noutputs * 2 + 65) * sizeof *want), nwant = 0;
        if (g->mode == EN_EQUIV)
            for (size_t k = 0; k < a->noutputs; k++) {
                want[nwant++] = cur_a[a->outputs[k]];
                want[nwant++] = cur_b[g->b->outputs[g->out_map[k]]];
            }
        else
            for (int bit = 0; bit < s->width; bit++)
                want[nwant++] = cur_a[s->out[bit]];
        const int size = tc_net_size(net);
        int *order = tc_xmalloc(((size_t)size + 1) * sizeof *order), norder = 0;
        const int luts = tc_net_map(net, want, nwant, order, &norder);
        /* the inputs each node depends on */
        uint64_t *nsup = tc_xcalloc((size_t)size + 1, sizeof *nsup);
        uint64_t *sup = tc_xmalloc(((size_t)norder + 1) * sizeof *sup);
        int (*lv)[3] = tc_xmalloc(((size_t)norder + 1) * sizeof *lv);
        uint8_t *tts = tc_xmalloc((size_t)norder + 1);
        for (size_t k = 0; k < n; k++)
            nsup[leaf[k]] = 1ull << k;
        for (int i = 0; i < norder; i++) {
            int nl;
            tc_net_lut(net, order[i], lv[i], &nl, &tts[i]);
            for (int q = nl; q < 3; q++)
                lv[i][q] = 0;
            nsup[order[i]] = nsup[lv[i][0]] | nsup[lv[i][1]] | nsup[lv[i][2]];
            sup[i] = nsup[order[i]];
        }
        /* once per stretch besides the LUTs: a verify's per-lane spec and transpose */
        const int outer_extra = g->mode == EN_VERIFY ? 64 * s->nrpn + 256 : 0;
        choose_layout(&L, n, sup, norder, outer_extra, g->step_bits);
        /* values of the chunk read by the steps: kept in TcInv */
        char *field = tc_xcalloc((size_t)size + 1, 1);
        int nfields = 0;
#define STEADY(nd) ((nsup[nd] & L.inner) == 0 && (nd) > 1 &&                                    \
                    !(tc_net_node(net, nd)->kind == TN_LEAF &&                                  \
                      L.sigma[n - 1 - (size_t)tc_net_node(net, nd)->id] < 5))
        for (int i = 0; i < norder; i++)
            for (int q = 0; q < 3 && (sup[i] & L.inner); q++)
                if (STEADY(lv[i][q]) && !field[lv[i][q]]) {
                    field[lv[i][q]] = 1;
                    nfields++;
                }
        for (int w = 0; w < nwant; w++)
            if (STEADY(want[w]) && !field[want[w]]) {
                field[want[w]] = 1;
                nfields++;
            }
#undef STEADY
        const int hoisted = invariant_luts(sup, norder, L.inner);
        L.split = L.inner && hoisted > 0 && 5 * hoisted >= norder &&
                  nfields <= SPLIT_MAX_FIELDS;
        work.luts_per_step = L.split ? norder - hoisted : norder;
        work.luts_per_stretch = L.split ? hoisted : 0;
        if (!L.split) {
            memset(field, 0, (size_t)size + 1);
            L.permuted = 0;
            L.step_bits = 5;
            for (int j = 0; j < 64; j++)
                L.sigma[j] = j;
        }
        for (size_t k = 0; k < n; k++) {
            const int q = L.sigma[n - 1 - k];
            if (!L.split || (L.inner >> k & 1)) {
                emit_input(&inner, k, n, q, "wlo", "word");
            } else {
                emit_input(&outer, k, n, q, "clo", "cword");
                if (q < 5)
                    emit_input(&inner, k, n, q, "wlo", "word");
            }
        }
        for (int i = 0; i < norder; i++) {
            char x[32], y[32], z[32];
            node_name(x, sizeof x, net, lv[i][0]);
            node_name(y, sizeof y, net, lv[i][1]);
            node_name(z, sizeof z, net, lv[i][2]);
            emit(L.split && !(sup[i] & L.inner) ? &outer : &inner,
                 "    u32 n%d; TC_LOP3(n%d, %s, %s, %s, 0x%02x);\n", order[i], order[i], x, y, z,
                 (unsigned)tts[i]);
        }
        for (int nd = 0; nd <= size; nd++)
            if (field[nd]) {
                char f[32];
                node_name(f, sizeof f, net, nd);
                emit(&fields, " u32 %s;", f);
                emit(&stores, "    v->%s = %s;\n", f, f);
                emit(&loads, "    const u32 %s = v->%s;\n", f, f);
            }
        emit(&inner, "    // %d LOP3 for %zu + %zu NAND/STO instructions, %d of them once per stretch\n",
             luts, a->len, g->b ? g->b->len : (size_t)0, L.split ? hoisted : 0);
        for (uint32_t c = 0; c < a->ncells; c++)
            node_name(val_a[c], sizeof val_a[c], net, cur_a[c]);
        for (uint32_t c = 0; g->mode == EN_EQUIV && c < g->b->ncells; c++)
            node_name(val_b[c], sizeof val_b[c], net, cur_b[c]);
        free(field);
        free(tts);
        free(lv);
        free(sup);
        free(nsup);
        free(order);
        free(want);
        free(cur_a);
        free(cur_b);
        free(leaf);
        tc_net_free(net);
    } else {
        for (size_t i = 0; i < a->len; i++)
            work.luts_per_step += (a->code[i].op == OP_NAND) * (int)g->ticks;
        for (size_t i = 0; g->mode == EN_EQUIV && i < g->b->len; i++)
            work.luts_per_step += (g->b->code[i].op == OP_NAND) * (int)g->ticks;
        for (size_t k = 0; k < n; k++)
            emit_input(&inner, k, n, (int)(n - 1 - k), "wlo", "word");
        body(&inner, a, "a", a->inputs, n, g->ticks);
        if (g->mode == EN_EQUIV)
            body(&inner, g->b, "b", g->b_inputs, n, g->ticks);
        for (uint32_t c = 0; c < a->ncells; c++)
            snprintf(val_a[c], sizeof val_a[c], c == 0 ? "0u" : c == 1 ? "TC_ONES" : "a%u", c);
        for (uint32_t c = 0; g->mode == EN_EQUIV && c < g->b->ncells; c++)
            snprintf(val_b[c], sizeof val_b[c], c == 0 ? "0u" : c == 1 ? "TC_ONES" : "b%u", c);
    }
    work.compare_ops = g->mode == EN_SEARCH ? s->width : g->mode == EN_EQUIV ? (int)a->noutputs
                                                                            : -1;
    if (g->mode == EN_SEARCH) {
        emit(&inner, "    u32 m = TC_ONES;\n");
        for (int b = 0; b < s->width; b++) {
            int bit = (int)((g->target >> b) & 1);
            emit(&inner, "    m &= %s%s;\n", bit ? "" : "~", val_a[s->out[b]]);
        }
    } else if (g->mode == EN_EQUIV) {
        emit(&inner, "    u32 m = 0u;\n");
        for (size_t k = 0; k < a->noutputs; k++)
            emit(&inner, "    m |= %s ^ %s;\n", val_a[a->outputs[k]],
                 val_b[g->b->outputs[g->out_map[k]]]);
    } else if (spec_fits_32(s) && spec_separable(s, L.sigma, L.step_bits, &step_tz)) {
        /* once per stretch: every lane's value at step 0, bit-sliced (32 words kept), and lane 0's;
           each step: lane 0's value now minus at step 0 is every lane's difference d, added to
           the bit-sliced values with one carry chain over the bits, each sum bit compared at once */
        emit(&outer, "    const u64 xw = cword << 5;\n");
        emit(&outer, "    const u64 brx = __brevll(xw);\n    (void)brx;\n");
        for (int k = 0; k < s->nvars; k++)
            emit_var_high(&outer, s, k, L.sigma);
        emit(&outer, "    u32 e[32];\n");
        for (int l = 0; l < 32; l++)
            emit_lane(&outer, s, l, 1, L.sigma);
        emit(&outer, "    const u32 sf0 = e[0];\n");
        emit(&outer, "    tc_transpose32(e);\n");
        emit(&fields, " u32 sf0;");
        emit(&stores, "    v->sf0 = sf0;\n");
        emit(&loads, "    const u32 sf0 = v->sf0;\n");
        for (int b = 0; b < s->width; b++) {
            emit(&outer, "    const u32 sp%d = e[%d];\n", b, b);
            emit(&fields, " u32 sp%d;", b);
            emit(&stores, "    v->sp%d = sp%d;\n", b, b);
            emit(&loads, "    const u32 sp%d = v->sp%d;\n", b, b);
        }
        emit(&inner, "    const u64 xw = word << 5;\n");
        emit(&inner, "    const u64 brx = __brevll(xw);\n    (void)brx;\n");
        for (int k = 0; k < s->nvars; k++)
            emit_var_high(&inner, s, k, L.sigma);
        emit(&inner, "    u32 e[1];\n");
        emit_lane(&inner, s, 0, 1, L.sigma);
        emit(&inner, "    const u32 d = e[0] - sf0;\n");
        emit(&inner, "    u32 m = 0u, c = 0u;\n    (void)c;\n    (void)d;\n");
        /* below bit step_tz, d is known to be zero: no carry, the sum bit is the kept one */
        work.compare_ops = 0;
        for (int b = 0; b < s->width; b++) {
            /* below step_tz: one XOR-OR; above: the sign spread of d's bit (2 ops), a 4-input
               XOR-OR (2) and, but for the top bit, the carry's majority (1) */
            work.compare_ops += b < step_tz ? 1 : b + 1 < s->width ? 5 : 4;
            if (b < step_tz) {
                emit(&inner, "    m |= %s ^ sp%d;\n", val_a[s->out[b]], b);
                continue;
            }
            emit(&inner, "    {\n      const u32 q = (u32)((int)(d << %d) >> 31);\n", 31 - b);
            emit(&inner, "      m |= %s ^ sp%d ^ q ^ c;\n", val_a[s->out[b]], b);
            if (b + 1 < s->width)
                emit(&inner, "      c = (sp%d & q) | (sp%d & c) | (q & c);\n", b, b);
            emit(&inner, "    }\n");
        }
    } else {
        int narrow = spec_fits_32(s);
        emit(&inner, "    const u64 xw = word << 5;\n");
        emit(&inner, "    const u64 brx = __brevll(xw);\n    (void)brx;\n");
        for (int k = 0; k < s->nvars; k++)
            emit_var_high(&inner, s, k, L.sigma);
        emit(&inner, "    u32 e[32];\n");
        if (!narrow)
            emit(&inner, "    u32 eh[32];\n");
        for (int l = 0; l < 32; l++)
            emit_lane(&inner, s, l, narrow, L.sigma);
        emit(&inner, "    tc_transpose32(e);\n");
        if (!narrow)
            emit(&inner, "    tc_transpose32(eh);\n");
        emit(&inner, "    u32 m = 0u;\n");
        for (int b = 0; b < s->width; b++)
            emit(&inner, "    m |= %s ^ %s[%d];\n", val_a[s->out[b]], b < 32 ? "e" : "eh", b & 31);
    }
    free(val_a);
    free(val_b);
    work.stretch_steps = 1 << L.step_bits;
    if (!work.luts_per_stretch)
        work.stretch_steps = 1;
    if (g->work)
        *g->work = work;
    /* what a chunk computes once (cword: the word with its step bits, 5..9, zero), what each step
       computes, and the two together for one word */
    emit(o, "typedef struct {%s } TcInv;\n", fields.len ? fields.s : " u32 unused_;");
    emit(o, "TC_DEV void tc_outer(const u64 cword, TcInv *v)\n{\n");
    emit(o, "    const u32 clo = (u32)cword;\n    (void)clo;\n    (void)v;\n");
    emit(o, "%s%s}\n", outer.len ? outer.s : "", stores.len ? stores.s : "");
    emit(o, "TC_DEV u32 tc_inner(const u64 word, const TcInv *v)\n{\n");
    emit(o, "    const u32 wlo = (u32)word;\n    (void)wlo;\n    (void)v;\n");
    emit(o, "%s%s    return m;\n}\n", loads.len ? loads.s : "", inner.s);
    /* a stretch: 2^TC_STEP_BITS steps of 32 words, word bits 5 .. 4 + TC_STEP_BITS */
    emit(o, "#define TC_STEP_BITS %d\n#define TC_STEP_MASK ((32ull << TC_STEP_BITS) - 32ull)\n",
         L.step_bits);
    emit(o, "TC_DEV u32 tc_word(const u64 word)\n{\n    TcInv v;\n"
            "    tc_outer(word & ~TC_STEP_MASK, &v);\n    return tc_inner(word, &v);\n}\n");
    /* y -> x: the assignment a hit at y stands for */
    emit(o, "#define TC_PERMUTED %d\n", L.permuted);
    emit(o, "TC_DEV u64 tc_unperm(const u64 y)\n{\n");
    if (!L.permuted) {
        emit(o, "    return y;\n}\n");
    } else {
        uint64_t fixed = 0;
        for (size_t j = 0; j < 64; j++)
            if (j >= n || L.sigma[j] == (int)j)
                fixed |= 1ull << j;
        emit(o, "    u64 x = y & 0x%llxull;\n", (unsigned long long)fixed);
        for (size_t j = 0; j < n; j++)
            if (L.sigma[j] != (int)j)
                emit(o, "    x |= ((y >> %d) & 1ull) << %zu;\n", L.sigma[j], j);
        emit(o, "    return x;\n}\n");
    }
    free(outer.s);
    free(inner.s);
    free(fields.s);
    free(stores.s);
    free(loads.s);
}

/* The kernel template: each warp takes a contiguous run of the selected words (a multiple of 32),
   32 words per step, one per lane.  Words are selected in chunks of 1024 (64 passes of 512
   lanes, the reference's hand-out unit, src/enum.c:11), chunk c belonging to share c % parts
   (src/enum.c:232-234); a stretch's invariant LUTs are computed once before its steps.  Hits
   are counted with popcount; each warp's 16 smallest hits go to list[warp]: its first 16 when
   the order is the identity (the warp's assignments rise), else a sorted insertion. */
static const char *KERNEL =
    "#ifndef TC_HOST_EMULATION\n"
    "struct TcEnumArgs {\n    "
    TC_TEXT(TC_ENUM_ARGS_FIELDS(u64, u32))
    "\n};\n"
    "extern \"C\" __global__ void __launch_bounds__(TC_BLOCK) tc_enum(const TcEnumArgs a)\n{\n"
    "    const u32 lane = threadIdx.x & 31u;\n"
    "    const u64 warp = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;\n"
    "    const u64 s0 = warp * a.per_warp;\n"
    "    const u64 s1 = s0 + a.per_warp < a.words ? s0 + a.per_warp : a.words;\n"
    "    u32 recorded = 0;\n"
    "    u64 hits = 0, thr = ~0ull;  /* thr: the 16th smallest hit kept so far */\n"
    "    (void)thr;\n"
    "    for (u64 s = s0; s < s1;) {\n"
    "        const u64 j = s >> 10;\n"
    "        const u64 chunk = a.nsel == a.parts ? j : (j / a.nsel) * a.parts + a.part + j % a.nsel;\n"
    "        const u64 span = 32ull << TC_STEP_BITS;  /* words of a stretch */\n"
    "        const u64 cbase = (chunk << 10) | (s & 992u & ~TC_STEP_MASK) | lane;\n"
    "        const u64 s_end = (s / span + 1) * span < s1 ? (s / span + 1) * span : s1;\n"
    "        TcInv inv;\n"
    "        tc_outer(cbase, &inv);  /* what stays the same for the stretch's steps */\n"
    "        for (; s < s_end; s += 32) {\n"
    "        const u64 word = cbase | (s & TC_STEP_MASK);  /* s is a multiple of 32 */\n"
    "        const u64 x0 = word << 5;\n"
    "        u32 valid = 0u;\n"
    "        if (s + lane < s1 && x0 < a.space)\n"
    "            valid = a.space - x0 >= 32u ? TC_ONES : (1u << (u32)(a.space - x0)) - 1u;\n"
    "        const u32 m = tc_inner(word, &inv) & valid;\n"
    "        hits += __popc(m);\n"
    "        u32 any = __ballot_sync(TC_ONES, m != 0u);\n"
    "#if TC_PERMUTED\n"
    "        /* the warp's assignments do not come in order: keep its 16 smallest, sorted.  A lane's\n"
    "           hits rise with their bit (the bit lanes take x bits in order), so its smallest is\n"
    "           its lowest bit; the warp's smallest goes in while it beats the 16th kept. */\n"
    "        if (any) {\n"
    "            const u64 bx = tc_unperm(x0);\n"
    "            u32 mm = m;\n"
    "            for (;;) {\n"
    "                const u64 mine = mm ? bx | tc_unperm((u64)(__ffs(mm) - 1)) : ~0ull;\n"
    "                u64 least = mine;\n"
    "                for (int d = 16; d > 0; d >>= 1) {\n"
    "                    const u64 other = __shfl_xor_sync(TC_ONES, least, d);\n"
    "                    least = other < least ? other : least;\n"
    "                }\n"
    "                if (least == ~0ull || (recorded == 16u && least >= thr))\n"
    "                    break;\n"
    "                if (lane == 0) {\n"
    "                    u64 *L = a.list + warp * 16u;\n"
    "                    u32 i = recorded < 16u ? recorded : 15u;\n"
    "                    while (i > 0 && L[i - 1] > least) {\n"
    "                        L[i] = L[i - 1];\n"
    "                        i--;\n"
    "                    }\n"
    "                    L[i] = least;\n"
    "                }\n"
    "                recorded = recorded < 16u ? recorded + 1u : 16u;\n"
    "                u64 t = 0;\n"
    "                if (lane == 0 && recorded == 16u)\n"
    "                    t = a.list[warp * 16u + 15u];\n"
    "                thr = __shfl_sync(TC_ONES, t, 0);\n"
    "                if (mine == least)\n"
    "                    mm &= mm - 1u;\n"
    "            }\n"
    "        }\n"
    "#else\n"
    "        while (any && recorded < 16u) {\n"
    "            const int src = __ffs(any) - 1;\n"
    "            u32 mm = __shfl_sync(TC_ONES, m, src);\n"
    "            const u64 xb = __shfl_sync(TC_ONES, x0, src);\n"
    "            while (mm && recorded < 16u) {\n"
    "                if (lane == 0)\n"
    "                    a.list[warp * 16u + recorded] = xb + (u64)(__ffs(mm) - 1);\n"
    "                recorded++;\n"
    "                mm &= mm - 1u;\n"
    "            }\n"
    "            any &= any - 1u;\n"
    "        }\n"
    "#endif\n"
    "        }\n"
    "    }\n"
    "    for (int d = 16; d > 0; d >>= 1)\n"
    "        hits += __shfl_xor_sync(TC_ONES, hits, d);\n"
    "    if (lane == 0) {\n"
    "        a.count[warp] = recorded;\n"
    "        if (hits)\n"
    "            atomicAdd(a.hits, hits);\n"
    "    }\n"
    "}\n"
    "#endif\n";

char *tc_codegen_enum(const TcGenEnum *g, size_t *len)
{
    Src o = {0};
    emit(&o, "// generated by the tesseract GB300 engine: %s over %zu inputs, %u tick(s)\n",
         g->mode == EN_VERIFY ? "verify" : g->mode == EN_EQUIV ? "equiv" : "search",
         g->a->ninputs, g->ticks);
    emit(&o, "#define TC_BLOCK %d\n", g->block);
    emit(&o, "%s", PRELUDE);
    emit_word_function(&o, g);
    emit(&o, "%s", KERNEL);
    if (len)
        *len = o.len;
    return o.s;
}

/* ---- truth tables (run --table) ------------------------------------------------------------ */

/* CUDA C for `tc_table`: thread w runs rows 32w .. 32w + 31 of program p from the reset state
   (input k of n is bit n-1-k of the row: the first .in cell is the high bit), `ticks` passes,
   and stores each output column's word at out[col * words + w]; with no .out cells the one
   column is RR (src/main.c:219-258). */
char *tc_codegen_table(const Program *p, unsigned ticks, int block, size_t *len)
{
    Src o = {0};
    size_t n = p->ninputs;
    emit(&o, "// generated by the tesseract GB300 engine: truth table over %zu inputs, %u tick(s)\n",
         n, ticks);
    emit(&o, "#define TC_BLOCK %d\n", block);
    emit(&o, "%s", PRELUDE);
    emit(&o, "extern \"C\" __global__ void __launch_bounds__(TC_BLOCK) tc_table(u32 *out, "
             "const u64 words)\n{\n");
    emit(&o, "    const u64 word = (u64)blockIdx.x * blockDim.x + threadIdx.x;\n");
    emit(&o, "    if (word >= words)\n        return;\n");
    for (size_t k = 0; k < n; k++) {
        int j = (int)(n - 1 - k);
        if (j < 5)
            emit(&o, "    const u32 in%zu = TC_PAT%d;\n", k, j);
        else
            emit(&o, "    const u32 in%zu = 0u - (u32)((word >> %d) & 1ull);\n", k, j - 5);
    }
    char (*val)[24] = tc_xcalloc(p->ncells + 2, sizeof *val);
    if (ticks == 1 && p->noutputs) {
        TcNet *net = tc_net_new();
        int *leaf = tc_xmalloc((n + 1) * sizeof *leaf);
        for (size_t k = 0; k < n; k++)
            leaf[k] = tc_net_leaf(net, (int)k);
        int *cur = tc_xmalloc((p->ncells + 1) * sizeof *cur);
        tc_net_pass(net, p, p->inputs, n, leaf, cur);
        int *want = tc_xmalloc((p->noutputs + 1) * sizeof *want);
        for (size_t i = 0; i < p->noutputs; i++)
            want[i] = cur[p->outputs[i]];
        int luts = emit_luts(&o, net, want, (int)p->noutputs);
        emit(&o, "    // %d LOP3 for %zu NAND/STO instructions\n", luts, p->len);
        for (uint32_t c = 0; c < p->ncells; c++)
            node_name(val[c], sizeof val[c], net, cur[c]);
        free(want);
        free(cur);
        free(leaf);
        tc_net_free(net);
    } else {
        body(&o, p, "a", p->inputs, n, ticks);
        for (uint32_t c = 0; c < p->ncells; c++)
            snprintf(val[c], sizeof val[c], c == 0 ? "0u" : c == 1 ? "TC_ONES" : "a%u", c);
        snprintf(val[p->ncells], sizeof val[p->ncells], "ar");
    }
    if (p->noutputs)
        for (size_t i = 0; i < p->noutputs; i++)
            emit(&o, "    out[%zuull * words + word] = %s;\n", i, val[p->outputs[i]]);
    else
        emit(&o, "    out[word] = %s;\n", val[p->ncells]);
    emit(&o, "}\n");
    free(val);
    if (len)
        *len = o.len;
    return o.s;
}
