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

/* The part of input vector k that comes from the word number (x with its 5 low bits zero):
   runs of vector bits b0..b1 whose x bits descend (pos = P - b) come from one shift of the
   bit-reversed x; other bits one at a time. */
static void emit_var_high(Src *o, const TcSpec *s, int k)
{
    emit(o, "    const u64 vh%d = 0ull", k);
    int w = s->var_bits[k];
    for (int b0 = 0; b0 < w;) {
        int P = s->var_pos[k][b0] + b0, b1 = b0;
        while (b1 + 1 < w && s->var_pos[k][b1 + 1] == P - (b1 + 1))
            b1++;
        /* bit b of the vector = bit (63 - pos) = bit (63 - P + b) of brx */
        int sh = 63 - P;
        uint64_t mask = (b1 - b0 + 1 == 64 ? ~0ull : ((1ull << (b1 - b0 + 1)) - 1)) << b0;
        if (b1 > b0 && sh >= 0)
            emit(o, " | ((brx >> %d) & 0x%llxull)", sh, (unsigned long long)mask);
        else if (b1 > b0)
            emit(o, " | ((brx << %d) & 0x%llxull)", -sh, (unsigned long long)mask);
        else
            emit(o, " | (((xw >> %d) & 1ull) << %d)", s->var_pos[k][b0], b0);
        b0 = b1 + 1;
    }
    emit(o, ";\n");
}

/* The part of input vector k that comes from lane l (x bits 0..4). */
static uint64_t var_low(const TcSpec *s, int k, int l)
{
    uint64_t v = 0;
    for (int b = 0; b < s->var_bits[k]; b++)
        if (s->var_pos[k][b] < 5)
            v |= (uint64_t)((l >> s->var_pos[k][b]) & 1) << b;
    return v;
}

/* RPN for lane l into e[l] (and eh[l] when the left side is wider than 32 bits).  Every item
   gets its own variable t<i>; a compile-time stack holds the item numbers. */
static void emit_lane(Src *o, const TcSpec *s, int l, int narrow)
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
                 (unsigned long long)var_low(s, (int)v, l));
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

static void emit_word_function(Src *o, const TcGenEnum *g)
{
    const Program *a = g->a;
    size_t n = a->ninputs;
    emit(o, "TC_DEV u32 tc_word(const u64 word)\n{\n");
    /* input k is bit j = n-1-k of x = 32 word + lane: a lane pattern for j < 5, else bit j - 5
       of the word spread over all 32 lanes (a shift up to the sign bit and an arithmetic shift
       down: two instructions; words fit 32 bits up to 37 inputs) */
    if (n > 5 && n <= 37)
        emit(o, "    const u32 wlo = (u32)word;\n");
    for (size_t k = 0; k < n; k++) {
        int j = (int)(n - 1 - k);
        if (j < 5)
            emit(o, "    const u32 in%zu = TC_PAT%d;\n", k, j);
        else if (n <= 37)
            emit(o, "    const u32 in%zu = (u32)((int)(wlo << %d) >> 31);\n", k, 31 - (j - 5));
        else
            emit(o, "    const u32 in%zu = 0u - (u32)((word >> %d) & 1ull);\n", k, j - 5);
    }
    const TcSpec *s = g->spec;
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
        int luts = emit_luts(o, net, want, nwant);
        emit(o, "    // %d LOP3 for %zu + %zu NAND/STO instructions\n", luts, a->len,
             g->b ? g->b->len : (size_t)0);
        for (uint32_t c = 0; c < a->ncells; c++)
            node_name(val_a[c], sizeof val_a[c], net, cur_a[c]);
        for (uint32_t c = 0; g->mode == EN_EQUIV && c < g->b->ncells; c++)
            node_name(val_b[c], sizeof val_b[c], net, cur_b[c]);
        free(want);
        free(cur_a);
        free(cur_b);
        free(leaf);
        tc_net_free(net);
    } else {
        body(o, a, "a", a->inputs, n, g->ticks);
        if (g->mode == EN_EQUIV)
            body(o, g->b, "b", g->b_inputs, n, g->ticks);
        for (uint32_t c = 0; c < a->ncells; c++)
            snprintf(val_a[c], sizeof val_a[c], c == 0 ? "0u" : c == 1 ? "TC_ONES" : "a%u", c);
        for (uint32_t c = 0; g->mode == EN_EQUIV && c < g->b->ncells; c++)
            snprintf(val_b[c], sizeof val_b[c], c == 0 ? "0u" : c == 1 ? "TC_ONES" : "b%u", c);
    }
    if (g->mode == EN_SEARCH) {
        emit(o, "    u32 m = TC_ONES;\n");
        for (int b = 0; b < s->width; b++) {
            int bit = (int)((g->target >> b) & 1);
            emit(o, "    m &= %s%s;\n", bit ? "" : "~", val_a[s->out[b]]);
        }
    } else if (g->mode == EN_EQUIV) {
        emit(o, "    u32 m = 0u;\n");
        for (size_t k = 0; k < a->noutputs; k++)
            emit(o, "    m |= %s ^ %s;\n", val_a[a->outputs[k]],
                 val_b[g->b->outputs[g->out_map[k]]]);
    } else {
        int narrow = spec_fits_32(s);
        emit(o, "    const u64 xw = word << 5;\n");
        emit(o, "    const u64 brx = __brevll(xw);\n    (void)brx;\n");
        for (int k = 0; k < s->nvars; k++)
            emit_var_high(o, s, k);
        emit(o, "    u32 e[32];\n");
        if (!narrow)
            emit(o, "    u32 eh[32];\n");
        for (int l = 0; l < 32; l++)
            emit_lane(o, s, l, narrow);
        emit(o, "    tc_transpose32(e);\n");
        if (!narrow)
            emit(o, "    tc_transpose32(eh);\n");
        emit(o, "    u32 m = 0u;\n");
        for (int b = 0; b < s->width; b++)
            emit(o, "    m |= %s ^ %s[%d];\n", val_a[s->out[b]], b < 32 ? "e" : "eh", b & 31);
    }
    free(val_a);
    free(val_b);
    emit(o, "    return m;\n}\n");
}

/* The kernel template: each warp takes a contiguous run of the selected words (a multiple of 32),
   32 words per step, one per lane.  Words are selected in chunks of 1024 (64 passes of 512
   lanes, the reference's hand-out unit, src/enum.c:11), chunk c belonging to share c % parts
   (src/enum.c:232-234).  Hits are counted with popcount; the first 16 hits of each warp, which
   are its 16 smallest because the warp's words rise, are written to list[warp]. */
static const char *KERNEL =
    "#ifndef TC_HOST_EMULATION\n"
    "struct TcEnumArgs {\n"
    "    u64 words, space, per_warp;\n"
    "    u32 parts, part, nsel, pad;\n"
    "    u64 *hits;\n"
    "    u64 *list;\n"
    "    u32 *count;\n"
    "};\n"
    "extern \"C\" __global__ void __launch_bounds__(TC_BLOCK) tc_enum(const TcEnumArgs a)\n{\n"
    "    const u32 lane = threadIdx.x & 31u;\n"
    "    const u64 warp = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;\n"
    "    const u64 s0 = warp * a.per_warp;\n"
    "    const u64 s1 = s0 + a.per_warp < a.words ? s0 + a.per_warp : a.words;\n"
    "    u32 recorded = 0;\n"
    "    u64 hits = 0;\n"
    "    for (u64 s = s0; s < s1; s += 32) {\n"
    "        const u64 j = s >> 10;\n"
    "        const u64 chunk = a.nsel == a.parts ? j : (j / a.nsel) * a.parts + a.part + j % a.nsel;\n"
    "        const u64 word = (chunk << 10) | (s & 992u) | lane;  /* s is a multiple of 32 */\n"
    "        const u64 x0 = word << 5;\n"
    "        u32 valid = 0u;\n"
    "        if (s + lane < s1 && x0 < a.space)\n"
    "            valid = a.space - x0 >= 32u ? TC_ONES : (1u << (u32)(a.space - x0)) - 1u;\n"
    "        const u32 m = tc_word(word) & valid;\n"
    "        hits += __popc(m);\n"
    "        u32 any = __ballot_sync(TC_ONES, m != 0u);\n"
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
