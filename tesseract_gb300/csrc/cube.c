/* The cube on the GPU: programs with id and link cells over 2^dims machines (dims 9..16), the
   replacement of LaneCube + jit_cube_run (src/lanes.c:341-415, src/jit.c:526-560, 775-793), and
   cuda_check, the replacement of check_lanes (src/check.c:52-113).

   Layout.  Machine m is bit m % 32 of word m / 32; the device holds cell c of every machine as
   W = 2^dims / 32 consecutive words (mem[c * W + w]) and RR as W more.  Per group of 512 machines
   this is exactly the reference's Line layout (lane k at bit k % 64 of u64 word k / 64), so a
   group's lines copy in and out with one strided copy.

   A word (32 machines) runs through straight-line generated code, LOP3-mapped: a kernel's
   written cells are shared out over up to tc_cube_groups warps of a block, each computing the
   cone of its share from the cells' values loaded at the kernel's start, so a cube of 2,048
   words (Life on 65,536 machines) runs on up to 512 warps instead of 64.  A
   read across a link from machine m reaches machine m ^ M:
     M bits 0..4   move lanes inside the word (bit swaps, byte permutes, a 16-bit rotate)
     M bits 5..9   another lane of the same warp: __shfl_xor_sync on the register
     M bits 10..15 another warp: a load of that word from the cell's memory
   Warps do not run in lockstep, so the pass is cut into segments as src/jit.c:526-560 cuts it
   for groups: wherever a segment would both write a cell and read it across a dimension of 10 or
   more, unless the value read can be computed again by the reading warp from cells the segment
   does not write (then it is: a Life board's halo corners).  Each segment is its own kernel
   launch; inside a segment every far load sees the value the cell had when the segment started,
   which is what lockstep shows it.  A segment longer than tc_cube_chunk
   instructions is split into equal kernels of at most tc_cube_piece that hand their cells over
   through memory, so no single kernel is too large for the compiler.  When the whole pass is one kernel and no
   read crosses warps (at most 1024 machines), the passes loop inside the kernel.

   A pass that ends in a segment of plain copies A <- B (a Life board taking its next generation
   from the cells it was computed into) runs without that segment: every kernel is compiled twice,
   the second time with the memory of each A and its B exchanged, and the passes alternate between
   the two.  After a pass without the copies A's value is in B's memory, which is where the other
   variant reads A; B's own memory is free because every pass writes B before reading it.  The
   last pass of a run includes the copy kernels (in its variant), so the state is as the program
   leaves it whenever the host looks. */
#include <pthread.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include "codegen.h"
#include "engine.h"
#include "lutmap.h"
#include "ref_host.h"

#define TC_CUBE_BLOCK 32
#define FAR_DIM 10

/* 1: cube kernels are LOP3-mapped networks (lutmap.c); 0: the instructions as written */
int tc_cube_map = 1;
/* the most warps per word a mapped kernel splits its written cells over, and the fewest cells a
   warp gets */
int tc_cube_groups = 32;
int tc_cube_min_cells = 16;
/* warps per block of a group-major kernel (0: never group-major) */
int tc_cube_gm_warps = 4;
/* 1: a pass's closing copies are left out of all but a run's last pass (two memory variants) */
int tc_cube_copy_swap = 1;
/* 1: far reads of computed cells are recomputed where they can be, instead of cutting */
int tc_cube_recompute = 1;
/* (node, mask) visits the recomputations of one segment may take in all: a bound on the code
   recomputing adds to one kernel, which cannot be split (Life on 65,536 machines takes under 6,000;
   the NTT product on 2,048 machines wanted over 300,000 and made one kernel of 400,000 LOP3 that
   compiled for minutes, against 8 kernels of at most 170,000 with cuts) */
int tc_cube_recompute_budget = 65536;
/* the most instructions in one kernel: longer segments are split.  Fewer, longer kernels win
   once they are split over warps (Life on 65,536 machines: 3 kernels of up to 125,722
   instructions run 36-38k generations/s, 13 kernels of 12,000 run 29k), at the price of a longer
   compile (7 s against 0.5 s) */
int tc_cube_chunk = 140000;
/* a segment too long for one kernel is split into equal kernels of at most this many
   instructions: they compile in parallel, and NVRTC's time grows faster than a kernel's length
   (the NTT product on 512 machines, 272,001 instructions: 2 kernels took 85 s to compile, 6 take
   13.5 s) */
int tc_cube_piece = 50000;

struct CudaCube {
    Program     p;
    unsigned    dims, groups, W, machines;
    uint32_t   *mem, *rr;   /* device */
    size_t     *first;      /* kernel k runs instructions first[k] .. first[k + 1] - 1 */
    unsigned    nk, nseg, isa_seg;
    int         loop;       /* one kernel, passes loop inside it */
    unsigned    copy_k0;    /* kernels copy_k0.. are the pass's closing copies (nk: none) */
    uint32_t   *slot1;      /* with copies: cell -> memory of the second variant (A <-> B) */
    unsigned    variants;   /* 2 with copies, else 1 */
    cudaKernel_t *fn;       /* variant v's kernel k at fn[v * nk + k] */
    unsigned    *warps;     /* warp groups of kernel k */
    int         *gmajor;    /* kernel k is group-major (one group per block) */
    cudaGraphExec_t graph;
    unsigned    graph_passes;
    unsigned    iters;      /* runs of words each group-major block walks (cuda_cube_tune) */
    unsigned    gmw;        /* warps per group-major block (cuda_cube_tune) */
};

struct CudaCode {
    CudaCube *cube;
};

/* ---- the plan --------------------------------------------------------------------------------- */

/* The cuts of a pass into segments, as late as possible: a new segment starts wherever a cell the
   segment has written is read across dimension far_dim or up, or a cell it has read that way is
   written.  The ISA's rule (docs/ISA.md, step 7f) uses far_dim = 9; this engine needs far_dim =
   FAR_DIM only, since dimensions 0..9 stay inside one warp's 1,024 machines, which run in
   lockstep.  Returns the number of segments; first[n] = len. */
static unsigned find_cuts(const Program *p, size_t *first, unsigned far_dim)
{
    uint32_t *stored = tc_xcalloc(p->ncells + 1, sizeof *stored);
    uint32_t *read = tc_xcalloc(p->ncells + 1, sizeof *read);
    uint32_t seg = 1;
    unsigned n = 0;
    first[n++] = 0;
    for (size_t i = 0; i < p->len; i++) {
        Instr in = p->code[i];
        if (in.op == OP_NAND) {
            unsigned mask;
            uint32_t a = tc_program_resolve(p, in.addr, &mask);
            if ((mask >> far_dim) && !tc_program_readonly(p, a)) {
                if (stored[a] == seg) {
                    seg++;
                    first[n++] = i;
                }
                read[a] = seg;
            }
        } else if (!tc_program_readonly(p, in.addr)) {
            if (read[in.addr] == seg) {
                seg++;
                first[n++] = i;
            }
            stored[in.addr] = seg;
        }
    }
    first[n] = p->len;
    free(stored);
    free(read);
    return n;
}

/* Cuts with far reads of computed cells recomputed.  find_cuts ends a segment where a cell it has
   written is read across a far dimension, because another warp's copy of that cell may not be
   written yet.  But when the value read is a function of cells the segment never writes (and of
   id cells and constants), the reading warp can compute it itself from the other machine's cells:
   their memory holds the same values all through the segment.  So such a read does not cut; the
   cells the recomputation reads count as read across a far dimension (a later write to one cuts).

   The values of a segment form a DAG: start values of cells, id patterns, RR's start value,
   NANDs, and reads of a value in another machine (a link: that node at machine ^ mask).  A far
   read of a computed cell is recomputable when its node, evaluated at machine ^ mask, reaches
   only start values of cells not written so far in the segment, ids and constants (not RR's
   start value), in at most RECOMPUTE_LIMIT (node, mask) visits, and the segment's
   recomputations stay within tc_cube_recompute_budget visits in all.  flags[s] is set for segments that recompute; their code must be
   generated as one kernel (the recomputation starts from the segment's start values). */
enum { V_CONST, V_START, V_ID, V_RR0, V_NAND, V_LINK };
#define RECOMPUTE_LIMIT 4096

typedef struct {
    uint8_t  *kind;
    int32_t  *a, *b;      /* NAND: fanins; LINK: a = node, b = mask; START: a = cell; CONST: a */
    size_t    n, cap;
    /* the visit of one recomputability check */
    uint64_t *seen;       /* (node, mask) pairs, open addressing; 0 = empty */
    size_t    nseen, capseen;
    uint32_t *reads;      /* cells whose start values the recomputation reads */
    size_t    nreads, capreads;
    const uint32_t *stored;  /* per cell: the last segment that wrote it */
    uint32_t  seg;
} Dag;

static int32_t dag_add(Dag *g, uint8_t kind, int32_t a, int32_t b)
{
    if (g->n == g->cap) {
        g->cap = g->cap ? 2 * g->cap : 4096;
        g->kind = tc_xrealloc(g->kind, g->cap);
        g->a = tc_xrealloc(g->a, g->cap * sizeof *g->a);
        g->b = tc_xrealloc(g->b, g->cap * sizeof *g->b);
    }
    g->kind[g->n] = kind;
    g->a[g->n] = a;
    g->b[g->n] = b;
    return (int32_t)g->n++;
}

/* 1: a new (node, mask) pair; 0: seen before; -1: over the limit */
static int dag_visit(Dag *g, int32_t v, unsigned mask)
{
    uint64_t key = ((uint64_t)(uint32_t)v << 20 | mask) + 1;
    if (g->nseen >= RECOMPUTE_LIMIT)
        return -1;
    if (2 * (g->nseen + 1) > g->capseen) {
        size_t cap = g->capseen ? 2 * g->capseen : 1024;
        uint64_t *t = tc_xcalloc(cap, sizeof *t);
        for (size_t i = 0; i < g->capseen; i++)
            if (g->seen[i]) {
                size_t h = (size_t)(g->seen[i] * 0x9E3779B97F4A7C15ull) & (cap - 1);
                while (t[h])
                    h = (h + 1) & (cap - 1);
                t[h] = g->seen[i];
            }
        free(g->seen);
        g->seen = t;
        g->capseen = cap;
    }
    size_t h = (size_t)(key * 0x9E3779B97F4A7C15ull) & (g->capseen - 1);
    while (g->seen[h]) {
        if (g->seen[h] == key)
            return 0;
        h = (h + 1) & (g->capseen - 1);
    }
    g->seen[h] = key;
    g->nseen++;
    return 1;
}

static int dag_recomputable(Dag *g, int32_t v, unsigned mask)
{
    int fresh = dag_visit(g, v, mask);
    if (fresh <= 0)
        return fresh == 0;
    switch (g->kind[v]) {
    case V_CONST:
    case V_ID:
        return 1;
    case V_RR0:
        return 0;
    case V_START:
        if (g->stored[g->a[v]] == g->seg)  /* written since: its memory has moved on */
            return 0;
        if (g->nreads == g->capreads) {
            g->capreads = g->capreads ? 2 * g->capreads : 64;
            g->reads = tc_xrealloc(g->reads, g->capreads * sizeof *g->reads);
        }
        g->reads[g->nreads++] = (uint32_t)g->a[v];
        return 1;
    case V_LINK:
        return dag_recomputable(g, g->a[v], mask ^ (unsigned)g->b[v]);
    default:
        return dag_recomputable(g, g->a[v], mask) && dag_recomputable(g, g->b[v], mask);
    }
}

static unsigned find_cuts_recompute(const Program *p, size_t *first, unsigned char *flags)
{
    uint32_t *stored = tc_xcalloc(p->ncells + 1, sizeof *stored);
    uint32_t *read = tc_xcalloc(p->ncells + 1, sizeof *read);
    int32_t *cur = tc_xmalloc((p->ncells + 1) * sizeof *cur);
    uint32_t *cur_seg = tc_xcalloc(p->ncells + 1, sizeof *cur_seg);  /* cur[c] valid in seg */
    Dag g = {0};
    int32_t zero = dag_add(&g, V_CONST, 0, 0), one = dag_add(&g, V_CONST, 1, 0);
    uint32_t seg = 1;
    unsigned n = 0;
    size_t spent = 0;  /* visits of this segment's recomputations */
    int32_t rr = dag_add(&g, V_RR0, 0, 0);
    first[n] = 0;
    flags[n++] = 0;
#define CELL_NODE(c)                                                                               (cur_seg[c] == seg ? cur[c] : (cur_seg[c] = seg, cur[c] = dag_add(&g, V_START, (int32_t)(c), 0)))
    for (size_t i = 0; i < p->len; i++) {
        Instr in = p->code[i];
        if (in.op == OP_NAND) {
            unsigned mask;
            uint32_t a = tc_program_resolve(p, in.addr, &mask);
            int32_t v;
            if (a == CELL_ZERO || a == CELL_ONE) {
                v = a == CELL_ONE ? one : zero;
            } else if (p->special && p->special[a].kind == CK_ID) {
                v = dag_add(&g, V_ID, 0, 0);
            } else if (mask >> FAR_DIM && stored[a] == seg) {
                g.nseen = 0;
                g.nreads = 0;
                g.stored = stored;
                g.seg = seg;
                if (g.seen)
                    memset(g.seen, 0, g.capseen * sizeof *g.seen);
                if (dag_recomputable(&g, cur[a], mask) &&
                    spent + g.nseen <= (size_t)tc_cube_recompute_budget) {
                    spent += g.nseen;
                    for (size_t k = 0; k < g.nreads; k++)
                        read[g.reads[k]] = seg;
                    flags[n - 1] = 1;
                    v = dag_add(&g, V_LINK, cur[a], (int32_t)mask);
                } else {  /* a new segment: the value is read from memory there */
                    seg++;
                    spent = 0;
                    rr = dag_add(&g, V_RR0, 0, 0);
                    first[n] = i;
                    flags[n++] = 0;
                    read[a] = seg;
                    v = dag_add(&g, V_LINK, CELL_NODE(a), (int32_t)mask);
                }
            } else {
                if (mask >> FAR_DIM && !tc_program_readonly(p, a))
                    read[a] = seg;
                int32_t src = CELL_NODE(a);
                v = mask ? dag_add(&g, V_LINK, src, (int32_t)mask) : src;
            }
            /* NAND with 0 is 1 whatever RR was (the usual start of a gate) */
            rr = v == zero || rr == zero ? one
                 : v == one && rr == one ? zero
                                         : dag_add(&g, V_NAND, rr, v);
        } else if (!tc_program_readonly(p, in.addr)) {
            if (read[in.addr] == seg) {
                seg++;
                spent = 0;
                rr = dag_add(&g, V_RR0, 0, 0);
                first[n] = i;
                flags[n++] = 0;
            }
            stored[in.addr] = seg;
            cur_seg[in.addr] = seg;
            cur[in.addr] = rr;
        }
    }
#undef CELL_NODE
    first[n] = p->len;
    free(stored);
    free(read);
    free(cur);
    free(cur_seg);
    free(g.kind);
    free(g.a);
    free(g.b);
    free(g.seen);
    free(g.reads);
    return n;
}

/* The segments the engine runs: with mapped kernels, far reads of computed cells are recomputed
   where they can be (flags[s] set for those segments); else the plain rule. */
static unsigned plan_cuts(const Program *p, size_t *cuts, unsigned char *flags)
{
    if (tc_cube_map && tc_cube_recompute)
        return find_cuts_recompute(p, cuts, flags);
    unsigned n = find_cuts(p, cuts, FAR_DIM);
    memset(flags, 0, n);
    return n;
}

/* The closing copies of a pass, if the last segment (from `cut`, moved back over the NANDs that
   compute RR for its first store) is only that: loads of plain cells (NAND ZERO, NAND B,
   NAND ONE: RR = B) each stored into a cell A (A <- B), no B written and no A read in it, every B
   copied to one A.  And for the memory exchange to be sound, before it: the pass starts by
   setting RR (NAND ZERO), and every B is written before anything reads it, so what a pass finds
   in B's memory (A's value of the pass before, in the other variant) is never seen.  On success *from is where the copies start
   and slot1 the second variant's memory map (A and B exchanged, the rest in place). */
static int copy_tail(const Program *p, size_t cut, uint32_t *slot1, size_t *from_out)
{
    size_t from = cut;
    while (from > 0 && from <= p->len && p->code[from - 1].op == OP_NAND)
        from--;
    if (from == 0 || from >= p->len || p->code[0].op != OP_NAND)
        return 0;
    unsigned mask;
    if (tc_program_resolve(p, p->code[0].addr, &mask) != CELL_ZERO)
        return 0;
    uint32_t n = p->ncells;
    uint32_t *src = tc_xcalloc(n + 1, sizeof *src);     /* A -> B + 1 */
    uint32_t *dst = tc_xcalloc(n + 1, sizeof *dst);     /* B -> A + 1 */
    unsigned char *touch = tc_xcalloc(n + 1, 1);        /* 1 read, 2 written (in the tail) */
    int ok = 1, copies = 0;
    enum { RR_OTHER, RR_ONE, RR_CELL, RR_NOT_CELL } rr = RR_OTHER;
    uint32_t rc = 0;
    for (size_t i = from; i < p->len && ok; i++) {
        Instr in = p->code[i];
        if (in.op == OP_NAND) {
            uint32_t c = tc_program_resolve(p, in.addr, &mask);
            if (c == CELL_ZERO) {
                rr = RR_ONE;
            } else if (c == CELL_ONE) {
                rr = rr == RR_CELL ? RR_NOT_CELL : rr == RR_NOT_CELL ? RR_CELL : RR_OTHER;
            } else if (rr == RR_ONE && mask == 0 && !tc_program_readonly(p, c) &&
                       !(p->special && p->special[c].kind != CK_PLAIN) && touch[c] != 2) {
                rr = RR_NOT_CELL;
                rc = c;
                touch[c] = 1;
            } else {
                ok = 0;
            }
        } else if (!tc_program_readonly(p, in.addr)) {
            uint32_t a = in.addr;
            if (rr != RR_CELL || touch[a] || (p->special && p->special[a].kind != CK_PLAIN) ||
                (dst[rc] && dst[rc] != a + 1)) {
                ok = 0;
            } else {
                src[a] = rc + 1;
                dst[rc] = a + 1;
                touch[a] = 2;
                copies++;
            }
        }
    }
    /* the rest of the pass: every B written before it is read */
    unsigned char *first = tc_xcalloc(n + 1, 1);  /* 1 read first, 2 written first */
    for (size_t i = 0; i < from && ok; i++) {
        Instr in = p->code[i];
        if (in.op == OP_NAND) {
            uint32_t c = tc_program_resolve(p, in.addr, &mask);
            if (!first[c])
                first[c] = 1;
        } else if (!tc_program_readonly(p, in.addr) && !first[in.addr]) {
            first[in.addr] = 2;
        }
    }
    for (uint32_t b = 0; b < n && ok; b++)
        if (dst[b] && first[b] != 2)
            ok = 0;
    ok = ok && copies > 0;
    *from_out = from;
    if (ok) {
        for (uint32_t c = 0; c < n; c++)
            slot1[c] = c;
        for (uint32_t a = 0; a < n; a++)
            if (src[a]) {
                slot1[a] = src[a] - 1;
                slot1[src[a] - 1] = a;
            }
    }
    free(src);
    free(dst);
    free(touch);
    free(first);
    return ok;
}

/* ---- code generation ------------------------------------------------------------------------ */

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

static const char *CUBE_PRELUDE =
    "typedef unsigned int u32;\n"
    "#define TC_ONES 0xffffffffu\n"
    "#define TC_FULL 0xffffffffu\n"
    "#define TC_LOP3(d, a, b, c, tt) asm(\"lop3.b32 %0, %1, %2, %3, \" #tt \";\" "
    ": \"=r\"(d) : \"r\"(a), \"r\"(b), \"r\"(c))\n"
    /* lane k of the word reads lane k ^ mask (mask < 32): swap blocks of 1, 2, 4, 8, 16 lanes */
    "__device__ __forceinline__ u32 tc_perm(u32 v, const u32 mask)\n{\n"
    "    if (mask & 1u) v = ((v & 0x55555555u) << 1) | ((v >> 1) & 0x55555555u);\n"
    "    if (mask & 2u) v = ((v & 0x33333333u) << 2) | ((v >> 2) & 0x33333333u);\n"
    "    if (mask & 4u) v = ((v & 0x0f0f0f0fu) << 4) | ((v >> 4) & 0x0f0f0f0fu);\n"
    "    if (mask & 8u) v = __byte_perm(v, 0u, 0x2301);\n"
    "    if (mask & 16u) v = __funnelshift_l(v, v, 16);\n"
    "    return v;\n}\n";

/* The word of id cell bit d for machines 32 w .. 32 w + 31 */
static void id_word(Src *o, unsigned d, unsigned flip)
{
    static const char *pat[5] = {"0xaaaaaaaau", "0xccccccccu", "0xf0f0f0f0u", "0xff00ff00u",
                                 "0xffff0000u"};
    if (d < 5)
        emit(o, "%s%s", flip ? "~" : "", pat[d]);
    else
        emit(o, "(%s(0u - ((w >> %uu) & 1u)))", flip ? "~" : "", d - 5);
}

typedef struct {
    const Program *p;
    unsigned       W;
    unsigned char *loaded, *written;
    const uint32_t *slot;  /* cell -> where its words are in memory (NULL: the cell itself) */
    int            bad;    /* a far read of a computed cell that cannot be recomputed */
} Chunk;

static unsigned slot_of(const Chunk *k, uint32_t c)
{
    return (unsigned)(k->slot ? k->slot[c] : c);
}

static void use_cell(Src *o, Chunk *k, uint32_t c)
{
    if (!k->loaded[c]) {
        emit(o, "    u32 c%u = m[%uu * W];\n", (unsigned)c, slot_of(k, c));
        k->loaded[c] = 1;
    }
}

/* Emits the NAND operand expression for cell a (declaring loads first). */
static void operand(Src *o, Chunk *k, uint32_t a, char *expr, size_t len)
{
    const Program *p = k->p;
    unsigned mask;
    uint32_t c = tc_program_resolve(p, a, &mask);
    if (c == CELL_ZERO || c == CELL_ONE) {
        snprintf(expr, len, "%s", c == CELL_ONE ? "TC_ONES" : "0u");
        return;
    }
    if (p->special && p->special[c].kind == CK_ID) {
        Src t = {0};
        unsigned d = p->special[c].dim;
        id_word(&t, d, (mask >> d) & 1);
        snprintf(expr, len, "%s", t.s);
        free(t.s);
        return;
    }
    unsigned hi = mask >> 5, lo = mask & 31;
    char v[96];
    if (hi == 0) {
        use_cell(o, k, c);
        snprintf(v, sizeof v, "c%u", (unsigned)c);
    } else if (hi < 32) {
        use_cell(o, k, c);
        snprintf(v, sizeof v, "__shfl_xor_sync(TC_FULL, c%u, %uu)", (unsigned)c, hi);
    } else {
        snprintf(v, sizeof v, "mem[%uu * W + (w ^ %uu)]", slot_of(k, c), hi);
    }
    if (lo)
        snprintf(expr, len, "tc_perm(%s, %uu)", v, lo);
    else
        snprintf(expr, len, "%s", v);
}

static void chunk_body(Src *o, Chunk *k, size_t from, size_t to)
{
    const Program *p = k->p;
    char expr[160];
    for (size_t i = from; i < to; i++) {
        Instr in = p->code[i];
        if (in.op == OP_NAND) {
            operand(o, k, in.addr, expr, sizeof expr);
            emit(o, "    r = ~(r & %s);\n", expr);
        } else if (!tc_program_readonly(p, in.addr)) {
            if (!k->loaded[in.addr]) {
                emit(o, "    u32 c%u;\n", (unsigned)in.addr);
                k->loaded[in.addr] = 1;
            }
            emit(o, "    c%u = r;\n", (unsigned)in.addr);
            k->written[in.addr] = 1;
        }
    }
}

/* The chunk's instructions as a NAND network mapped onto LOP3.  Leaves: every cell's value at
   the start of the chunk (variable c<cell>), RR (variable r), id patterns, and link reads: a
   read across dimensions 0..9 is an opaque leaf computed from the source cell's value at that
   instruction (which is then kept in the cover), a read across 10 and up a load of the
   segment-start value. */
typedef struct {
    char         **expr;  /* per node: the expression of a leaf, or NULL */
    int           *cell;  /* per node: the cell whose start value the leaf is, else -1 */
    int           *src;   /* per node: the node a near link read takes its value from, else -1 */
    unsigned char *far;   /* per node: a far load */
    int           *fcell; /* per node: a far load's cell, else -1 */
    int           *mask;  /* per node: a link read's mask (near or far) */
    int           *idd;   /* per node: an id pattern's dimension, else -1 */
    unsigned char *flip;  /* per node: an id pattern complemented */
    size_t         n, cap;
} Leaves;

static int leaf(TcNet *net, Leaves *L, const char *expr)
{
    int id = (int)L->n;
    int node = tc_net_leaf(net, id);
    if ((size_t)node >= L->cap) {
        size_t cap = L->cap ? 2 * L->cap : 256;
        while (cap <= (size_t)node)
            cap *= 2;
        L->expr = tc_xrealloc(L->expr, cap * sizeof *L->expr);
        L->cell = tc_xrealloc(L->cell, cap * sizeof *L->cell);
        L->src = tc_xrealloc(L->src, cap * sizeof *L->src);
        L->far = tc_xrealloc(L->far, cap);
        L->fcell = tc_xrealloc(L->fcell, cap * sizeof *L->fcell);
        L->mask = tc_xrealloc(L->mask, cap * sizeof *L->mask);
        L->idd = tc_xrealloc(L->idd, cap * sizeof *L->idd);
        L->flip = tc_xrealloc(L->flip, cap);
        for (size_t i = L->cap; i < cap; i++) {
            L->expr[i] = NULL;
            L->cell[i] = L->src[i] = L->fcell[i] = L->idd[i] = -1;
            L->mask[i] = 0;
            L->far[i] = L->flip[i] = 0;
        }
        L->cap = cap;
    }
    L->expr[node] = tc_xstrdup(expr);
    L->n++;
    return node;
}

static int is_leaf(const Leaves *L, int node)
{
    return node >= 0 && (size_t)node < L->cap && L->expr[node];
}

static void name_of(char *buf, size_t len, int node)
{
    if (node == 0)
        snprintf(buf, len, "0u");
    else if (node == 1)
        snprintf(buf, len, "TC_ONES");
    else
        snprintf(buf, len, "n%d", node);
}

typedef struct {
    TcNet  *net;
    Leaves  L;
    int    *cur, *start;         /* per cell: its value's node now, its start-value leaf (or -1) */
    int     rr;                  /* RR's node at the end */
    int    *order, norder, luts; /* the chosen LUTs in topological order */
    unsigned char *mapped;       /* per node: a chosen LUT */
} ChunkNet;

/* A far read of a cell the kernel has computed, recomputed from the other machine's start values
   (find_cuts_recompute allows it only where that works: start values of cells the segment does
   not write, ids, constants).  rc_node(v, M) is node v evaluated at machine ^ M, built into the
   network; memo holds the (node, mask) pairs done. */
typedef struct {
    Chunk    *k;
    TcNet    *net;
    Leaves   *L;
    int      *cur, *start;
    uint64_t *key;
    int      *val;
    size_t    n, cap;
} Recompute;

static int *rc_find(Recompute *r, uint64_t key, int add)
{
    if (add && 2 * (r->n + 1) > r->cap) {
        size_t cap = r->cap ? 2 * r->cap : 1024;
        uint64_t *k2 = tc_xcalloc(cap, sizeof *k2);
        int *v2 = tc_xmalloc(cap * sizeof *v2);
        for (size_t i = 0; i < r->cap; i++)
            if (r->key[i]) {
                size_t h = (size_t)(r->key[i] * 0x9E3779B97F4A7C15ull) & (cap - 1);
                while (k2[h])
                    h = (h + 1) & (cap - 1);
                k2[h] = r->key[i];
                v2[h] = r->val[i];
            }
        free(r->key);
        free(r->val);
        r->key = k2;
        r->val = v2;
        r->cap = cap;
    }
    if (!r->cap)
        return NULL;
    size_t h = (size_t)(key * 0x9E3779B97F4A7C15ull) & (r->cap - 1);
    while (r->key[h]) {
        if (r->key[h] == key)
            return &r->val[h];
        h = (h + 1) & (r->cap - 1);
    }
    if (!add)
        return NULL;
    r->key[h] = key;
    r->n++;
    return &r->val[h];
}

/* cell c's start value at machine ^ M */
static int rc_start(Recompute *r, uint32_t c, unsigned M)
{
    Leaves *L = r->L;
    char buf[160], src[96], nm[32];
    if (r->start[c] < 0) {
        snprintf(buf, sizeof buf, "c%u", (unsigned)c);
        r->start[c] = leaf(r->net, L, buf);
        L->cell[r->start[c]] = (int)c;
        if (r->cur[c] < 0)
            r->cur[c] = r->start[c];
    }
    int sl = r->start[c];
    unsigned hi = M >> 5, lo = M & 31;
    if (M == 0)
        return sl;
    int from = -1;
    if (hi >= 32) {
        snprintf(src, sizeof src, "mem[%uu * W + (w ^ %uu)]", slot_of(r->k, c), hi);
    } else {
        from = sl;
        name_of(nm, sizeof nm, sl);
        if (hi)
            snprintf(src, sizeof src, "__shfl_xor_sync(TC_FULL, %s, %uu)", nm, hi);
        else
            snprintf(src, sizeof src, "%s", nm);
    }
    if (lo)
        snprintf(buf, sizeof buf, "tc_perm(%s, %uu)", src, lo);
    else
        snprintf(buf, sizeof buf, "%s", src);
    int v = leaf(r->net, L, buf);
    L->src[v] = from;
    L->far[v] = hi >= 32;
    L->fcell[v] = hi >= 32 ? (int)c : -1;
    L->mask[v] = (int)M;
    return v;
}

static int rc_node(Recompute *r, int v, unsigned M)
{
    uint64_t key = ((uint64_t)(unsigned)v << 16 | M) + 1;
    int *hit = rc_find(r, key, 0);
    if (hit)
        return *hit;
    const TcNode nd = *tc_net_node(r->net, v);
    Leaves *L = r->L;
    int out = -1;
    if (nd.kind == TN_CONST) {
        out = v;
    } else if (nd.kind == TN_NAND) {
        int a = rc_node(r, nd.a, M), b = rc_node(r, nd.b, M);
        out = a < 0 || b < 0 ? -1 : tc_net_nand(r->net, a, b);
    } else if (nd.kind == TN_NOT) {
        int a = rc_node(r, nd.a, M);
        out = a < 0 ? -1 : tc_net_not(r->net, a);
    } else if (L->cell[v] >= 0) {
        out = rc_start(r, (uint32_t)L->cell[v], M);
    } else if (L->idd[v] >= 0) {
        unsigned d = (unsigned)L->idd[v], flip = L->flip[v] ^ ((M >> d) & 1);
        Src t = {0};
        id_word(&t, d, flip);
        out = leaf(r->net, L, t.s);
        L->idd[out] = (int)d;
        L->flip[out] = (unsigned char)flip;
        free(t.s);
    } else if (L->far[v]) {
        out = rc_start(r, (uint32_t)L->fcell[v], M ^ (unsigned)L->mask[v]);
    } else if (L->src[v] >= 0) {
        out = rc_node(r, L->src[v], M ^ (unsigned)L->mask[v]);
    }
    if (out >= 0)
        *rc_find(r, key, 1) = out;
    return out;
}

/* Builds and maps the network of instructions from .. to-1 (marks the cells written). */
static void chunk_net(Chunk *k, size_t from, size_t to, ChunkNet *cn)
{
    const Program *p = k->p;
    memset(cn, 0, sizeof *cn);
    TcNet *net = cn->net = tc_net_new();
    Leaves *L = &cn->L;
    int *cur = cn->cur = tc_xmalloc((p->ncells + 1) * sizeof *cur);
    int *start = cn->start = tc_xmalloc((p->ncells + 1) * sizeof *start);
    int *need = tc_xmalloc(((to - from) + p->ncells + 4) * sizeof *need), nneed = 0;
    char buf[160];
    for (uint32_t c = 0; c < p->ncells; c++)
        cur[c] = start[c] = -1;
    cur[CELL_ZERO] = 0;
    cur[CELL_ONE] = 1;
    int rr = leaf(net, L, "r");
    Recompute rc = {k, net, L, cur, start, NULL, NULL, 0, 0};
    for (size_t i = from; i < to; i++) {
        Instr in = p->code[i];
        if (in.op != OP_NAND) {
            if (!tc_program_readonly(p, in.addr)) {
                cur[in.addr] = rr;
                k->written[in.addr] = 1;
            }
            continue;
        }
        unsigned mask;
        uint32_t c = tc_program_resolve(p, in.addr, &mask);
        int v;
        if (c == CELL_ZERO || c == CELL_ONE) {
            v = (int)c;
        } else if (p->special && p->special[c].kind == CK_ID) {
            Src t = {0};
            unsigned d = p->special[c].dim;
            id_word(&t, d, (mask >> d) & 1);
            v = leaf(net, L, t.s);
            L->idd[v] = (int)d;
            L->flip[v] = (unsigned char)((mask >> d) & 1);
            free(t.s);
        } else if ((mask >> 5) >= 32 && k->written[c]) {
            /* a far read of a value this kernel computed: computed again for the other machine */
            v = rc_node(&rc, cur[c], mask);
            if (v < 0) {  /* cannot happen after find_cuts_recompute: fail the compile */
                k->bad = 1;
                v = 0;
            }
        } else {
            unsigned hi = mask >> 5, lo = mask & 31;
            if (hi < 32 && cur[c] < 0) {  /* first use: the value loaded at the chunk start */
                snprintf(buf, sizeof buf, "c%u", (unsigned)c);
                cur[c] = start[c] = leaf(net, L, buf);
                L->cell[cur[c]] = (int)c;
            }
            if (hi == 0 && lo == 0) {
                v = cur[c];
            } else {
                char src[96];
                int from_node = -1;
                if (hi >= 32) {
                    snprintf(src, sizeof src, "mem[%uu * W + (w ^ %uu)]", slot_of(k, c), hi);
                } else {
                    from_node = cur[c];
                    need[nneed++] = cur[c];  /* the source value must exist as a register */
                    char nm[32];
                    name_of(nm, sizeof nm, cur[c]);
                    if (hi)
                        snprintf(src, sizeof src, "__shfl_xor_sync(TC_FULL, %s, %uu)", nm, hi);
                    else
                        snprintf(src, sizeof src, "%s", nm);
                }
                if (lo)
                    snprintf(buf, sizeof buf, "tc_perm(%s, %uu)", src, lo);
                else
                    snprintf(buf, sizeof buf, "%s", src);
                v = leaf(net, L, buf);
                L->src[v] = from_node;
                L->far[v] = hi >= 32;
                L->fcell[v] = hi >= 32 ? (int)c : -1;
                L->mask[v] = (int)mask;
            }
        }
        rr = tc_net_nand(net, rr, v);
    }
    free(rc.key);
    free(rc.val);
    cn->rr = rr;
    for (uint32_t c = CELL_FIRST_FREE; c < p->ncells; c++)
        if (k->written[c])
            need[nneed++] = cur[c];
    need[nneed++] = rr;
    int n = tc_net_size(net);
    cn->order = tc_xmalloc(((size_t)n + 1) * sizeof *cn->order);
    cn->luts = tc_net_map(net, need, nneed, cn->order, &cn->norder);
    cn->mapped = tc_xcalloc((size_t)n + 1, 1);
    for (int i = 0; i < cn->norder; i++)
        cn->mapped[cn->order[i]] = 1;
    free(need);
}

static void chunk_net_free(ChunkNet *cn)
{
    for (size_t i = 0; i < cn->L.cap; i++)
        free(cn->L.expr[i]);
    free(cn->L.expr);
    free(cn->L.cell);
    free(cn->L.src);
    free(cn->L.far);
    free(cn->L.fcell);
    free(cn->L.mask);
    free(cn->L.idd);
    free(cn->L.flip);
    free(cn->order);
    free(cn->mapped);
    free(cn->cur);
    free(cn->start);
    tc_net_free(cn->net);
}

static void emit_lut(Src *o, const ChunkNet *cn, int node, const char *indent)
{
    int lv[3], nl;
    uint8_t tt;
    tc_net_lut(cn->net, node, lv, &nl, &tt);
    char a[32], b[32], c[32];
    name_of(a, sizeof a, lv[0]);
    name_of(b, sizeof b, nl > 1 ? lv[1] : 0);
    name_of(c, sizeof c, nl > 2 ? lv[2] : 0);
    emit(o, "%su32 n%d; TC_LOP3(n%d, %s, %s, %s, 0x%02x);\n", indent, node, node, a, b, c,
         (unsigned)tt);
}

/* Marks in in_cone the nodes warp group needs for `outs` (and RR when own_rr). */
static void cone_of(const ChunkNet *cn, const uint32_t *outs, int nouts, int own_rr,
                    unsigned char *in_cone, int *stack)
{
    int n = tc_net_size(cn->net);
    memset(in_cone, 0, (size_t)n + 1);
    int sp = 0;
    for (int i = 0; i < nouts; i++)
        stack[sp++] = cn->cur[outs[i]];
    if (own_rr)
        stack[sp++] = cn->rr;
    while (sp) {
        int v = stack[--sp];
        if (v < 2 || in_cone[v])
            continue;
        in_cone[v] = 1;
        if (is_leaf(&cn->L, v)) {
            if (cn->L.src[v] >= 0)
                stack[sp++] = cn->L.src[v];
            continue;
        }
        int lv[3], nl;
        uint8_t tt;
        tc_net_lut(cn->net, v, lv, &nl, &tt);
        for (int j = 0; j < nl; j++)
            stack[sp++] = lv[j];
    }
}

/* One warp group's code in a split kernel: the cone of `outs` (cells, plus RR when own_rr) in
   node order.  Every load comes first (start values and far reads, all in flight at once), then
   with `barrier` a barrier of the whole block, then the LUTs with each cell's store right after
   its new value, so values do not stay live to the end (a Life generation's last segment writes
   1,023 cells).  The barrier makes storing safe when another group of the block reads a start
   value this group overwrites; without such a conflict there is none and the groups need not
   share a block.  Inside a segment no written cell is read across a far dimension, so no other
   word's warps read these cells. */
static void emit_group(Src *o, Chunk *k, const ChunkNet *cn, const uint32_t *outs, int nouts,
                       int own_rr, const unsigned char *in_cone, int barrier, int *store_at,
                       int *store_next)
{
    int n = tc_net_size(cn->net);
    for (int i = 0; i <= n; i++)
        store_at[i] = -1;
    for (int i = 0; i < nouts; i++) {
        int at = cn->cur[outs[i]] < 2 ? n : cn->cur[outs[i]];
        store_next[outs[i]] = store_at[at];
        store_at[at] = (int)outs[i];
    }
    char nm[32];
    for (int v = 2; v < n; v++)
        if (in_cone[v] && is_leaf(&cn->L, v) && cn->L.cell[v] >= 0)
            emit(o, "        const u32 c%d = m[%uu * W];\n", cn->L.cell[v],
                 slot_of(k, (uint32_t)cn->L.cell[v]));
    for (int v = 2; v < n; v++)
        if (in_cone[v] && is_leaf(&cn->L, v) && cn->L.far[v])
            emit(o, "        const u32 n%d = %s;\n", v, cn->L.expr[v]);
    /* the non-.aligned barrier may be reached from different code, once per warp */
    if (barrier)
        emit(o, "        asm volatile(\"barrier.sync 0;\" ::: \"memory\");\n");
    int luts = 0;
    for (int v = 2; v <= n; v++) {
        if (v < n && in_cone[v]) {
            if (is_leaf(&cn->L, v)) {
                if (!cn->L.far[v])
                    emit(o, "        const u32 n%d = %s;\n", v, cn->L.expr[v]);
            } else if (cn->mapped[v]) {
                emit_lut(o, cn, v, "        ");
                luts++;
            }
        }
        for (int c = store_at[v]; c >= 0; c = store_next[c]) {
            name_of(nm, sizeof nm, cn->cur[c]);
            emit(o, "        if (t < W) m[%uu * W] = %s;\n", slot_of(k, (uint32_t)c), nm);
            k->written[c] = 2;
        }
    }
    if (own_rr) {
        name_of(nm, sizeof nm, cn->rr);
        emit(o, "        if (t < W) rr[w] = %s;\n", nm);
    }
    emit(o, "        // %d LOP3\n", luts);
}

/* Warp groups of a chunk kernel: its written cells split into groups of at least
   tc_cube_min_cells, at most tc_cube_groups groups (small looping passes: 1). */
static unsigned chunk_groups(const Program *p, size_t from, size_t to, int loop)
{
    /* a small cube's passes loop in one warp with every cell in registers, unless the pass is
       long enough that splitting it over warps pays for a block barrier per pass (measured: a
       130,000-instruction Life pass 4.8x faster split, an 18,000-instruction sort slower) */
    if (!tc_cube_map || (loop && to - from < 50000))
        return 1;
    unsigned char *w = tc_xcalloc(p->ncells + 1, 1);
    unsigned nw = 0;
    for (size_t i = from; i < to; i++)
        if (p->code[i].op != OP_NAND && !tc_program_readonly(p, p->code[i].addr) &&
            !w[p->code[i].addr]) {
            w[p->code[i].addr] = 1;
            nw++;
        }
    free(w);
    unsigned g = nw / (unsigned)(tc_cube_min_cells > 0 ? tc_cube_min_cells : 1);
    if (g > (unsigned)tc_cube_groups)
        g = (unsigned)tc_cube_groups;
    return g ? g : 1;
}

/* The mapped body of a kernel that does not loop: `groups` warp groups per word, group y
   computing the cone of the y-th share of the written cells (RR with the last), so a chunk runs
   on `groups` times as many warps; nodes that several cones share are computed in each.

   A cell one group overwrites while another group reads its start value would be a conflict,
   so outputs that read a written cell's start value are kept in that cell's group (and the same
   for RR).  When that leaves the groups balanced the kernel is "group-major": each block runs
   tc_cube_gm_warps warps of ONE group over as many words, so the warps on an SM share their
   instructions, and no barrier is needed.  Otherwise the shares ignore the conflicts, and every
   block holds all groups of 32 words and waits at a barrier between loads and stores.
   *group_major gets the choice. */
static void split_body(Src *o, Chunk *k, size_t from, size_t to, unsigned groups,
                       int word_major, int *group_major)
{
    const Program *p = k->p;
    ChunkNet cn;
    chunk_net(k, from, to, &cn);
    uint32_t *outs = tc_xmalloc((p->ncells + 1) * sizeof *outs);
    int nouts = 0;
    for (uint32_t c = CELL_FIRST_FREE; c < p->ncells; c++)
        if (k->written[c])
            outs[nouts++] = c;
    int n = tc_net_size(cn.net);
    int *stack = tc_xmalloc((((size_t)n + 1) * 3 + p->ncells + 2) * sizeof *stack);
    int *store_at = tc_xmalloc(((size_t)n + 1) * sizeof *store_at);
    int *store_next = tc_xmalloc(((size_t)p->ncells + 1) * sizeof *store_next);
    /* Each output's own cone: its size (LUTs, at least 1) for the balance, and the start values
       it reads.  An output that reads the start value of a cell this kernel writes must be in
       that cell's group (the writer would otherwise overwrite it under the reader): such
       outputs are joined (union-find; RR is output nouts, its start value the first leaf). */
    int nall = nouts + 1, rr_leaf = 2;
    double *weight = tc_xmalloc(((size_t)nall + 1) * sizeof *weight), total = 0;
    int *stamp = tc_xcalloc((size_t)n + 1, sizeof *stamp);
    int *out_of = tc_xmalloc(((size_t)p->ncells + 1) * sizeof *out_of);  /* cell -> output */
    int *root = tc_xmalloc(((size_t)nall + 1) * sizeof *root);
    for (uint32_t c = 0; c < p->ncells; c++)
        out_of[c] = -1;
    for (int i = 0; i < nouts; i++)
        out_of[outs[i]] = i;
    for (int i = 0; i < nall; i++)
        root[i] = i;
#define FIND(x)                                                                                \
    ({                                                                                         \
        int r_ = (x);                                                                          \
        while (root[r_] != r_)                                                                 \
            r_ = root[r_] = root[root[r_]];                                                    \
        r_;                                                                                    \
    })
    for (int i = 0; i < nall; i++) {
        int sp = 0, size = 0;
        stack[sp++] = i < nouts ? cn.cur[outs[i]] : cn.rr;
        while (sp) {
            int v = stack[--sp];
            if (v < 2 || stamp[v] == i + 1)
                continue;
            stamp[v] = i + 1;
            if (is_leaf(&cn.L, v)) {
                int j = cn.L.cell[v] >= 0 ? out_of[cn.L.cell[v]] : v == rr_leaf ? nouts : -1;
                if (j >= 0 && j != i) {
                    int a = FIND(i), b = FIND(j);
                    if (a != b)
                        root[a < b ? b : a] = a < b ? a : b;
                }
                if (cn.L.src[v] >= 0)
                    stack[sp++] = cn.L.src[v];
                continue;
            }
            int lv[3], nl;
            uint8_t tt;
            tc_net_lut(cn.net, v, lv, &nl, &tt);
            size++;
            for (int j = 0; j < nl; j++)
                stack[sp++] = lv[j];
        }
        weight[i] = size > 0 ? size : 1;
        total += weight[i];
    }
    free(stamp);
    /* joined outputs go together; whole clusters to groups in output order, about equal total
       size each */
    double *cw = tc_xcalloc((size_t)nall + 1, sizeof *cw), biggest = 0;
    for (int i = 0; i < nall; i++)
        cw[FIND(i)] += weight[i];
    for (int i = 0; i < nall; i++)
        if (cw[i] > biggest)
            biggest = cw[i];
    int *cgroup = tc_xmalloc(((size_t)nall + 1) * sizeof *cgroup);
    for (int i = 0; i < nall; i++)
        cgroup[i] = -1;
    int *owner = tc_xmalloc(((size_t)nall + 1) * sizeof *owner);
    {
        double acc = 0;
        unsigned g = 0;
        for (int i = 0; i < nall; i++) {
            int r0 = FIND(i);
            if (cgroup[r0] < 0) {
                cgroup[r0] = (int)g;
                acc += cw[r0];
                if (g + 1 < groups && acc >= total * (g + 1) / groups)
                    g++;
            }
            owner[i] = cgroup[r0];
        }
    }
#undef FIND
    /* a cluster much larger than a share leaves the groups unbalanced: then word-major */
    int conflicts = biggest > 1.5 * total / groups;
    if (conflicts) {  /* contiguous shares, ignoring the clusters */
        double acc = 0;
        unsigned g = 0;
        for (int i = 0; i < nall; i++) {
            owner[i] = (int)g;
            acc += weight[i];
            if (g + 1 < groups && acc >= total * (g + 1) / groups &&
                nall - (i + 1) >= (int)(groups - g - 1))
                g++;
        }
    }
    free(weight);
    free(cw);
    free(cgroup);
    free(root);
    free(out_of);
    int rr_owner = owner[nouts];
    /* per group: its outputs and its cone */
    uint32_t *gouts = tc_xmalloc(((size_t)nouts + 1) * groups * sizeof *gouts);
    int *gn = tc_xcalloc(groups, sizeof *gn);
    unsigned char *cone = tc_xmalloc(((size_t)n + 1) * groups);
#define GROUP_CONE(g) (cone + (size_t)(g) * ((size_t)n + 1))
    for (unsigned g = 0; g < groups; g++) {
        for (int i = 0; i < nouts; i++)
            if (owner[i] == (int)g)
                gouts[(size_t)g * nouts + gn[g]++] = outs[i];
        cone_of(&cn, gouts + (size_t)g * nouts, gn[g], rr_owner == (int)g, GROUP_CONE(g), stack);
    }
    *group_major = !word_major && conflicts == 0 && groups > 1 && tc_cube_gm_warps > 0;
    emit(o, "    // %d LOP3 for %zu NAND/STO instructions, %u group(s), %s\n", cn.luts, to - from,
         groups, *group_major ? "group-major" : "word-major with a barrier");
    for (unsigned g = 0; g < groups; g++) {
        emit(o, "    if (%s == %uu) {\n", *group_major ? "group" : "threadIdx.y", g);
        emit_group(o, k, &cn, gouts + (size_t)g * nouts, gn[g], rr_owner == (int)g,
                   GROUP_CONE(g), !*group_major, store_at, store_next);
        emit(o, "    }\n");
    }
#undef GROUP_CONE
    free(gouts);
    free(gn);
    free(cone);
    free(owner);
    free(outs);
    free(stack);
    free(store_at);
    free(store_next);
    chunk_net_free(&cn);
}

/* The mapped body of a kernel that loops over passes: cells are the loop-carried variables
   c<cell>, assigned their new values at the end of each pass. */
static void loop_body(Src *o, Chunk *k, size_t from, size_t to)
{
    const Program *p = k->p;
    ChunkNet cn;
    chunk_net(k, from, to, &cn);
    emit(o, "    // %d LOP3 for %zu NAND/STO instructions\n", cn.luts, to - from);
    int n = tc_net_size(cn.net);
    for (int v = 2; v < n; v++) {
        if (is_leaf(&cn.L, v)) {
            if (cn.L.cell[v] >= 0)
                use_cell(o, k, (uint32_t)cn.L.cell[v]);  /* a cell the pass only reads */
            emit(o, "    const u32 n%d = %s;\n", v, cn.L.expr[v]);
        } else if (cn.mapped[v])
            emit_lut(o, &cn, v, "    ");
    }
    char nm[32];
    for (uint32_t c = CELL_FIRST_FREE; c < p->ncells; c++)
        if (k->written[c]) {
            name_of(nm, sizeof nm, cn.cur[c]);
            emit(o, "    c%u = %s;\n", (unsigned)c, nm);
        }
    name_of(nm, sizeof nm, cn.rr);
    emit(o, "    r = %s;\n", nm);
    chunk_net_free(&cn);
}

/* One kernel for instructions from .. to-1; with loop != 0 the whole pass, `passes` times. */
/* Blocks of a group-major kernel over W words: `want` warps (at most enough for W). */
static unsigned gm_warps(unsigned W, unsigned want)
{
    unsigned wpb = want > 0 ? want : 1;
    while (wpb > 1 && 32 * wpb > W)
        wpb /= 2;
    return wpb;
}

/* The runs of 32 * gm_warps(W, gmw) words a group-major block walks: `iters` (a power of two),
   as far as the word blocks of a group divide evenly. */
static unsigned gm_iters(unsigned W, unsigned gmw, unsigned iters)
{
    unsigned wpb = gm_warps(W, gmw), nwb = (W + 32 * wpb - 1) / (32 * wpb), it = 1;
    while (2 * it <= iters && nwb % (2 * it) == 0)
        it *= 2;
    return it;
}

static void emit_kernel(Src *o, const Program *p, unsigned W, unsigned idx, size_t from, size_t to,
                        int loop, int *group_major, unsigned iters, const uint32_t *slot,
                        unsigned gmw)
{
    Chunk k = {p, W, tc_xcalloc(p->ncells + 1, 1), tc_xcalloc(p->ncells + 1, 1), slot, 0};
    unsigned groups = chunk_groups(p, from, to, loop);
    int gm = 0;
    if (tc_cube_map && loop && groups > 1) {
        /* the whole cube is one block (W <= 32 words, every link inside a warp): the groups
           loop over the passes together, a block barrier after each pass's stores */
        Src body = {0};
        split_body(&body, &k, from, to, groups, 1, &gm);
        emit(o, "extern \"C\" __global__ void __launch_bounds__(%u) tc_cube_%u(u32 *__restrict__ "
                "mem, u32 *__restrict__ rr, const u32 passes)\n{\n", TC_CUBE_BLOCK * groups, idx);
        emit(o, "    const u32 t = threadIdx.x;\n");
        emit(o, "    const u32 w = t & (W - 1u);\n");
        emit(o, "    u32 *const m = mem + w;\n");
        emit(o, "#pragma unroll 1\n    for (u32 pass = 0; pass < passes; pass++) {\n");
        emit(o, "    u32 r = rr[w];\n");
        emit(o, "%.*s", (int)body.len, body.s ? body.s : "");
        emit(o, "    __syncthreads();\n    }\n}\n");
        free(body.s);
        if (k.bad)
            emit(o, "#error \"a far read of a computed cell that cannot be recomputed\"\n");
        free(k.loaded);
        free(k.written);
        if (group_major)
            *group_major = 0;
        return;
    }
    if (tc_cube_map && !loop) {
        Src body = {0};
        split_body(&body, &k, from, to, groups, 0, &gm);
        unsigned wpb = gm_warps(W, gmw), nwb = (W + 32 * wpb - 1) / (32 * wpb);
        unsigned it = gm ? gm_iters(W, gmw, iters) : 1;
        emit(o, "extern \"C\" __global__ void __launch_bounds__(%u) tc_cube_%u(u32 *__restrict__ "
                "mem, u32 *__restrict__ rr, const u32 passes)\n{\n",
             gm ? 32 * wpb : TC_CUBE_BLOCK * groups, idx);
        if (gm) {
            /* a block is one group over `it` runs of 32 * wpb words, one after the other: the
               group's straight-line code is fetched for the first run and found in the
               instruction cache for the others */
            emit(o, "    const u32 group = blockIdx.x / %uu;\n", nwb / it);
            emit(o, "#pragma unroll 1\n    for (u32 it = 0; it < %uu; it++) {\n", it);
            emit(o, "    const u32 t = ((blockIdx.x %% %uu) * %uu + it) * %uu + threadIdx.y * 32u + "
                    "threadIdx.x;\n", nwb / it, it, 32 * wpb);
        } else {
            emit(o, "    {\n    const u32 t = blockIdx.x * blockDim.x + threadIdx.x;\n");
        }
        emit(o, "    const u32 w = t & (W - 1u);\n");
        emit(o, "    u32 *const m = mem + w;\n");
        emit(o, "    u32 r = rr[w];\n");
        emit(o, "%.*s    }\n}\n", (int)body.len, body.s ? body.s : "");
        free(body.s);
        if (k.bad)
            emit(o, "#error \"a far read of a computed cell that cannot be recomputed\"\n");
        free(k.loaded);
        free(k.written);
        if (group_major)
            *group_major = gm;
        return;
    }
    if (group_major)
        *group_major = 0;
    emit(o, "extern \"C\" __global__ void __launch_bounds__(%u) tc_cube_%u(u32 *__restrict__ mem, "
            "u32 *__restrict__ rr, const u32 passes)\n{\n", TC_CUBE_BLOCK * groups, idx);
    emit(o, "    const u32 t = blockIdx.x * blockDim.x + threadIdx.x;\n");
    emit(o, "    const u32 w = t & (W - 1u);\n");
    emit(o, "    u32 *const m = mem + w;\n");
    emit(o, "    u32 r = rr[w];\n");
    if (loop) {
        /* every cell the pass touches is loop-carried: load before the loop */
        for (size_t i = from; i < to; i++) {
            unsigned mask;
            uint32_t a = p->code[i].op == OP_NAND ? tc_program_resolve(p, p->code[i].addr, &mask)
                                                  : p->code[i].addr;
            if (a >= CELL_FIRST_FREE && !tc_program_readonly(p, a))
                use_cell(o, &k, a);
        }
        emit(o, "#pragma unroll 1\n    for (u32 pass = 0; pass < passes; pass++) {\n");
    }
    if (tc_cube_map)
        loop_body(o, &k, from, to);
    else
        chunk_body(o, &k, from, to);
    if (loop)
        emit(o, "    }\n");
    emit(o, "    if (t < W) {\n");
    for (uint32_t c = CELL_FIRST_FREE; c < p->ncells; c++)
        if (k.written[c] == 1)
            emit(o, "        m[%uu * W] = c%u;\n", slot_of(&k, c), (unsigned)c);
    emit(o, "        rr[w] = r;\n    }\n}\n");
    if (k.bad)
        emit(o, "#error \"a far read of a computed cell that cannot be recomputed\"\n");
    free(k.loaded);
    free(k.written);
}

char *tc_codegen_cube(const Program *p, const size_t *first, unsigned nk, int block, size_t *len)
{
    (void)block;
    unsigned dims = tc_program_dims(p);
    unsigned W = (1u << dims) / 32;
    int loop = nk == 1 && dims <= FAR_DIM;
    Src o = {0};
    emit(&o, "// generated by the tesseract GB300 engine: cube of 2^%u machines, %u kernel(s)\n",
         dims, nk);
    emit(&o, "#define W %uu\n", W);
    emit(&o, "%s", CUBE_PRELUDE);
    for (unsigned k = 0; k < nk; k++)
        emit_kernel(&o, p, W, k, first[k], first[k + 1], loop, NULL, 1, NULL,
                    (unsigned)(tc_cube_gm_warps > 0 ? tc_cube_gm_warps : 1));
    if (len)
        *len = o.len;
    return o.s;
}

/* ---- compilation: kernels in parallel NVRTC programs ---------------------------------------- */

typedef struct {
    CudaCube     *c;
    unsigned      k0, k1;  /* kernels of this module */
    unsigned      iters;   /* group-major runs per block */
    unsigned      variant; /* 1: the second variant's memory (A and B exchanged) */
    unsigned      gmw;     /* warps per group-major block */
    cudaKernel_t *fn;      /* where the kernels go (variant v's kernel k at fn[v * nk + k]) */
    int          *gm;      /* where each kernel's group-major choice goes */
    int           ok;
    char          err[512];
} CompileJob;

static void *compile_job(void *arg)
{
    CompileJob *j = arg;
    CudaCube *c = j->c;
    size_t len;
    /* a module with kernels k0..k1-1: generate with shifted indices */
    unsigned nk = j->k1 - j->k0;
    size_t *first = tc_xmalloc((nk + 1) * sizeof *first);
    for (unsigned k = 0; k <= nk; k++)
        first[k] = c->first[j->k0 + k];
    int loop = c->nk == 1 && c->dims <= FAR_DIM;
    Src o = {0};
    emit(&o, "// generated by the tesseract GB300 engine: cube of 2^%u machines, kernels %u..%u, "
            "%u run(s) per group-major block, memory variant %u\n", c->dims, j->k0, j->k1 - 1,
         j->iters, j->variant);
    emit(&o, "#define W %uu\n", c->W);
    emit(&o, "%s", CUBE_PRELUDE);
    for (unsigned k = 0; k < nk; k++) {
        int gm;  /* the same in both variants: variant 0's job reports it */
        emit_kernel(&o, &c->p, c->W, j->k0 + k, first[k], first[k + 1], loop, &gm, j->iters,
                    j->variant ? c->slot1 : NULL, j->gmw);
        if (!j->variant)
            j->gm[j->k0 + k] = gm;
    }
    len = o.len;
    char **names = tc_xmalloc(nk * sizeof *names);
    for (unsigned k = 0; k < nk; k++) {
        names[k] = tc_xmalloc(32);
        snprintf(names[k], 32, "tc_cube_%u", j->k0 + k);
    }
    TcModule m;
    j->ok = 1;
    for (unsigned k0 = 0; k0 < nk && j->ok; k0 += TC_MAX_KERNELS) {
        unsigned n = nk - k0 < TC_MAX_KERNELS ? nk - k0 : TC_MAX_KERNELS;
        j->ok = tc_module(o.s, len, (const char *const *)names + k0, (int)n, NULL, &m, j->err,
                          sizeof j->err);
        for (unsigned k = 0; j->ok && k < n; k++)
            j->fn[j->variant * c->nk + j->k0 + k0 + k] = m.fn[k];
    }
    for (unsigned k = 0; k < nk; k++)
        free(names[k]);
    free(names);
    free(first);
    free(o.s);
    return NULL;
}

/* ---- the cube -------------------------------------------------------------------------------- */

unsigned cuda_cube_groups(const CudaCube *c) { return c->groups; }
unsigned cuda_cube_closing_copies(const CudaCube *c) { return c->nk - c->copy_k0; }

/* The plan cuda_cube_new makes for a program's closing copies: 1 with the first instruction of
   the copy segment in *from and the second variant's memory map in slot1 (ncells entries). */
static void plan_cube(CudaCube *c, const Program *p);

/* A plan made on the host alone (no device memory, no kernels) */
static void plan_free(CudaCube *c)
{
    free(c->first);
    free(c->slot1);
    free(c->warps);
    free(c->gmajor);
    tc_program_free(&c->p);
    free(c);
}

int tc_cube_copy_plan(const Program *p, size_t *from, uint32_t *slot1)
{
    CudaCube *c = tc_xcalloc(1, sizeof *c);
    tc_program_copy(p, &c->p);
    plan_cube(c, &c->p);
    int ok = c->variants == 2;
    *from = ok ? c->first[c->copy_k0] : p->len;
    if (ok)
        memcpy(slot1, c->slot1, p->ncells * sizeof *slot1);
    plan_free(c);
    return ok;
}

/* The source of every kernel of the cube's pass in memory variant `variant` (0, or 1 for the
   exchanged memory of a program with closing copies), as the cube compiles them, in one text;
   *nk gets the kernel count.  NULL when there is no such variant.  For tests: the text compiles
   for sm_103a. */
char *tc_cube_source(const Program *p, unsigned variant, unsigned *nk, size_t *len)
{
    CudaCube *c = tc_xcalloc(1, sizeof *c);
    tc_program_copy(p, &c->p);
    plan_cube(c, &c->p);
    char *out = NULL;
    *nk = c->nk;
    if (variant < c->variants) {
        Src o = {0};
        emit(&o, "#define W %uu\n", c->W);
        emit(&o, "%s", CUBE_PRELUDE);
        for (unsigned k = 0; k < c->nk; k++) {
            int gm;
            emit_kernel(&o, &c->p, c->W, k, c->first[k], c->first[k + 1], c->loop, &gm, 1,
                        variant ? c->slot1 : NULL, c->gmw);
        }
        out = o.s;
        *len = o.len;
    }
    plan_free(c);
    return out;
}
unsigned cuda_cube_segments(const CudaCube *c) { return c->isa_seg; }
unsigned cuda_cube_kernels(const CudaCube *c) { return c->nk; }

void cuda_cube_free(CudaCube *c)
{
    if (!c)
        return;
    if (c->graph)
        cudaGraphExecDestroy(c->graph);
    cudaFree(c->mem);
    cudaFree(c->rr);
    free(c->first);
    free(c->fn);
    free(c->slot1);
    free(c->warps);
    free(c->gmajor);
    tc_program_free(&c->p);
    free(c);
}

/* The cube's plan: segments (far reads of computed cells recomputed where they can be), the
   closing copies and their memory variant, kernels (long segments split), warp groups. */
static void plan_cube(CudaCube *c, const Program *p)
{
    c->gmw = (unsigned)(tc_cube_gm_warps > 0 ? tc_cube_gm_warps : 1);
    c->dims = tc_program_dims(p);
    c->machines = 1u << c->dims;
    c->groups = c->machines / 512;
    c->W = c->machines / 32;
    size_t *cuts = tc_xmalloc((p->len + 2) * sizeof *cuts);
    unsigned char *recomputes = tc_xmalloc(p->len + 2);
    c->nseg = plan_cuts(p, cuts, recomputes);
    {
        size_t *isa = tc_xmalloc((p->len + 2) * sizeof *isa);
        c->isa_seg = find_cuts(p, isa, CUBE_DIMS);
        free(isa);
    }
    /* closing copies: their segment starts where they do (cuts[nseg - 1] moves back over the
       loads of the first copy) */
    int copies = 0;
    if (tc_cube_copy_swap && c->nseg >= 2 && c->dims > FAR_DIM) {
        size_t from;
        c->slot1 = tc_xmalloc((p->ncells + 1) * sizeof *c->slot1);
        copies = copy_tail(p, cuts[c->nseg - 1], c->slot1, &from) && from > cuts[c->nseg - 2];
        if (copies) {
            cuts[c->nseg - 1] = from;
        } else {
            free(c->slot1);
            c->slot1 = NULL;
        }
    }
    /* split segments longer than tc_cube_chunk instructions into equal kernels of at most
       tc_cube_piece (not those that recompute: the recomputation starts from the segment's start
       values) */
    size_t chunk = tc_cube_chunk > 0 ? (size_t)tc_cube_chunk : 12000;
    size_t piece = tc_cube_piece > 0 && (size_t)tc_cube_piece < chunk ? (size_t)tc_cube_piece
                                                                         : chunk;
    c->first = tc_xmalloc((p->len / piece + c->nseg + 2) * sizeof *c->first);
    c->nk = 0;
    for (unsigned s = 0; s < c->nseg; s++) {
        size_t len = cuts[s + 1] - cuts[s], step = len;
        if (!recomputes[s] && len > chunk) {
            size_t kernels = (len + piece - 1) / piece;
            step = (len + kernels - 1) / kernels;
        }
        for (size_t i = cuts[s]; i < cuts[s + 1] || (i == cuts[s] && cuts[s] == cuts[s + 1]);
             i += step) {
            c->first[c->nk++] = i;
            if (cuts[s] == cuts[s + 1])
                break;
        }
    }
    free(recomputes);
    c->first[c->nk] = p->len;
    c->loop = c->nk == 1 && c->dims <= FAR_DIM;
    c->copy_k0 = c->nk;
    c->variants = 1;
    if (copies) {
        for (unsigned k = c->nk; k-- > 0;)
            if (c->first[k] == cuts[c->nseg - 1])
                c->copy_k0 = k;
        c->variants = 2;
    }
    free(cuts);
    c->warps = tc_xcalloc(c->nk, sizeof *c->warps);
    c->gmajor = tc_xcalloc(c->nk, sizeof *c->gmajor);
    for (unsigned k = 0; k < c->nk; k++)
        c->warps[k] = chunk_groups(p, c->first[k], c->first[k + 1], c->loop);
}

int cuda_cube_new(const Program *p, CudaCube **out, char *err, size_t errlen)
{
    *out = NULL;
    if (!cuda_engine_init(0, err, errlen))
        return 0;
    CudaCube *c = tc_xcalloc(1, sizeof *c);
    tc_program_copy(p, &c->p);
    plan_cube(c, &c->p);
    c->fn = tc_xcalloc((size_t)c->nk * c->variants, sizeof *c->fn);
    size_t words = (size_t)c->W * (p->ncells + 1);
    if (!tc_cu_check(cudaMalloc((void **)&c->mem, words * 4), "cudaMalloc", err, errlen) ||
        !tc_cu_check(cudaMalloc((void **)&c->rr, (size_t)c->W * 4), "cudaMalloc", err, errlen))
        goto fail;
    /* power-on state (src/lanes.c:176-192): all 0, ONE all 1, RR 0; id cells are computed */
    if (!tc_cu_check(cudaMemset(c->mem, 0, words * 4), "cudaMemset", err, errlen) ||
        !tc_cu_check(cudaMemset(c->mem + (size_t)CELL_ONE * c->W, 0xff, (size_t)c->W * 4),
                     "cudaMemset", err, errlen) ||
        !tc_cu_check(cudaMemset(c->rr, 0, (size_t)c->W * 4), "cudaMemset", err, errlen))
        goto fail;
    /* compile: one module per kernel and memory variant, all in parallel */
    unsigned nj = c->nk * c->variants;
    CompileJob *jobs = tc_xcalloc(nj, sizeof *jobs);
    pthread_t *tid = tc_xcalloc(nj, sizeof *tid);
    c->iters = 1;
    for (unsigned j = 0; j < nj; j++) {
        jobs[j].c = c;
        jobs[j].k0 = j % c->nk;
        jobs[j].k1 = j % c->nk + 1;
        jobs[j].variant = j / c->nk;
        jobs[j].iters = c->iters;
        jobs[j].gmw = c->gmw;
        jobs[j].fn = c->fn;
        jobs[j].gm = c->gmajor;
        pthread_create(&tid[j], NULL, compile_job, &jobs[j]);
    }
    int ok = 1;
    for (unsigned j = 0; j < nj; j++) {
        pthread_join(tid[j], NULL);
        if (!jobs[j].ok && ok) {
            ok = 0;
            tc_fail(err, errlen, "%s", jobs[j].err);
        }
    }
    free(jobs);
    free(tid);
    if (!ok)
        goto fail;
    *out = c;
    return 1;
fail:
    cuda_cube_free(c);
    return 0;
}

int cuda_cube_load(CudaCube *c, unsigned g, const uint64_t *lines, const uint64_t *rr, char *err,
                   size_t errlen)
{
    if (g >= c->groups)
        return tc_fail(err, errlen, "group %u of %u", g, c->groups);
    uint32_t *dst = c->mem + (size_t)g * 16;
    if (lines && !tc_cu_check(cudaMemcpy2D(dst, (size_t)c->W * 4, lines, 64, 64, c->p.ncells,
                                           cudaMemcpyHostToDevice), "load", err, errlen))
        return 0;
    /* ZERO and ONE keep their values whatever the host line holds */
    if (lines && (!tc_cu_check(cudaMemset(c->mem + (size_t)g * 16, 0, 64), "load", err, errlen) ||
                  !tc_cu_check(cudaMemset(c->mem + (size_t)CELL_ONE * c->W + (size_t)g * 16, 0xff,
                                          64), "load", err, errlen)))
        return 0;
    if (rr && !tc_cu_check(cudaMemcpy(c->rr + (size_t)g * 16, rr, 64, cudaMemcpyHostToDevice),
                           "load", err, errlen))
        return 0;
    return 1;
}

int cuda_cube_store(const CudaCube *c, unsigned g, uint64_t *lines, uint64_t *rr, char *err,
                    size_t errlen)
{
    if (g >= c->groups)
        return tc_fail(err, errlen, "group %u of %u", g, c->groups);
    if (lines && !tc_cu_check(cudaMemcpy2D(lines, 64, c->mem + (size_t)g * 16, (size_t)c->W * 4,
                                           64, c->p.ncells, cudaMemcpyDeviceToHost),
                              "store", err, errlen))
        return 0;
    if (rr && !tc_cu_check(cudaMemcpy(rr, c->rr + (size_t)g * 16, 64, cudaMemcpyDeviceToHost),
                           "store", err, errlen))
        return 0;
    return 1;
}

/* Whole-cube copies: cell-major words, W per cell (ncells x W u32), and W words of RR. */
int cuda_cube_read_words(const CudaCube *c, uint32_t *mem, uint32_t *rr, char *err, size_t errlen)
{
    if (mem && !tc_cu_check(cudaMemcpy(mem, c->mem, (size_t)c->W * c->p.ncells * 4,
                                       cudaMemcpyDeviceToHost), "read", err, errlen))
        return 0;
    if (rr && !tc_cu_check(cudaMemcpy(rr, c->rr, (size_t)c->W * 4, cudaMemcpyDeviceToHost), "read",
                           err, errlen))
        return 0;
    return 1;
}

int cuda_cube_write_words(CudaCube *c, const uint32_t *mem, const uint32_t *rr, char *err,
                          size_t errlen)
{
    if (mem && !tc_cu_check(cudaMemcpy(c->mem, mem, (size_t)c->W * c->p.ncells * 4,
                                       cudaMemcpyHostToDevice), "write", err, errlen))
        return 0;
    if (mem && (!tc_cu_check(cudaMemset(c->mem, 0, (size_t)c->W * 4), "write", err, errlen) ||
                !tc_cu_check(cudaMemset(c->mem + (size_t)CELL_ONE * c->W, 0xff, (size_t)c->W * 4),
                             "write", err, errlen)))
        return 0;
    if (rr && !tc_cu_check(cudaMemcpy(c->rr, rr, (size_t)c->W * 4, cudaMemcpyHostToDevice), "write",
                           err, errlen))
        return 0;
    return 1;
}

/* One pass (or `passes` for a looping cube) in memory variant `variant`; the closing copies only
   with `copies`. */
static int launch_pass(CudaCube *c, cudaStream_t s, unsigned passes, unsigned variant, int copies)
{
    unsigned threads = c->W < 32 ? 32 : c->W;
    unsigned block = threads < TC_CUBE_BLOCK ? threads : TC_CUBE_BLOCK;
    unsigned grid = (threads + block - 1) / block;
    unsigned nk = copies ? c->nk : c->copy_k0;
    for (unsigned k = 0; k < nk; k++) {
        uint32_t *mem = c->mem, *rr = c->rr;
        void *args[] = {&mem, &rr, &passes};
        dim3 b = dim3u(block), g = dim3u(grid);
        if (c->gmajor[k]) {  /* blocks of one group: gm_warps warps over gm_iters runs */
            unsigned wpb = gm_warps(c->W, c->gmw);
            b.y = wpb;
            g.x = ((c->W + 32 * wpb - 1) / (32 * wpb)) / gm_iters(c->W, c->gmw, c->iters) *
                  c->warps[k];
        } else {
            b.y = c->warps[k];
        }
        if (cudaLaunchKernel((const void *)c->fn[variant * c->nk + k], g, b, args, 0, s) !=
            cudaSuccess)
            return 0;
    }
    return 1;
}

int cuda_cube_run(CudaCube *c, uint64_t passes, char *err, size_t errlen)
{
    cudaStream_t s = tc_engine.stream;
    if (!tc_cu_check(cudaEventRecord(tc_engine.ev0, s), "event", err, errlen))
        return 0;
    if (c->loop) {
        while (passes) {
            unsigned n = passes > (1u << 30) ? 1u << 30 : (unsigned)passes;
            if (!launch_pass(c, s, n, 0, 1))
                return tc_cu_check(cudaGetLastError(), "cube launch", err, errlen);
            passes -= n;
        }
    } else if (passes) {
        /* many passes of several kernels: replay a captured graph of 16 passes.  With two memory
           variants pass i runs in variant i % 2 without the closing copies, except the last,
           which has them (and stays out of the graph) */
        const unsigned G = 16;
        int swap = c->variants == 2;
        uint64_t open = swap ? passes - 1 : passes, done = 0;
        if (open >= G && !c->graph) {
            cudaGraph_t g;
            cudaStream_t cs;
            if (!tc_cu_check(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "stream", err,
                             errlen))
                return 0;
            int ok = tc_cu_check(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal),
                                 "capture", err, errlen);
            for (unsigned i = 0; ok && i < G; i++)
                ok = launch_pass(c, cs, 1, swap ? i % 2 : 0, !swap);
            cudaError_t e = cudaStreamEndCapture(cs, &g);
            if (ok)
                ok = tc_cu_check(e, "capture", err, errlen);
            if (ok)
                ok = tc_cu_check(cudaGraphInstantiate(&c->graph, g, 0), "graph", err, errlen);
            if (ok)
                cudaGraphDestroy(g);
            cudaStreamDestroy(cs);
            if (!ok)
                return 0;
            c->graph_passes = G;
        }
        while (c->graph && open - done >= c->graph_passes) {
            if (!tc_cu_check(cudaGraphLaunch(c->graph, s), "graph launch", err, errlen))
                return 0;
            done += c->graph_passes;
        }
        for (; done < open; done++)
            if (!launch_pass(c, s, 1, swap ? (unsigned)(done % 2) : 0, !swap))
                return tc_cu_check(cudaGetLastError(), "cube launch", err, errlen);
        if (swap && !launch_pass(c, s, 1, (unsigned)(done % 2), 1))
            return tc_cu_check(cudaGetLastError(), "cube launch", err, errlen);
    }
    if (!tc_cu_check(cudaEventRecord(tc_engine.ev1, s), "event", err, errlen) ||
        !tc_cu_check(cudaEventSynchronize(tc_engine.ev1), "cube run", err, errlen))
        return 0;
    float ms = 0;
    cudaEventElapsedTime(&ms, tc_engine.ev0, tc_engine.ev1);
    tc_engine.last_kernel_ms = ms;
    return 1;
}

/* ---- the autotuner for cube kernels ------------------------------------------------------------

   A group-major kernel's block runs one group's straight-line code, once per warp; with the code
   fetched cold every time, instruction fetch, not the ALU, sets the pace (Life on 65,536
   machines: no_instruction the first stall).  Blocks that walk 2, 4 or 8 runs of words in a loop
   find the code cached after the first run, at the price of fewer blocks in flight.  Which is
   fastest depends on the program and the cube's size, so it is measured: every variant is
   compiled (in parallel), run for probe_passes passes from the cube's present state, which is
   saved before and restored after, and the fastest kept. */
int cuda_cube_tune(CudaCube *c, unsigned probe_passes, CudaCubeTune *t, char *err, size_t errlen)
{
    memset(t, 0, sizeof *t);
    int any_gm = 0;
    for (unsigned k = 0; k < c->nk; k++)
        any_gm |= c->gmajor[k];
    /* (warps per block, runs per block) as the cube's size allows them, the present one first */
    static const unsigned want_w[2] = {4, 8}, want_it[3] = {1, 2, 4};
    unsigned ws[CUBE_TUNE_MAX], its[CUBE_TUNE_MAX];
    int n = 0;
    ws[n] = c->gmw;
    its[n++] = c->iters;
    for (int a = 0; any_gm && !c->loop && a < 2; a++)
        for (int i = 0; i < 3 && n < CUBE_TUNE_MAX; i++) {
            unsigned w = gm_warps(c->W, want_w[a]), it = gm_iters(c->W, w, want_it[i]);
            int seen = 0;
            for (int j = 0; j < n; j++)
                seen |= gm_warps(c->W, ws[j]) == w && its[j] == it;
            if (!seen) {
                ws[n] = w;
                its[n++] = it;
            }
        }
    t->n = n;
    t->probe_passes = probe_passes;
    for (int i = 0; i < n; i++) {
        t->cand[i].warps = gm_warps(c->W, ws[i]);
        t->cand[i].iters = its[i];
        t->cand[i].ms = -1;
    }
    if (n == 1 || probe_passes == 0) {
        t->best = 0;
        return 1;
    }
    cudaKernel_t *fns[CUBE_TUNE_MAX];
    unsigned nkv = c->nk * c->variants;
    int *gms = tc_xcalloc(c->nk, sizeof *gms);
    CompileJob *jobs = tc_xcalloc((size_t)n * nkv, sizeof *jobs);
    pthread_t *tid = tc_xcalloc((size_t)n * nkv, sizeof *tid);
    unsigned nj = 0;
    for (int i = 0; i < n; i++) {
        fns[i] = i == 0 ? c->fn : tc_xcalloc(nkv, sizeof *fns[i]);
        for (unsigned kv = 0; i > 0 && kv < nkv; kv++) {
            jobs[nj] = (CompileJob){c, kv % c->nk, kv % c->nk + 1, its[i], kv / c->nk, ws[i],
                                    fns[i], gms, 0, ""};
            if (pthread_create(&tid[nj], NULL, compile_job, &jobs[nj]) == 0)
                nj++;
        }
    }
    int ok = 1;
    for (unsigned j = 0; j < nj; j++) {
        pthread_join(tid[j], NULL);
        if (!jobs[j].ok && ok)
            ok = tc_fail(err, errlen, "%s", jobs[j].err);
    }
    free(jobs);
    free(tid);
    free(gms);
    size_t words = (size_t)c->W * (c->p.ncells + 1);
    uint32_t *save_mem = NULL, *save_rr = NULL;
    cudaStream_t s = tc_engine.stream;
    ok = ok &&
         tc_cu_check(cudaMalloc((void **)&save_mem, words * 4), "cudaMalloc", err, errlen) &&
         tc_cu_check(cudaMalloc((void **)&save_rr, (size_t)c->W * 4), "cudaMalloc", err, errlen) &&
         tc_cu_check(cudaMemcpyAsync(save_mem, c->mem, words * 4, cudaMemcpyDeviceToDevice, s),
                     "save", err, errlen) &&
         tc_cu_check(cudaMemcpyAsync(save_rr, c->rr, (size_t)c->W * 4, cudaMemcpyDeviceToDevice,
                                     s), "save", err, errlen);
    cudaKernel_t *keep_fn = c->fn;
    unsigned keep_iters = c->iters, keep_gmw = c->gmw;
    int best = -1;
    for (int i = 0; ok && i < n; i++) {
        c->fn = fns[i];
        c->iters = its[i];
        c->gmw = ws[i];
        for (int rep = 0; ok && rep < 2; rep++) {  /* a warm-up run, then the timed one */
            ok = tc_cu_check(cudaMemcpyAsync(c->mem, save_mem, words * 4,
                                             cudaMemcpyDeviceToDevice, s), "restore", err,
                             errlen) &&
                 tc_cu_check(cudaMemcpyAsync(c->rr, save_rr, (size_t)c->W * 4,
                                             cudaMemcpyDeviceToDevice, s), "restore", err,
                             errlen) &&
                 tc_cu_check(cudaEventRecord(tc_engine.ev0, s), "event", err, errlen);
            for (unsigned q = 0; ok && q < probe_passes; q++)  /* as cuda_cube_run runs them */
                ok = launch_pass(c, s, 1, c->variants == 2 ? q % 2 : 0,
                                 c->variants == 1 || q + 1 == probe_passes) ||
                     tc_cu_check(cudaGetLastError(), "cube launch", err, errlen);
            ok = ok && tc_cu_check(cudaEventRecord(tc_engine.ev1, s), "event", err, errlen) &&
                 tc_cu_check(cudaEventSynchronize(tc_engine.ev1), "tune", err, errlen);
        }
        float ms = 0;
        if (ok)
            cudaEventElapsedTime(&ms, tc_engine.ev0, tc_engine.ev1);
        t->cand[i].ms = ms;
        if (ok && (best < 0 || ms < t->cand[best].ms))
            best = i;
    }
    if (ok)
        ok = tc_cu_check(cudaMemcpyAsync(c->mem, save_mem, words * 4, cudaMemcpyDeviceToDevice,
                                         s), "restore", err, errlen) &&
             tc_cu_check(cudaMemcpyAsync(c->rr, save_rr, (size_t)c->W * 4,
                                         cudaMemcpyDeviceToDevice, s), "restore", err, errlen) &&
             tc_cu_check(cudaStreamSynchronize(s), "restore", err, errlen);
    c->fn = ok ? fns[best] : keep_fn;
    c->iters = ok ? its[best] : keep_iters;
    c->gmw = ok ? ws[best] : keep_gmw;
    for (int i = 0; i < n; i++)
        if (fns[i] != c->fn)
            free(fns[i]);
    cudaFree(save_mem);
    cudaFree(save_rr);
    if (ok && c->graph) {  /* the captured passes hold the old kernels */
        cudaGraphExecDestroy(c->graph);
        c->graph = NULL;
    }
    t->best = ok ? best : 0;
    return ok;
}

/* ---- compiled code handles (jit_compile / jit_free) ----------------------------------------- */

int cuda_compile(const Program *p, CudaCode **out, char *err, size_t errlen)
{
    *out = NULL;
    CudaCube *c;
    if (!cuda_cube_new(p, &c, err, errlen))
        return 0;
    *out = tc_xcalloc(1, sizeof **out);
    (*out)->cube = c;
    return 1;
}

void cuda_free(CudaCode *code)
{
    if (!code)
        return;
    cuda_cube_free(code->cube);
    free(code);
}

/* ---- check_lanes on the GPU ------------------------------------------------------------------- */

static int differ(CheckResult *r, unsigned lane, long cell, unsigned want, unsigned got)
{
    r->ok = 0;
    r->lane = lane;
    r->cell = cell;
    r->want = want;
    r->got = got;
    return 0;
}

/* Compares RR and every cell, constants, ids and links included, of every machine, in the
   order of src/check.c:35-50. */
static int same_state(const CudaCube *c, const TcRef *ref, const uint32_t *mem, const uint32_t *rr,
                      CheckResult *r)
{
    const Program *p = &c->p;
    for (unsigned k = 0; k < c->machines; k++) {
        unsigned got = (rr[k >> 5] >> (k & 31)) & 1;
        if (got != ref->rr[k])
            return differ(r, k, -1, ref->rr[k], got);
        for (uint32_t a = 0; a < p->ncells; a++) {
            unsigned mask;
            uint32_t cell = tc_program_resolve(p, a, &mask);
            unsigned mk = k ^ mask, g;
            if (p->special && p->special[cell].kind == CK_ID)
                g = (mk >> p->special[cell].dim) & 1;
            else
                g = (mem[(size_t)cell * c->W + (mk >> 5)] >> (mk & 31)) & 1;
            unsigned want = tc_ref_get(ref, k, a);
            if (g != want)
                return differ(r, k, (long)a, want, g);
        }
        r->compared++;
    }
    return 1;
}

int cuda_check(const Program *p, uint64_t seed, unsigned ticks, CheckResult *r, char *err,
               size_t errlen)
{
    memset(r, 0, sizeof *r);
    r->ok = 1;
    CudaCube *c;
    if (!cuda_cube_new(p, &c, err, errlen))
        return 0;
    TcRef ref;
    size_t nwords = (size_t)c->W * p->ncells;
    uint32_t *mem = tc_xcalloc(nwords + 1, 4), *rr = tc_xcalloc(c->W + 1, 4);
    int ok = 0;
    if (!tc_ref_init(&ref, p, c->machines)) {
        tc_fail(err, errlen, "out of memory");
        goto done;
    }
    /* the starting state of src/check.c:60-72: splitmix64(seed), per group every cell from 2 up
       (kept only where writable), then RR */
    uint64_t s = seed;
    for (unsigned g = 0; g < c->groups; g++) {
        for (uint32_t a = CELL_FIRST_FREE; a < p->ncells; a++)
            for (int w = 0; w < 8; w++) {
                uint64_t v = tc_splitmix64(&s);
                if (tc_program_readonly(p, a))
                    continue;
                size_t at = (size_t)a * c->W + (size_t)g * 16 + 2 * (size_t)w;
                mem[at] = (uint32_t)v;
                mem[at + 1] = (uint32_t)(v >> 32);
            }
        for (int w = 0; w < 8; w++) {
            uint64_t v = tc_splitmix64(&s);
            rr[g * 16 + 2 * w] = (uint32_t)v;
            rr[g * 16 + 2 * w + 1] = (uint32_t)(v >> 32);
        }
    }
    for (uint32_t w = 0; w < c->W; w++)
        mem[(size_t)CELL_ONE * c->W + w] = 0xffffffffu;
    for (unsigned k = 0; k < c->machines; k++) {
        for (uint32_t a = CELL_FIRST_FREE; a < p->ncells; a++)
            if (!tc_program_readonly(p, a))
                ref.mem[(size_t)k * p->ncells + a] =
                    (uint8_t)((mem[(size_t)a * c->W + (k >> 5)] >> (k & 31)) & 1);
        ref.rr[k] = (uint8_t)((rr[k >> 5] >> (k & 31)) & 1);
    }
    if (!cuda_cube_write_words(c, mem, rr, err, errlen))
        goto done;
    same_state(c, &ref, mem, rr, r);
    for (unsigned t = 1; r->ok && t <= ticks; t++) {
        r->tick = t;
        r->pc = -1;
        if (!cuda_cube_run(c, 1, err, errlen) || !cuda_cube_read_words(c, mem, rr, err, errlen))
            goto done;
        tc_ref_tick(&ref);
        same_state(c, &ref, mem, rr, r);
    }
    ok = 1;
done:
    tc_ref_free(&ref);
    free(mem);
    free(rr);
    cuda_cube_free(c);
    return ok;
}
