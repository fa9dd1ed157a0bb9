/* PTX for the enumeration kernel of an equivalence or search job, written directly.  A quick-start
   build (a batch's or a served job's compiled kernel, which replaces interpreter time and must be
   ready while the interpreter still runs) then skips NVRTC's front end and NVVM: ptxas alone,
   through nvJitLink, turns the text into a cubin.  NVRTC spends ~50 ms on any program before its
   first line of code; a job's whole PTX build costs about a quarter of its NVRTC build.

   The kernel does what the CUDA C template of codegen.c does for these modes (src/enum.c:166-200),
   with the identity layout: word w holds assignments 32 w .. 32 w + 31, input k of n is bit
   n-1-k of the assignment, a warp takes a contiguous run of the selected words (chunks of 1,024
   words, chunk c belonging to share c % parts, src/enum.c:232-234), counts hits with popcount
   and records its first 16 hits in assignment order, which are its 16 smallest.

   Loops: a chunk's 1,024 words are 32 steps of 32 (one word per lane).  Within a chunk only the
   five inputs on word bits 5..9 change from step to step; the inputs on the lane's word bits
   0..4 and on the chunk's bits stay, and so does every LUT that depends on no step input.
   Those inputs and LUTs are computed once per chunk, before its steps, when the values the steps
   read from them fit in registers.  Every branch before the warp's final store is uniform across
   the warp and says so (bra.uni), so ptxas needs no reconvergence around the votes and shuffles;
   the per-lane valid mask is computed with selects. */
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include "codegen.h"
#include "lutmap.h"

typedef struct {
    char  *s;
    size_t len, cap;
} Ptx;

static void put(Ptx *o, const char *fmt, ...)
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
        o->cap = o->cap ? 2 * o->cap + (size_t)k : 16384 + (size_t)k;
        o->s = tc_xrealloc(o->s, o->cap);
    }
}

#define PTX_MAX_FIELDS 64  /* values held across a chunk's steps: registers */

int tc_ptx_enum_ok(const TcGenEnum *g)
{
    return (g->mode == EN_EQUIV || g->mode == EN_SEARCH) && g->ticks == 1 && !g->no_map &&
           g->a->ninputs >= 1 && g->a->ninputs <= 64;
}

/* Input k (leaf register r) from the word's low or high half: lane patterns for bits 0..4 of the
   assignment, else the word's bit spread over the 32 lanes (a shift up to the sign bit and an
   arithmetic shift down). */
static void put_input(Ptx *o, int r, int q, const char *lo, const char *hi)
{
    static const char *pat[5] = {"0xaaaaaaaa", "0xcccccccc", "0xf0f0f0f0", "0xff00ff00",
                                 "0xffff0000"};
    if (q < 5) {
        put(o, "\tmov.b32 %%v%d, %s;\n", r, pat[q]);
        return;
    }
    int b = q - 5;
    const char *w = b < 32 ? lo : hi;
    b &= 31;
    put(o, "\tshl.b32 %%t, %s, %d;\n\tshr.s32 %%v%d, %%t, 31;\n", w, 31 - b, r);
}

/* One kernel named `name` into o; *work gets its work per word. */
static void put_kernel(Ptx *o, const TcGenEnum *g, const char *name, TcGenWork *work)
{
    const Program *a = g->a;
    const int n = (int)a->ninputs;
    TcNet *net = tc_net_new();
    int *leaf = tc_xmalloc(((size_t)n + 1) * sizeof *leaf);
    for (int k = 0; k < n; k++)
        leaf[k] = tc_net_leaf(net, k);
    int *cur_a = tc_xmalloc((a->ncells + 1) * sizeof *cur_a);
    int *cur_b = g->b ? tc_xmalloc((g->b->ncells + 1) * sizeof *cur_b) : NULL;
    tc_net_pass(net, a, a->inputs, (size_t)n, leaf, cur_a);
    if (g->mode == EN_EQUIV)
        tc_net_pass(net, g->b, g->b_inputs, (size_t)n, leaf, cur_b);
    /* the compared values: equiv pairs (a, b) of outputs; search, the spec's output bits */
    int nwant = g->mode == EN_EQUIV ? 2 * (int)a->noutputs : g->spec->width;
    int *want = tc_xmalloc(((size_t)nwant + 1) * sizeof *want);
    if (g->mode == EN_EQUIV)
        for (size_t k = 0; k < a->noutputs; k++) {
            want[2 * k] = cur_a[a->outputs[k]];
            want[2 * k + 1] = cur_b[g->b->outputs[g->out_map[k]]];
        }
    else
        for (int bit = 0; bit < nwant; bit++)
            want[bit] = cur_a[g->spec->out[bit]];
    const int size = tc_net_size(net);
    int *order = tc_xmalloc(((size_t)size + 1) * sizeof *order), norder = 0;
    tc_net_map(net, want, nwant, order, &norder);

    /* registers: %v<reg[node]> for the constants, the leaves and the chosen LUTs */
    int *reg = tc_xmalloc(((size_t)size + 1) * sizeof *reg), nreg = 0;
    for (int i = 0; i <= size; i++)
        reg[i] = -1;
    reg[0] = nreg++;
    reg[1] = nreg++;
    for (int k = 0; k < n; k++)
        if (reg[leaf[k]] < 0)
            reg[leaf[k]] = nreg++;
    int (*lv)[3] = tc_xmalloc(((size_t)norder + 1) * sizeof *lv);
    uint8_t *tt = tc_xmalloc((size_t)norder + 1);
    uint64_t *sup = tc_xcalloc((size_t)size + 1, sizeof *sup);  /* inputs a node depends on */
    for (int k = 0; k < n; k++)
        sup[leaf[k]] = 1ull << k;
    for (int i = 0; i < norder; i++) {
        int nl;
        tc_net_lut(net, order[i], lv[i], &nl, &tt[i]);
        for (int q = nl; q < 3; q++)
            lv[i][q] = 0;
        sup[order[i]] = sup[lv[i][0]] | sup[lv[i][1]] | sup[lv[i][2]];
        reg[order[i]] = nreg++;
    }

    /* the step inputs: bits 10..14 of the assignment (word bits 5..9) */
    uint64_t step = 0;
    for (int k = 0; k < n; k++) {
        int q = n - 1 - k;
        if (q >= 10 && q < 15)
            step |= 1ull << k;
    }
    int hoisted = 0;
    for (int i = 0; i < norder; i++)
        hoisted += (sup[order[i]] & step) == 0;
    /* values the steps read that a chunk computes once: held in registers across the steps */
    char *held = tc_xcalloc((size_t)size + 1, 1);
    int nheld = 0;
#define HOLD(nd)                                                                         \
    do {                                                                                 \
        int nd_ = (nd);                                                                  \
        if (nd_ > 1 && (sup[nd_] & step) == 0 && !held[nd_]) {                           \
            held[nd_] = 1;                                                               \
            nheld++;                                                                     \
        }                                                                                \
    } while (0)
    for (int i = 0; i < norder; i++)
        if (sup[order[i]] & step)
            for (int q = 0; q < 3; q++)
                HOLD(lv[i][q]);
    for (int w = 0; w < nwant; w++)
        HOLD(want[w]);
#undef HOLD
    /* moving a chunk's invariant work out of its steps costs only the registers that hold it */
    const int split = nheld <= PTX_MAX_FIELDS;
    /* inputs that no LUT and no compare reads are not computed */
    char *used = tc_xcalloc((size_t)size + 1, 1);
    for (int i = 0; i < norder; i++)
        for (int q = 0; q < 3; q++)
            used[lv[i][q]] = 1;
    for (int w = 0; w < nwant; w++)
        used[want[w]] = 1;

    put(o, "\n.visible .entry %s(\n\t.param .align 8 .b8 tc_args[64]\n)\n.maxntid %d, 1, 1\n{\n",
        name, g->block);
    put(o, "\t.reg .pred %%p_ch, %%p_run, %%p_in, %%p_sp, %%p_full, %%p_any, %%p_rec, %%p_l0;\n"
           "\t.reg .b32 %%lane, %%tidx, %%cta, %%nthr, %%rec, %%nsel, %%parts, %%part, %%clo, "
           "%%chi, %%wlo, %%valid, %%vpart, %%dl, %%one, %%m, %%pc, %%any, %%src, %%mm, "
           "%%xlo, %%xhi, %%ylo, %%yhi, %%tz, %%t, %%st, %%stend, %%chits, %%x32, %%space32;\n"
           "\t.reg .b64 %%words, %%space, %%per_warp, %%hits_p, %%list_p, %%count_p, %%warp, "
           "%%s0, %%s1, %%s, %%send, %%j, %%chunk, %%cbase, %%word, %%x0, %%t64, %%u64, "
           "%%hits, %%xb, %%lane64, %%addr, %%q, %%rr, %%nsel64, %%parts64, %%part64;\n"
           "\t.reg .b32 %%v<%d>;\n", nreg);
    /* the argument block: TcEnumArgs (codegen.h) */
    put(o, "\tld.param.u64 %%words, [tc_args+0];\n"
           "\tld.param.u64 %%space, [tc_args+8];\n"
           "\tld.param.u64 %%per_warp, [tc_args+16];\n"
           "\tld.param.u32 %%parts, [tc_args+24];\n"
           "\tld.param.u32 %%part, [tc_args+28];\n"
           "\tld.param.u32 %%nsel, [tc_args+32];\n"
           "\tld.param.u64 %%hits_p, [tc_args+40];\n"
           "\tld.param.u64 %%list_p, [tc_args+48];\n"
           "\tld.param.u64 %%count_p, [tc_args+56];\n"
           "\tcvta.to.global.u64 %%hits_p, %%hits_p;\n"
           "\tcvta.to.global.u64 %%list_p, %%list_p;\n"
           "\tcvta.to.global.u64 %%count_p, %%count_p;\n");
    /* warp w: words [w per_warp, min((w + 1) per_warp, words)) */
    put(o, "\tmov.u32 %%tidx, %%tid.x;\n\tmov.u32 %%cta, %%ctaid.x;\n\tmov.u32 %%nthr, %%ntid.x;\n"
           "\tand.b32 %%lane, %%tidx, 31;\n\tcvt.u64.u32 %%lane64, %%lane;\n"
           "\tmul.wide.u32 %%warp, %%cta, %%nthr;\n\tcvt.u64.u32 %%t64, %%tidx;\n"
           "\tadd.u64 %%warp, %%warp, %%t64;\n\tshr.u64 %%warp, %%warp, 5;\n"
           "\tmul.lo.u64 %%s0, %%warp, %%per_warp;\n\tadd.u64 %%s1, %%s0, %%per_warp;\n"
           "\tmin.u64 %%s1, %%s1, %%words;\n"
           "\tmov.u32 %%rec, 0;\n\tmov.u64 %%hits, 0;\n\tmov.u64 %%s, %%s0;\n\tmov.b32 %%one, 1;\n"
           "\tmov.b32 %%v%d, 0;\n\tmov.b32 %%v%d, -1;\n"
           "\tcvt.u64.u32 %%nsel64, %%nsel;\n\tcvt.u64.u32 %%parts64, %%parts;\n"
           "\tcvt.u64.u32 %%part64, %%part;\n"
           "\tsetp.eq.u32 %%p_ch, %%nsel, %%parts;\n\tmov.u32 %%space32, %u;\n"
           "\tsetp.ge.u64 %%p_run, %%s, %%s1;\n\t@%%p_run bra.uni $DONE;\n", reg[0], reg[1],
        n < 15 ? 1u << n : 0u);
    /* a chunk: the selected chunk's number, its base word (with the lane), the end of its steps */
    put(o, "$CHUNK:\n\tshr.u64 %%j, %%s, 10;\n\tmov.u64 %%chunk, %%j;\n\t@%%p_ch bra.uni $BASE;\n"
           "\tdiv.u64 %%q, %%j, %%nsel64;\n\trem.u64 %%rr, %%j, %%nsel64;\n"
           "\tmad.lo.u64 %%chunk, %%q, %%parts64, %%part64;\n\tadd.u64 %%chunk, %%chunk, %%rr;\n"
           "$BASE:\n\tshl.b64 %%cbase, %%chunk, 10;\n\tor.b64 %%cbase, %%cbase, %%lane64;\n"
           "\tor.b64 %%send, %%s, 1023;\n\tadd.u64 %%send, %%send, 1;\n"
           "\tmin.u64 %%send, %%send, %%s1;\n"
           "\tcvt.u32.u64 %%clo, %%cbase;\n\tshr.u64 %%t64, %%cbase, 32;\n"
           "\tcvt.u32.u64 %%chi, %%t64;\n"
           /* the steps as 32-bit word offsets within the chunk: st .. stend by 32 */
           "\tcvt.u32.u64 %%st, %%s;\n\tand.b32 %%st, %%st, 1023;\n"
           "\tsub.u64 %%t64, %%send, %%s;\n\tcvt.u32.u64 %%stend, %%t64;\n"
           "\tadd.u32 %%stend, %%stend, %%st;\n\tmov.u32 %%chits, 0;\n");
    if (split) {
        for (int k = 0; k < n; k++)
            if (!(step >> k & 1) && used[leaf[k]])
                put_input(o, reg[leaf[k]], n - 1 - k, "%clo", "%chi");
        for (int i = 0; i < norder; i++)
            if (!(sup[order[i]] & step))
                put(o, "\tlop3.b32 %%v%d, %%v%d, %%v%d, %%v%d, 0x%02x;\n", reg[order[i]],
                    reg[lv[i][0]], reg[lv[i][1]], reg[lv[i][2]], (unsigned)tt[i]);
    }
    /* a step: the word's low half (its high half is the chunk's), the step's inputs */
    put(o, "$STEP:\n\tor.b32 %%wlo, %%clo, %%st;\n");
    for (int k = 0; k < n; k++)
        if ((!split || (step >> k & 1)) && used[leaf[k]])
            put_input(o, reg[leaf[k]], n - 1 - k, "%wlo", "%chi");
    /* the lanes that count: a warp's words are whole multiples of 32 (per_warp and the selected
       words are), and with 15 inputs or more every selected chunk lies inside the space; only a
       space smaller than one chunk has words, and lanes, past its end */
    if (n < 15)
        put(o, "\tshl.b32 %%x32, %%wlo, 5;\n\tsub.u32 %%dl, %%space32, %%x32;\n"
               "\tsetp.lt.u32 %%p_in, %%x32, %%space32;\n\tsetp.ge.u32 %%p_full, %%dl, 32;\n"
               "\tand.b32 %%dl, %%dl, 31;\n\tshl.b32 %%vpart, %%one, %%dl;\n"
               "\tsub.u32 %%vpart, %%vpart, 1;\n"
               "\tselp.b32 %%valid, -1, %%vpart, %%p_full;\n"
               "\tselp.b32 %%valid, %%valid, 0, %%p_in;\n");
    for (int i = 0; i < norder; i++)
        if (!split || (sup[order[i]] & step))
            put(o, "\tlop3.b32 %%v%d, %%v%d, %%v%d, %%v%d, 0x%02x;\n", reg[order[i]],
                reg[lv[i][0]], reg[lv[i][1]], reg[lv[i][2]], (unsigned)tt[i]);
    /* the hit mask: equiv m |= a ^ b (0xf6 over m, a, b); search m &= bit ? v : ~v */
    if (g->mode == EN_EQUIV) {
        put(o, "\tmov.b32 %%m, 0;\n");
        for (int w = 0; w < nwant; w += 2)
            put(o, "\tlop3.b32 %%m, %%m, %%v%d, %%v%d, 0xf6;\n", reg[want[w]], reg[want[w + 1]]);
    } else {
        put(o, "\tmov.b32 %%m, -1;\n");
        for (int bit = 0; bit < nwant; bit++)
            put(o, "\tlop3.b32 %%m, %%m, %%v%d, %%v%d, 0x%s;\n", reg[want[bit]], reg[want[bit]],
                (g->target >> bit) & 1 ? "c0" : "30");
    }
    if (n < 15)
        put(o, "\tand.b32 %%m, %%m, %%valid;\n");
    put(o, "\tpopc.b32 %%pc, %%m;\n\tadd.u32 %%chits, %%chits, %%pc;\n"
           "\tsetp.ne.u32 %%p_any, %%m, 0;\n\tvote.sync.ballot.b32 %%any, %%p_any, -1;\n"
           "\tsetp.eq.u32 %%p_rec, %%any, 0;\n\t@%%p_rec bra.uni $NEXT;\n"
           "\tsetp.ge.u32 %%p_rec, %%rec, 16;\n\t@%%p_rec bra.uni $NEXT;\n"
           "\tmov.b64 %%word, {%%wlo, %%chi};\n\tshl.b64 %%x0, %%word, 5;\n");
    /* the warp's first 16 hits, lane by lane in order, each lane's bits in order: lane 0 stores */
    put(o, "$LANE:\n\tsetp.eq.u32 %%p_rec, %%any, 0;\n\t@%%p_rec bra.uni $NEXT;\n"
           "\tsetp.ge.u32 %%p_rec, %%rec, 16;\n\t@%%p_rec bra.uni $NEXT;\n"
           "\tbrev.b32 %%t, %%any;\n\tbfind.shiftamt.u32 %%src, %%t;\n"
           "\tshfl.sync.idx.b32 %%mm, %%m, %%src, 31, -1;\n"
           "\tmov.b64 {%%xlo, %%xhi}, %%x0;\n"
           "\tshfl.sync.idx.b32 %%xlo, %%xlo, %%src, 31, -1;\n"
           "\tshfl.sync.idx.b32 %%xhi, %%xhi, %%src, 31, -1;\n"
           "\tmov.b64 %%xb, {%%xlo, %%xhi};\n"
           "\tsetp.eq.u32 %%p_l0, %%lane, 0;\n"
           "$BIT:\n\tsetp.eq.u32 %%p_rec, %%mm, 0;\n\t@%%p_rec bra.uni $LANE_END;\n"
           "\tsetp.ge.u32 %%p_rec, %%rec, 16;\n\t@%%p_rec bra.uni $LANE_END;\n"
           "\tbrev.b32 %%t, %%mm;\n\tbfind.shiftamt.u32 %%tz, %%t;\n"
           "\tcvt.u64.u32 %%t64, %%tz;\n\tadd.u64 %%u64, %%xb, %%t64;\n"
           "\tshl.b64 %%addr, %%warp, 4;\n\tcvt.u64.u32 %%t64, %%rec;\n"
           "\tadd.u64 %%addr, %%addr, %%t64;\n\tshl.b64 %%addr, %%addr, 3;\n"
           "\tadd.u64 %%addr, %%list_p, %%addr;\n"
           "\t@%%p_l0 st.global.u64 [%%addr], %%u64;\n"
           "\tadd.u32 %%rec, %%rec, 1;\n\tsub.u32 %%t, %%mm, 1;\n\tand.b32 %%mm, %%mm, %%t;\n"
           "\tbra.uni $BIT;\n"
           "$LANE_END:\n\tsub.u32 %%t, %%any, 1;\n\tand.b32 %%any, %%any, %%t;\n"
           "\tbra.uni $LANE;\n");
    put(o, "$NEXT:\n\tadd.u32 %%st, %%st, 32;\n\tsetp.lt.u32 %%p_run, %%st, %%stend;\n"
           "\t@%%p_run bra.uni $STEP;\n"
           "\tcvt.u64.u32 %%t64, %%chits;\n\tadd.u64 %%hits, %%hits, %%t64;\n"
           "\tmov.u64 %%s, %%send;\n\tsetp.lt.u64 %%p_run, %%s, %%s1;\n\t@%%p_run bra.uni $CHUNK;\n");
    /* the warp's count and hit total */
    put(o, "$DONE:\n");
    for (int d = 16; d > 0; d >>= 1)
        put(o, "\tmov.b64 {%%xlo, %%xhi}, %%hits;\n"
               "\tshfl.sync.bfly.b32 %%ylo, %%xlo, %d, 31, -1;\n"
               "\tshfl.sync.bfly.b32 %%yhi, %%xhi, %d, 31, -1;\n"
               "\tmov.b64 %%t64, {%%ylo, %%yhi};\n\tadd.u64 %%hits, %%hits, %%t64;\n", d, d);
    put(o, "\tsetp.ne.u32 %%p_l0, %%lane, 0;\n\t@%%p_l0 bra $END;\n"
           "\tshl.b64 %%addr, %%warp, 2;\n\tadd.u64 %%addr, %%count_p, %%addr;\n"
           "\tst.global.u32 [%%addr], %%rec;\n"
           "\tsetp.eq.u64 %%p_rec, %%hits, 0;\n\t@%%p_rec bra $END;\n"
           "\tatom.global.add.u64 %%u64, [%%hits_p], %%hits;\n"
           "$END:\n\tret;\n}\n");

    if (work) {
        work->luts_per_step = split ? norder - hoisted : norder;
        work->luts_per_stretch = split ? hoisted : 0;
        work->stretch_steps = split ? 32 : 1;
        work->compare_ops = g->mode == EN_EQUIV ? (int)a->noutputs : nwant;
    }
    free(used);
    free(held);
    free(sup);
    free(tt);
    free(lv);
    free(reg);
    free(order);
    free(want);
    free(cur_a);
    free(cur_b);
    free(leaf);
    tc_net_free(net);
}

char *tc_ptx_enum(TcGenEnum *const *g, int n, const char *target, TcGenWork *work, size_t *len)
{
    Ptx o = {0};
    put(&o, "// generated by the tesseract GB300 engine: %d enumeration kernel(s)\n"
            ".version 9.0\n.target %s\n.address_size 64\n", n, target);
    for (int k = 0; k < n; k++) {
        char name[24];
        if (n == 1)
            snprintf(name, sizeof name, "tc_enum");
        else
            snprintf(name, sizeof name, "tc_enum_%d", k);
        put_kernel(&o, g[k], name, work ? &work[k] : NULL);
    }
    if (len)
        *len = o.len;
    return o.s;
}
