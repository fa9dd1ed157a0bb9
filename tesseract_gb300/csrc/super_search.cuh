// The superoptimizer's search model, shared by the host (frontier generation, replay) and the
// device (the depth-first search of every frontier subtree).
//
// The model is the reference's (src/super.c:373-706): a program is a chain of NANDs over truth
// tables; hist[i] is RR after NAND i.  A NAND reads ZERO, ONE, a readable cell (inputs, and
// outputs once written), or an earlier RR value hist[j]; such a value is stored lazily, one STO
// charged on its first read.  An output is written (one STO) right after a NAND that leaves its
// target in RR.  Cost = NANDs + STOs.  Sound pruning: one candidate per value (the cheapest), no
// NAND that leaves RR unchanged, interchangeable inputs read in order, and a lower bound on the
// instructions still needed.  Iterative deepening over the budget proves minimality: a budget
// searched in full without a program rules out every shorter program.
#ifndef TC_SUPER_SEARCH_CUH
#define TC_SUPER_SEARCH_CUH

#include <stdint.h>

#define SP_CELLS 16
#define SP_LEN 64
#define SP_CANDS (SP_CELLS + SP_LEN + 4)

#ifdef __CUDACC__
#define SP_HD __host__ __device__ __forceinline__
#else
#define SP_HD static inline
#endif

enum { SK_ZERO, SK_ONE, SK_CELL, SK_TEMP, SK_LAZY };

typedef struct {
    int      nvars, rr_in, rr_out, ncells;
    uint64_t mask, rr_target;
    uint64_t init[SP_CELLS], target[SP_CELLS];
    uint32_t alias[SP_CELLS];
    uint8_t  in[SP_CELLS], out[SP_CELLS];
    int8_t   sym_prev[SP_CELLS];
} SpSpec;

typedef struct {
    uint64_t hist[SP_LEN + 1];
    uint8_t  stored[SP_LEN + 1], op_kind[SP_LEN + 1];
    int8_t   op_ref[SP_LEN + 1], out_at[SP_CELLS];
    uint32_t readable, written, used;
    int      n, cost, def0;
} SpState;

/* A candidate operand: its value, the cost on top of the NAND (a lazy store), and where it
   comes from (kind, ref). */
typedef struct {
    uint64_t v;
    uint8_t  kind, extra;
    int8_t   ref;
} SpCand;

SP_HD uint64_t sp_var_table(int i)
{
    uint64_t t = 0;
    for (int r = 0; r < 64; r++)
        if ((r >> i) & 1)
            t |= 1ull << r;
    return t;
}

SP_HD void sp_reset(const SpSpec *sp, SpState *x)
{
    x->n = 0;
    x->cost = 0;
    x->def0 = sp->rr_in;
    x->hist[0] = sp->rr_in ? sp_var_table(0) & sp->mask : 0;
    x->stored[0] = 0;
    x->readable = 0;
    x->written = 0;
    x->used = 0;
    for (int c = 0; c < sp->ncells; c++) {
        x->out_at[c] = -1;
        if (sp->in[c])
            x->readable |= 1u << c;
    }
}

SP_HD int sp_rr_def(const SpState *x) { return x->n > 0 || x->def0; }

SP_HD uint64_t sp_cell_value(const SpSpec *sp, const SpState *x, int c)
{
    return ((x->written >> c) & 1) ? sp->target[c] : sp->init[c];
}

/* The operands a NAND may read now, one per value, the cheapest, in the order ZERO, ONE, cells,
   earlier RR values. */
SP_HD int sp_build(const SpSpec *sp, const SpState *x, SpCand *out)
{
    int n = 0;
    out[n].v = 0; out[n].kind = SK_ZERO; out[n].extra = 0; out[n].ref = 0; n++;
    out[n].v = sp->mask; out[n].kind = SK_ONE; out[n].extra = 0; out[n].ref = 0; n++;
    for (int c = 0; c < sp->ncells; c++) {
        if (!((x->readable >> c) & 1))
            continue;
        int prev = sp->sym_prev[c];
        if (prev >= 0 && !((x->used >> prev) & 1))
            continue;
        out[n].v = sp_cell_value(sp, x, c); out[n].kind = SK_CELL; out[n].extra = 0;
        out[n].ref = (int8_t)c; n++;
    }
    for (int j = x->def0 ? 0 : 1; j <= x->n; j++) {
        out[n].v = x->hist[j];
        out[n].kind = x->stored[j] ? SK_TEMP : SK_LAZY;
        out[n].extra = (uint8_t)!x->stored[j];
        out[n].ref = (int8_t)j;
        n++;
    }
    int m = 0;
    for (int i = 0; i < n; i++) {
        int k = 0;
        while (k < m && out[k].v != out[i].v)
            k++;
        if (k == m)
            out[m++] = out[i];
        else if (out[i].extra < out[k].extra)
            out[k] = out[i];
    }
    return m;
}

/* The fewest instructions still needed: one STO per unwritten output, one NAND per distinct
   target value RR does not hold yet, and RR's own target. */
SP_HD int sp_lower_bound(const SpSpec *sp, const SpState *x)
{
    uint64_t need[SP_CELLS + 1];
    int nneed = 0, stores = 0;
    uint64_t rr = x->hist[x->n];
    int def = sp_rr_def(x);
    for (int c = 0; c < sp->ncells; c++) {
        if (!sp->out[c] || ((x->written >> c) & 1))
            continue;
        stores++;
        uint64_t t = sp->target[c];
        int k = 0;
        while (k < nneed && need[k] != t)
            k++;
        if (k == nneed && !(def && t == rr))
            need[nneed++] = t;
    }
    int nands = nneed;
    if (sp->rr_out) {
        int k = 0;
        while (k < nneed && need[k] != sp->rr_target)
            k++;
        if (!(def && rr == sp->rr_target)) {
            if (k == nneed)
                nands++;
        } else if (nneed) {
            nands++;
        }
    }
    return stores + nands;
}

SP_HD int sp_goal(const SpSpec *sp, const SpState *x)
{
    for (int c = 0; c < sp->ncells; c++)
        if (sp->out[c] && !((x->written >> c) & 1))
            return 0;
    return !sp->rr_out || (sp_rr_def(x) && x->hist[x->n] == sp->rr_target);
}

/* Outputs whose target RR holds now and that are not written yet. */
SP_HD int sp_hits(const SpSpec *sp, const SpState *x, int8_t *list)
{
    int k = 0;
    if (!sp_rr_def(x))
        return 0;
    for (int c = 0; c < sp->ncells; c++)
        if (sp->out[c] && !((x->written >> c) & 1) && sp->target[c] == x->hist[x->n])
            list[k++] = (int8_t)c;
    return k;
}

SP_HD void sp_write(const SpSpec *sp, SpState *x, const int8_t *list, int mask)
{
    for (int i = 0; (mask >> i) != 0; i++) {
        if (!((mask >> i) & 1))
            continue;
        int c = list[i];
        x->written |= 1u << c;
        x->out_at[c] = (int8_t)x->n;
        x->cost++;
        x->readable &= ~sp->alias[c];
        x->readable |= 1u << c;
    }
}

/* Applies NAND with candidate c; returns 0 if the move is pruned. */
SP_HD int sp_nand(const SpSpec *sp, SpState *x, const SpCand *c, int budget)
{
    int def = sp_rr_def(x);
    if (!def && c->kind != SK_ZERO)
        return 0;
    uint64_t rr = x->hist[x->n];
    uint64_t r = ~(rr & c->v) & sp->mask;
    if (def && r == rr)
        return 0;
    if (x->cost + 1 + c->extra > budget)
        return 0;
    if (c->kind == SK_LAZY)
        x->stored[c->ref] = 1;
    if (c->kind == SK_CELL)
        x->used |= 1u << c->ref;
    x->cost += 1 + c->extra;
    x->n++;
    x->hist[x->n] = r;
    x->stored[x->n] = 0;
    x->op_kind[x->n] = c->kind;
    x->op_ref[x->n] = c->ref;
    return 1;
}

/* What node() checks on arrival: 0 go on, 1 pruned, 2 goal. */
SP_HD int sp_arrive(const SpSpec *sp, const SpState *x, int budget)
{
    if (x->cost > budget)
        return 1;
    if (sp_goal(sp, x))
        return 2;
    if (x->cost + sp_lower_bound(sp, x) > budget || x->n == SP_LEN)
        return 1;
    return 0;
}

#endif
