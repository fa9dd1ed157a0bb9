/* Technology mapping of a NAND network onto 3-input lookup tables: the LOP3 instruction.

   One pass of a NAND/STO program is a network of 2-input NANDs once STOs are read as renames.
   GB300's integer ALU evaluates any function of three 32-bit words per instruction (lop3.b32
   with an 8-bit truth table), so the fewest instructions for the pass are the fewest 3-input
   LUTs that cover the network.  This file builds the network with constant folding and
   structural hashing, enumerates the 3-feasible cuts of every node bottom up (keeping the best
   few by area flow, the usual priority-cuts method of FPGA mapping), selects a cover from the
   required outputs down, improves it by exact-area moves (one node at a time, then groups of
   nodes whose cuts share their leaves), and lists the chosen LUTs in topological order with
   their truth tables.  A full adder's sum and carry, for example, become one LUT each over
   (x, y, c), where the 19-instruction NAND/STO form needs eight or more 2-input operations; in
   an array multiplier that takes moving both at once, since each alone keeps the shared
   x ^ y node alive. */
#include <stdlib.h>
#include <string.h>

#include "lutmap.h"

#define PRIO 12  /* cuts kept per node */

typedef struct {
    int     leaf[3];
    int     n;
    uint8_t tt;     /* over leaf patterns 0xf0, 0xcc, 0xaa */
    float   flow;   /* area flow */
} Cut;

struct TcNet {
    TcNode  *node;
    int      n, cap;
    int     *slot;   /* hash table of gates: node + 1 */
    size_t   nslot;
    Cut     *cuts;   /* PRIO per node */
    int     *ncut;
    int     *refs;   /* fanout in the network */
    float   *flow;   /* best area flow */
    int     *best;   /* chosen cut index */
    char    *need;   /* in the cover */
};

TcNet *tc_net_new(void)
{
    TcNet *t = tc_xcalloc(1, sizeof *t);
    t->nslot = 1 << 12;
    t->slot = tc_xcalloc(t->nslot, sizeof *t->slot);
    tc_net_const(t, 0);  /* node 0 = 0, node 1 = ~0 */
    tc_net_const(t, 1);
    return t;
}

void tc_net_free(TcNet *t)
{
    if (!t)
        return;
    free(t->node);
    free(t->slot);
    free(t->cuts);
    free(t->ncut);
    free(t->refs);
    free(t->flow);
    free(t->best);
    free(t->need);
    free(t);
}

static int add(TcNet *t, int kind, int a, int b, int id)
{
    if (t->n == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 1024;
        t->node = tc_xrealloc(t->node, (size_t)t->cap * sizeof *t->node);
    }
    TcNode *x = &t->node[t->n];
    x->kind = kind;
    x->a = a;
    x->b = b;
    x->id = id;
    return t->n++;
}

int tc_net_const(TcNet *t, int v)
{
    if (t->n >= 2)
        return v ? 1 : 0;
    return add(t, TN_CONST, v, 0, 0);
}

int tc_net_leaf(TcNet *t, int id)
{
    return add(t, TN_LEAF, 0, 0, id);
}

static uint64_t hkey(int a, int b)
{
    return ((uint64_t)(uint32_t)a * 0x9E3779B97F4A7C15ull) ^ ((uint64_t)(uint32_t)b * 0xC2B2AE3D27D4EB4Full);
}

static void rehash(TcNet *t)
{
    free(t->slot);
    t->nslot *= 2;
    t->slot = tc_xcalloc(t->nslot, sizeof *t->slot);
    for (int i = 0; i < t->n; i++)
        if (t->node[i].kind == TN_NAND) {
            size_t h = hkey(t->node[i].a, t->node[i].b) & (t->nslot - 1);
            while (t->slot[h])
                h = (h + 1) & (t->nslot - 1);
            t->slot[h] = i + 1;
        }
}

/* ~(a & b), folded: with a constant, or an input twice, or a double negation. */
int tc_net_nand(TcNet *t, int a, int b)
{
    if (a > b) {
        int s = a;
        a = b;
        b = s;
    }
    if (a == 0)
        return 1;                    /* ~(0 & x) = ~0 */
    if (a == 1)
        return tc_net_not(t, b);     /* ~(~0 & x) = ~x */
    if (a == b)
        return tc_net_not(t, a);
    size_t h = hkey(a, b) & (t->nslot - 1);
    while (t->slot[h]) {
        const TcNode *x = &t->node[t->slot[h] - 1];
        if (x->kind == TN_NAND && x->a == a && x->b == b)
            return t->slot[h] - 1;
        h = (h + 1) & (t->nslot - 1);
    }
    int n = add(t, TN_NAND, a, b, 0);
    t->slot[h] = n + 1;
    if (2 * (size_t)t->n > t->nslot)
        rehash(t);
    return n;
}

/* ~a, represented as a one-input NAND; ~~x folds to x and ~const to the other constant. */
int tc_net_not(TcNet *t, int a)
{
    if (a == 0)
        return 1;
    if (a == 1)
        return 0;
    if (t->node[a].kind == TN_NOT)
        return t->node[a].a;
    size_t h = hkey(a, -1) & (t->nslot - 1);
    while (t->slot[h]) {
        const TcNode *x = &t->node[t->slot[h] - 1];
        if (x->kind == TN_NOT && x->a == a)
            return t->slot[h] - 1;
        h = (h + 1) & (t->nslot - 1);
    }
    int n = add(t, TN_NOT, a, -1, 0);
    t->slot[h] = n + 1;
    if (2 * (size_t)t->n > t->nslot)
        rehash(t);
    return n;
}

const TcNode *tc_net_node(const TcNet *t, int i) { return &t->node[i]; }
int tc_net_size(const TcNet *t) { return t->n; }

/* ---- cuts --------------------------------------------------------------------------------------- */

static const uint8_t PAT[3] = {0xf0, 0xcc, 0xaa};

/* tt over leaves `from` (nf of them) re-expressed over the superset `to` (nt). */
static uint8_t expand(uint8_t tt, const int *from, int nf, const int *to, int nt)
{
    int pos[3] = {0, 0, 0};
    for (int i = 0; i < nf; i++)
        for (int j = 0; j < nt; j++)
            if (from[i] == to[j])
                pos[i] = j;
    uint8_t out = 0;
    for (int r = 0; r < 8; r++) {
        int idx = 0;
        for (int i = 0; i < nf; i++)
            if ((PAT[pos[i]] >> r) & 1)
                idx |= 1 << (2 - i);
        /* idx: the row of tt where leaf i has the value it has in row r of `to` */
        if ((tt >> idx) & 1)
            out |= (uint8_t)(1u << r);
    }
    return out;
}

static int merge_leaves(const Cut *x, const Cut *y, int *out)
{
    int n = 0;
    for (int i = 0; i < x->n; i++)
        out[n++] = x->leaf[i];
    for (int j = 0; j < y->n; j++) {
        int dup = 0;
        for (int i = 0; i < x->n; i++)
            dup |= x->leaf[i] == y->leaf[j];
        if (!dup) {
            if (n == 3)
                return -1;
            out[n++] = y->leaf[j];
        }
    }
    /* sort */
    for (int i = 1; i < n; i++)
        for (int j = i; j > 0 && out[j - 1] > out[j]; j--) {
            int s = out[j];
            out[j] = out[j - 1];
            out[j - 1] = s;
        }
    return n;
}

static float leaf_flow(const TcNet *t, int l)
{
    const TcNode *x = &t->node[l];
    if (x->kind == TN_LEAF || x->kind == TN_CONST)
        return 0.f;
    return t->flow[l] / (float)(t->refs[l] > 0 ? t->refs[l] : 1);
}

static void add_cut(TcNet *t, int n, const Cut *c)
{
    Cut *cs = &t->cuts[(size_t)n * PRIO];
    int k = t->ncut[n];
    for (int i = 0; i < k; i++)
        if (cs[i].n == c->n && !memcmp(cs[i].leaf, c->leaf, (size_t)c->n * sizeof(int)))
            return;
    if (k < PRIO) {
        cs[k] = *c;
        t->ncut[n] = k + 1;
    } else {
        int worst = 0;
        for (int i = 1; i < k; i++)
            if (cs[i].flow > cs[worst].flow)
                worst = i;
        if (c->flow < cs[worst].flow)
            cs[worst] = *c;
    }
}

static void cuts_of(TcNet *t, int n)
{
    const TcNode *x = &t->node[n];
    t->ncut[n] = 0;
    if (x->kind == TN_CONST || x->kind == TN_LEAF) {
        Cut c = {{n, 0, 0}, 1, 0xf0, 0.f};
        t->cuts[(size_t)n * PRIO] = c;
        t->ncut[n] = 1;
        t->flow[n] = 0.f;
        return;
    }
    if (x->kind == TN_NOT) {
        const Cut *ca = &t->cuts[(size_t)x->a * PRIO];
        for (int i = 0; i < t->ncut[x->a]; i++) {
            Cut c = ca[i];
            if (c.n == 1 && c.leaf[0] == x->a && t->node[x->a].kind != TN_LEAF &&
                t->node[x->a].kind != TN_CONST) {
                /* the trivial cut of the fanin: NOT over it */
            }
            c.tt = (uint8_t)~c.tt;
            c.flow = 1.f;
            for (int j = 0; j < c.n; j++)
                c.flow += leaf_flow(t, c.leaf[j]);
            add_cut(t, n, &c);
        }
    } else {
        const Cut *ca = &t->cuts[(size_t)x->a * PRIO], *cb = &t->cuts[(size_t)x->b * PRIO];
        for (int i = 0; i < t->ncut[x->a]; i++)
            for (int j = 0; j < t->ncut[x->b]; j++) {
                Cut c;
                c.n = merge_leaves(&ca[i], &cb[j], c.leaf);
                if (c.n < 0)
                    continue;
                uint8_t ta = expand(ca[i].tt, ca[i].leaf, ca[i].n, c.leaf, c.n);
                uint8_t tb = expand(cb[j].tt, cb[j].leaf, cb[j].n, c.leaf, c.n);
                c.tt = (uint8_t)~(ta & tb);
                c.flow = 1.f;
                for (int k = 0; k < c.n; k++)
                    c.flow += leaf_flow(t, c.leaf[k]);
                add_cut(t, n, &c);
            }
    }
    float best = 1e30f;
    for (int i = 0; i < t->ncut[n]; i++)
        if (t->cuts[(size_t)n * PRIO + i].flow < best)
            best = t->cuts[(size_t)n * PRIO + i].flow;
    t->flow[n] = best;
    /* the node as a leaf of its fanouts' cuts */
    Cut self = {{n, 0, 0}, 1, 0xf0, 0.f};
    /* keep the trivial cut last-resort: it does not count toward this node's own flow */
    Cut *cs = &t->cuts[(size_t)n * PRIO];
    if (t->ncut[n] < PRIO) {
        cs[t->ncut[n]++] = self;
    } else {
        int worst = 0;
        for (int i = 1; i < PRIO; i++)
            if (cs[i].flow > cs[worst].flow)
                worst = i;
        cs[worst] = self;
    }
}

static int is_gate(const TcNet *t, int n)
{
    return t->node[n].kind == TN_NAND || t->node[n].kind == TN_NOT;
}

static const Cut *chosen(const TcNet *t, int n)
{
    return &t->cuts[(size_t)n * PRIO + t->best[n]];
}

/* Reference counting of the cover: taking cut c for node n references its leaves; a leaf whose
   count rises from 0 enters the cover with its own chosen cut.  Both return the LUTs entering
   (or leaving) the cover. */
static int cover_ref(TcNet *t, const Cut *c)
{
    int area = 1;
    for (int i = 0; i < c->n; i++) {
        int l = c->leaf[i];
        if (is_gate(t, l) && t->refs[l]++ == 0)
            area += cover_ref(t, chosen(t, l));
    }
    return area;
}

static int cover_deref(TcNet *t, const Cut *c)
{
    int area = 1;
    for (int i = 0; i < c->n; i++) {
        int l = c->leaf[i];
        if (is_gate(t, l) && --t->refs[l] == 0)
            area += cover_deref(t, chosen(t, l));
    }
    return area;
}

static int usable(const TcNet *t, int n, int k)
{
    const Cut *c = &t->cuts[(size_t)n * PRIO + k];
    return !(c->n == 1 && c->leaf[0] == n);  /* the trivial cut cannot implement n itself */
}

/* Area recovery: each node in the cover takes the cut that brings the fewest LUTs in. */
static void exact_area(TcNet *t, int passes)
{
    int n = t->n;
    for (int pass = 0; pass < passes; pass++)
        for (int j = 0; j < n; j++) {
            int i = pass & 1 ? n - 1 - j : j;
            if (!is_gate(t, i) || t->refs[i] == 0)
                continue;
            cover_deref(t, chosen(t, i));
            int b = t->best[i], least = 1 << 30;
            for (int k = 0; k < t->ncut[i]; k++) {
                if (!usable(t, i, k))
                    continue;
                const Cut *c = &t->cuts[(size_t)i * PRIO + k];
                int a = cover_ref(t, c);
                cover_deref(t, c);
                if (a < least) {
                    least = a;
                    b = k;
                }
            }
            t->best[i] = b;
            cover_ref(t, chosen(t, i));
        }
}

/* The cover from scratch: the outputs' chosen cuts and, recursively, their leaves'. */
static void recount(TcNet *t, const int *outputs, int nout)
{
    memset(t->refs, 0, (size_t)t->n * sizeof *t->refs);
    for (int i = 0; i < nout; i++)
        if (is_gate(t, outputs[i]) && t->refs[outputs[i]]++ == 0)
            cover_ref(t, chosen(t, outputs[i]));
}

static int cut_has(const Cut *c, int node)
{
    for (int j = 0; j < c->n; j++)
        if (c->leaf[j] == node)
            return 1;
    return 0;
}

typedef struct {
    uint64_t key;  /* the leaf set */
    int      node, cut;
} LeafSet;

static int by_leafset(const void *x, const void *y)
{
    const LeafSet *a = x, *b = y;
    return a->key < b->key ? -1 : a->key > b->key ? 1 : a->node - b->node;
}

/* One sweep of joint moves; returns how many groups moved. */
static int joint_moves(TcNet *t)
{
    int n = t->n, moved = 0;
    size_t cap = 0, m = 0;
    LeafSet *ls = NULL;
    for (int i = 0; i < n; i++) {
        if (!is_gate(t, i) || t->refs[i] == 0)
            continue;
        for (int k = 0; k < t->ncut[i]; k++) {
            const Cut *c = &t->cuts[(size_t)i * PRIO + k];
            if (!usable(t, i, k) || c->n < 2 || k == t->best[i])
                continue;
            if (m == cap) {
                cap = cap ? 2 * cap : 1024;
                ls = tc_xrealloc(ls, cap * sizeof *ls);
            }
            uint64_t key = 0;
            for (int j = 0; j < c->n; j++)
                key = key * 0x100000001b3ull + (uint64_t)(c->leaf[j] + 1);
            ls[m].key = key ^ (uint64_t)c->n << 60;
            ls[m].node = i;
            ls[m].cut = k;
            m++;
        }
    }
    qsort(ls, m, sizeof *ls, by_leafset);
    for (size_t a = 0; a < m;) {
        size_t b = a + 1;
        while (b < m && ls[b].key == ls[a].key)
            b++;
        if (b - a >= 2) {
            /* the group's nodes as they are, then all switched */
            int before = 0, after = 0, ok = 1, old[8], cnt = (int)(b - a < 8 ? b - a : 8);
            for (int q = 0; q < cnt; q++) {
                ok &= t->refs[ls[a + q].node] > 0;
                for (int r = 0; r < cnt; r++)  /* no member a leaf of another's cuts */
                    ok &= !cut_has(chosen(t, ls[a + q].node), ls[a + r].node) &&
                          !cut_has(&t->cuts[(size_t)ls[a + q].node * PRIO + ls[a + q].cut],
                                   ls[a + r].node);
            }
            if (ok) {
                for (int q = 0; q < cnt; q++) {
                    old[q] = t->best[ls[a + q].node];
                    before += cover_deref(t, chosen(t, ls[a + q].node));
                }
                for (int q = 0; q < cnt; q++) {
                    t->best[ls[a + q].node] = ls[a + q].cut;
                    after += cover_ref(t, chosen(t, ls[a + q].node));
                }
                if (after >= before) {  /* no gain: back as it was */
                    for (int q = 0; q < cnt; q++)
                        cover_deref(t, chosen(t, ls[a + q].node));
                    for (int q = 0; q < cnt; q++) {
                        t->best[ls[a + q].node] = old[q];
                        cover_ref(t, chosen(t, ls[a + q].node));
                    }
                } else {
                    moved++;
                }
            }
        }
        a = b;
    }
    free(ls);
    return moved;
}

int tc_net_map(TcNet *t, const int *outputs, int nout, int *order, int *norder)
{
    int n = t->n;
    t->cuts = tc_xrealloc(t->cuts, (size_t)n * PRIO * sizeof *t->cuts);
    t->ncut = tc_xrealloc(t->ncut, (size_t)n * sizeof *t->ncut);
    t->refs = tc_xcalloc((size_t)n, sizeof *t->refs);
    t->flow = tc_xcalloc((size_t)n, sizeof *t->flow);
    t->best = tc_xcalloc((size_t)n, sizeof *t->best);
    t->need = tc_xcalloc((size_t)n, 1);
    /* fanouts, for the area flow of the cuts */
    for (int i = 0; i < n; i++) {
        if (t->node[i].kind == TN_NAND) {
            t->refs[t->node[i].a]++;
            t->refs[t->node[i].b]++;
        } else if (t->node[i].kind == TN_NOT) {
            t->refs[t->node[i].a]++;
        }
    }
    for (int i = 0; i < nout; i++)
        t->refs[outputs[i]]++;
    for (int i = 0; i < n; i++)
        cuts_of(t, i);
    /* first choice: the least area flow */
    for (int i = 0; i < n; i++) {
        if (!is_gate(t, i))
            continue;
        int b = -1;
        for (int k = 0; k < t->ncut[i]; k++)
            if (usable(t, i, k) &&
                (b < 0 || t->cuts[(size_t)i * PRIO + k].flow < t->cuts[(size_t)i * PRIO + b].flow))
                b = k;
        t->best[i] = b;
    }
    /* area flow again with the fanouts the cover really has (blended with the estimate before),
       twice: cuts that absorb a shared node into several LUTs lose their false advantage */
    float *est = tc_xmalloc((size_t)n * sizeof *est);
    for (int i = 0; i < n; i++)
        est[i] = (float)(t->refs[i] > 0 ? t->refs[i] : 1);
    for (int round = 0; round < 3; round++) {
        memset(t->refs, 0, (size_t)n * sizeof *t->refs);
        for (int i = 0; i < nout; i++)
            if (is_gate(t, outputs[i]) && t->refs[outputs[i]]++ == 0)
                cover_ref(t, chosen(t, outputs[i]));
        for (int i = 0; i < n; i++)
            est[i] = 0.5f * est[i] + 0.5f * (float)(t->refs[i] > 0 ? t->refs[i] : 1);
        for (int i = 0; i < n; i++) {
            if (!is_gate(t, i))
                continue;
            float bestf = 1e30f;
            for (int k = 0; k < t->ncut[i]; k++) {
                if (!usable(t, i, k))
                    continue;
                const Cut *c = &t->cuts[(size_t)i * PRIO + k];
                float f = 1.f;
                for (int j = 0; j < c->n; j++)
                    if (is_gate(t, c->leaf[j]))
                        f += t->flow[c->leaf[j]] / est[c->leaf[j]];
                if (f < bestf) {
                    bestf = f;
                    t->best[i] = k;
                }
            }
            t->flow[i] = bestf;
        }
    }
    free(est);
    /* the cover of the outputs, reference counted */
    memset(t->refs, 0, (size_t)n * sizeof *t->refs);
    for (int i = 0; i < nout; i++)
        if (is_gate(t, outputs[i]) && t->refs[outputs[i]]++ == 0)
            cover_ref(t, chosen(t, outputs[i]));
    exact_area(t, 6);
    /* joint moves: cover nodes that each have a cut over the same leaves (a full adder's sum
       and carry over its three inputs) switch to those cuts together when that shrinks the
       cover, which no single node's move shows; then the single moves again */
    for (int round = 0; round < 3; round++) {
        int moved = joint_moves(t);
        recount(t, outputs, nout);
        if (!moved)
            break;
        exact_area(t, 2);
    }
    recount(t, outputs, nout);
    int m = 0;
    for (int i = 0; i < n; i++)
        if (is_gate(t, i) && t->refs[i] > 0) {
            t->need[i] = 1;
            order[m++] = i;
        }
    *norder = m;
    return m;
}

void tc_net_lut(const TcNet *t, int node, int *leaves, int *nleaves, uint8_t *tt)
{
    const Cut *c = &t->cuts[(size_t)node * PRIO + t->best[node]];
    for (int i = 0; i < c->n; i++)
        leaves[i] = c->leaf[i];
    *nleaves = c->n;
    *tt = c->tt;
}

/* One pass of p from power-on (cells 0, ONE ~0, RR 0) with input k held by node leaves[k]:
   cur[c] gets the node of cell c's value at the end of the pass. */
void tc_net_pass(TcNet *net, const Program *p, const uint32_t *in_cells, size_t n,
                 const int *leaves, int *cur)
{
    for (uint32_t c = 0; c < p->ncells; c++)
        cur[c] = 0;
    cur[CELL_ONE] = 1;
    for (size_t k = 0; k < n; k++)
        cur[in_cells[k]] = leaves[k];
    int rr = 0;
    for (size_t i = 0; i < p->len; i++) {
        Instr in = p->code[i];
        if (in.op == OP_NAND)
            rr = tc_net_nand(net, rr, cur[in.addr]);
        else if (in.addr >= CELL_FIRST_FREE)
            cur[in.addr] = rr;
    }
}
