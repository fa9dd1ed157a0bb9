/* The superoptimizer's host side: the specification language, the drop-in entry points and the
   program check.

   The language is the reference's (src/super.h:1-16): statements "name [{a,b}] = expr" or
   "name := expr" (a given cell), separated by ';'.  Names on the left are written (RR or cells),
   every other name read is an input; a cell on both sides starts with its input value and ends
   with its output value; "{a,b}" lets an output share its cell with those inputs.  Expressions:
   names, 0, 1, ! ~ (prefix), & (tightest), ^, |, ?: (loosest, right associative) and
   parentheses, on truth tables (row r of input variable i is bit i of r).  The variables are RR
   first when it is read, then the names read, in order of first appearance; given cells are not
   variables.  The parsed form is the reference's SuperSpec (src/super.h:24-40), byte for byte,
   and the error messages are its own, so either parser's output can be passed on.

   Here the text is read once: each statement's right side becomes a small expression tree while
   the names are collected; the trees are evaluated after the variables are numbered, given cells
   first.  Interchangeable inputs (swapping two leaves every target, given cell and sharing
   unchanged) are found by permuting truth-table rows, so the search reads them in order.  The
   check runs a program over every sharing of cells and, exactly, over every value of the garbage
   it can observe. */
#include <ctype.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include "engine.h"
#include "super_search.cuh"

int tc_super_run(const SpSpec *sp, int max_cost, int lb, int *found, int *cost, int *below,
                 SpState *sol, unsigned long long *nodes, double *seconds, int quiet, char *err,
                 size_t errlen);

/* ---- the language ------------------------------------------------------------------------------ */

enum { X_ZERO, X_ONE, X_NAME, X_NOT, X_AND, X_XOR, X_OR, X_COND };

typedef struct {
    uint8_t kind;
    int     a, b, c;  /* operands (node indices); X_NAME: a = index into the names read */
} XNode;

typedef struct {
    char lhs[SUPER_NAME];
    char alias[4][SUPER_NAME];
    int  nalias, given, root;
} XStmt;

typedef struct {
    const char *at;
    char       *err;
    size_t      errlen;
    int         bad;
    XNode      *node;
    int         nnode, capnode;
    char        read[SUPER_CELLS + 1][SUPER_NAME];  /* names read, in order of first appearance */
    int         nread;
    XStmt       st[SUPER_CELLS];
    int         nst;
} XParse;

static void xfail(XParse *p, const char *fmt, ...)
{
    if (p->bad++)
        return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(p->err, p->errlen, fmt, ap);
    va_end(ap);
}

static void xskip(XParse *p)
{
    while (isspace((unsigned char)*p->at))
        p->at++;
}

/* A name, of at most SUPER_NAME - 1 characters: a longer run of name characters leaves its tail
   for the next token, as the reference's reader does.  0 if no name starts here. */
static int xname(XParse *p, char *out)
{
    xskip(p);
    if (!isalpha((unsigned char)*p->at) && *p->at != '_')
        return 0;
    int n = 0;
    while (n < SUPER_NAME - 1 && (isalnum((unsigned char)*p->at) || *p->at == '_'))
        out[n++] = *p->at++;
    out[n] = '\0';
    return 1;
}

static int is_rr(const char *n)
{
    return tc_same_name(n, "RR");
}

static int xnode(XParse *p, int kind, int a, int b, int c)
{
    if (p->nnode == p->capnode) {
        p->capnode = p->capnode ? 2 * p->capnode : 64;
        p->node = tc_xrealloc(p->node, (size_t)p->capnode * sizeof *p->node);
    }
    XNode *x = &p->node[p->nnode];
    x->kind = (uint8_t)kind;
    x->a = a;
    x->b = b;
    x->c = c;
    return p->nnode++;
}

static int xcond(XParse *p);

/* operand: ( cond ) | 0 | 1 | ! operand | ~ operand | name */
static int xoperand(XParse *p)
{
    xskip(p);
    char c = *p->at;
    if (c == '(') {
        p->at++;
        int e = xcond(p);
        xskip(p);
        if (*p->at == ')')
            p->at++;
        else
            xfail(p, "expected )");
        return e;
    }
    if (c == '0' || c == '1') {
        p->at++;
        return xnode(p, c == '1' ? X_ONE : X_ZERO, 0, 0, 0);
    }
    if (c == '!' || c == '~') {
        p->at++;
        return xnode(p, X_NOT, xoperand(p), 0, 0);
    }
    char name[SUPER_NAME];
    if (!xname(p, name)) {
        xfail(p, "expected a name, 0, 1 or ( at \"%.20s\"", p->at);
        return xnode(p, X_ZERO, 0, 0, 0);
    }
    int k = 0;
    while (k < p->nread && strcmp(p->read[k], name))
        k++;
    if (k == p->nread) {
        if (p->nread == SUPER_CELLS + 1) {
            xfail(p, "too many names");
            return xnode(p, X_ZERO, 0, 0, 0);
        }
        snprintf(p->read[p->nread++], SUPER_NAME, "%s", name);
    }
    return xnode(p, X_NAME, k, 0, 0);
}

/* Binary operators by precedence climbing: & binds tighter than ^, ^ tighter than |. */
static int xbinary(XParse *p, int min_prec)
{
    int left = xoperand(p);
    while (!p->bad) {
        xskip(p);
        char c = *p->at;
        int prec = c == '&' ? 3 : c == '^' ? 2 : c == '|' ? 1 : 0;
        if (!prec || prec < min_prec)
            break;
        p->at++;
        int right = xbinary(p, prec + 1);
        left = xnode(p, prec == 3 ? X_AND : prec == 2 ? X_XOR : X_OR, left, right, 0);
    }
    return left;
}

/* cond: binary [ ? cond : cond ] */
static int xcond(XParse *p)
{
    int c = xbinary(p, 1);
    xskip(p);
    if (p->bad || *p->at != '?')
        return c;
    p->at++;
    int a = xcond(p);
    xskip(p);
    if (*p->at == ':')
        p->at++;
    else
        xfail(p, "expected : in ?:");
    int b = p->bad ? a : xcond(p);
    return xnode(p, X_COND, c, a, b);
}

/* Statements: name [{a, b, ...}] (= | :=) cond, separated by ';'. */
static void xstatements(XParse *p)
{
    for (xskip(p); *p->at && !p->bad; xskip(p)) {
        if (p->nst == SUPER_CELLS) {
            xfail(p, "too many statements");
            return;
        }
        XStmt *t = &p->st[p->nst++];
        memset(t, 0, sizeof *t);
        if (!xname(p, t->lhs)) {
            xfail(p, "expected a name at \"%.20s\"", p->at);
            return;
        }
        xskip(p);
        if (*p->at == '{') {
            p->at++;
            do {
                if (t->nalias == 4 || !xname(p, t->alias[t->nalias])) {
                    xfail(p, "expected names in { }");
                    return;
                }
                t->nalias++;
                xskip(p);
            } while (*p->at == ',' && p->at++);
            if (*p->at != '}') {
                xfail(p, "expected }");
                return;
            }
            p->at++;
            xskip(p);
        }
        if (p->at[0] == ':' && p->at[1] == '=') {
            t->given = 1;
            p->at += 2;
        } else if (p->at[0] == '=') {
            p->at++;
        } else {
            xfail(p, "expected = after %s", t->lhs);
            return;
        }
        t->root = xcond(p);
        xskip(p);
        if (*p->at == ';')
            p->at++;
        else if (*p->at && !p->bad)
            xfail(p, "unexpected \"%.20s\"", p->at);
    }
}

static int spec_cell(const SuperSpec *sp, const char *name)
{
    for (int i = 0; i < sp->ncells; i++)
        if (!strcmp(sp->cell[i].name, name))
            return i;
    return -1;
}

/* The truth table of node x (64 rows; the caller masks), reading names through the spec's cells
   (RR is variable 0).  Operands are evaluated in source order, so the first unknown name is the
   one reported. */
static uint64_t xvalue(XParse *p, const SuperSpec *sp, int x)
{
    const XNode *n = &p->node[x];
    switch (n->kind) {
    case X_ZERO: return 0;
    case X_ONE:  return ~0ull;
    case X_NOT:  return ~xvalue(p, sp, n->a);
    case X_NAME: {
        const char *name = p->read[n->a];
        if (is_rr(name))
            return sp_var_table(0);
        int c = spec_cell(sp, name);
        if (c < 0)
            xfail(p, "unknown name %s", name);
        return c < 0 ? 0 : sp->cell[c].init;
    }
    case X_COND: {
        uint64_t c = xvalue(p, sp, n->a), t = xvalue(p, sp, n->b), f = xvalue(p, sp, n->c);
        return (c & t) | (~c & f);
    }
    default: {
        uint64_t l = xvalue(p, sp, n->a), r = xvalue(p, sp, n->b);
        return n->kind == X_AND ? l & r : n->kind == X_XOR ? l ^ r : l | r;
    }
    }
}

static int new_cell(XParse *p, SuperSpec *sp, const char *name)
{
    if (sp->ncells == SUPER_CELLS) {
        xfail(p, "too many cells");
        return -1;
    }
    int c = sp->ncells++;
    snprintf(sp->cell[c].name, SUPER_NAME, "%s", name);
    return c;
}

/* ---- interchangeable inputs ---------------------------------------------------------------------- */

/* The truth table f over n variables with variables i and j exchanged: row r moves to the row
   whose bits i and j are swapped. */
static uint64_t exchanged(uint64_t f, int i, int j, int n)
{
    uint64_t g = 0;
    for (int r = 0; r < 1 << n; r++) {
        int d = ((r >> i) ^ (r >> j)) & 1;           /* bits differ: the rows pair up */
        int q = r ^ (d << i) ^ (d << j);
        g |= ((f >> r) & 1) << q;
    }
    return g;
}

/* Inputs i < j (plain inputs: read, not written, not given) are interchangeable when exchanging
   their variables leaves RR's target, every output's target and every given cell's value
   unchanged, and every output may share with both or neither.  The interchangeable inputs form
   chains: j follows the last member of the chain that i is in, and the search reads a member
   only after the one before it (sym_prev). */
static void interchangeable(SuperSpec *sp, const int *var_of)
{
    int next[SUPER_CELLS];
    for (int c = 0; c < sp->ncells; c++) {
        sp->cell[c].sym_prev = -1;
        next[c] = -1;
    }
    const uint64_t m = sp->mask;
#define PLAIN_INPUT(c) (sp->cell[c].in && !sp->cell[c].out && var_of[c] >= 0)
    for (int i = 0; i < sp->ncells; i++) {
        if (!PLAIN_INPUT(i))
            continue;
        for (int j = i + 1; j < sp->ncells; j++) {
            if (!PLAIN_INPUT(j) || sp->cell[j].sym_prev >= 0)
                continue;
            int vi = var_of[i], vj = var_of[j], n = sp->nvars;
            int same = !sp->rr_out || exchanged(sp->rr_target, vi, vj, n) == sp->rr_target;
            for (int c = 0; c < sp->ncells && same; c++) {
                const uint64_t *t = sp->cell[c].out ? &sp->cell[c].target : NULL;
                if (t && (exchanged(*t, vi, vj, n) & m) != (*t & m))
                    same = 0;
                if (sp->cell[c].in && var_of[c] < 0 &&
                    (exchanged(sp->cell[c].init, vi, vj, n) & m) != (sp->cell[c].init & m))
                    same = 0;
                if (((sp->cell[c].alias >> i) ^ (sp->cell[c].alias >> j)) & 1)
                    same = 0;
            }
            if (!same)
                continue;
            int tail = i;
            while (next[tail] >= 0)
                tail = next[tail];
            sp->cell[j].sym_prev = tail;
            next[tail] = j;
        }
    }
#undef PLAIN_INPUT
}

int cuda_super_parse(const char *text, SuperSpec *sp, char *err, size_t errlen)
{
    XParse p;
    memset(&p, 0, sizeof p);
    memset(sp, 0, sizeof *sp);
    p.at = text;
    p.err = err;
    p.errlen = errlen;
    err[0] = '\0';
    xstatements(&p);
    if (p.bad) {
        free(p.node);
        return 0;
    }

    /* variables: RR first when read, then the other names read, in order; given cells are not */
    int var_of[SUPER_CELLS];
    for (int c = 0; c < SUPER_CELLS; c++)
        var_of[c] = -1;
    for (int k = 0; k < p.nread; k++)
        sp->rr_in |= is_rr(p.read[k]);
    sp->nvars = sp->rr_in;
    for (int k = 0; k < p.nread && !p.bad; k++) {
        int given = 0;
        for (int s = 0; s < p.nst; s++)
            given |= p.st[s].given && !strcmp(p.st[s].lhs, p.read[k]);
        if (is_rr(p.read[k]) || given)
            continue;
        if (sp->nvars == SUPER_VARS) {
            xfail(&p, "more than %d inputs", SUPER_VARS);
            break;
        }
        int c = sp->ncells++;
        snprintf(sp->cell[c].name, SUPER_NAME, "%s", p.read[k]);
        sp->cell[c].in = 1;
        var_of[c] = sp->nvars;
        sp->cell[c].init = sp_var_table(sp->nvars++);
    }
    sp->mask = sp->nvars == SUPER_VARS ? ~0ull : (1ull << (1 << sp->nvars)) - 1;

    /* the given cells' values, then the outputs' targets */
    for (int outputs = 0; outputs < 2 && !p.bad; outputs++)
        for (int s = 0; s < p.nst && !p.bad; s++) {
            XStmt *t = &p.st[s];
            if (t->given == outputs)
                continue;
            uint64_t v = xvalue(&p, sp, t->root) & sp->mask;
            if (is_rr(t->lhs)) {
                if (t->given || sp->rr_out || t->nalias)
                    xfail(&p, "RR is set once, with =");
                sp->rr_out = 1;
                sp->rr_target = v;
                continue;
            }
            int c = spec_cell(sp, t->lhs);
            if (t->given) {
                if (c >= 0)
                    xfail(&p, "%s is defined twice", t->lhs);
                else if ((c = new_cell(&p, sp, t->lhs)) >= 0) {
                    sp->cell[c].in = 1;
                    sp->cell[c].init = v;
                }
                continue;
            }
            if (c >= 0 && sp->cell[c].out) {
                xfail(&p, "%s is set twice", t->lhs);
                break;
            }
            if (c < 0 && (c = new_cell(&p, sp, t->lhs)) < 0)
                break;
            if (sp->cell[c].in && var_of[c] < 0) {
                xfail(&p, "%s is a given cell", t->lhs);
                break;
            }
            sp->cell[c].out = 1;
            sp->cell[c].target = v;
            for (int k = 0; k < t->nalias; k++) {
                int a = spec_cell(sp, t->alias[k]);
                if (a < 0 || !sp->cell[a].in || a == c)
                    xfail(&p, "%s{%s}: %s must be another input", t->lhs, t->alias[k],
                          t->alias[k]);
                else
                    sp->cell[c].alias |= 1u << a;
            }
        }
    int any_output = 0;
    for (int c = 0; c < sp->ncells && !p.bad; c++) {
        any_output |= sp->cell[c].out;
        for (int a = 0; a < sp->ncells && sp->cell[c].out; a++)
            if (((sp->cell[c].alias >> a) & 1) && sp->cell[a].out)
                xfail(&p, "%s may share a cell only with inputs that are not written",
                      sp->cell[c].name);
    }
    if (!p.bad && !sp->rr_out && !any_output)
        xfail(&p, "nothing to compute: no RR = ... and no cell = ...");
    free(p.node);
    if (p.bad)
        return 0;
    interchangeable(sp, var_of);
    return 1;
}

/* ---- the search ------------------------------------------------------------------------------- */

static void to_device_spec(const SuperSpec *s, SpSpec *d)
{
    memset(d, 0, sizeof *d);
    d->nvars = s->nvars;
    d->rr_in = s->rr_in;
    d->rr_out = s->rr_out;
    d->ncells = s->ncells;
    d->mask = s->mask;
    d->rr_target = s->rr_target;
    for (int c = 0; c < s->ncells; c++) {
        d->init[c] = s->cell[c].init;
        d->target[c] = s->cell[c].target;
        d->alias[c] = s->cell[c].alias;
        d->in[c] = (uint8_t)s->cell[c].in;
        d->out[c] = (uint8_t)s->cell[c].out;
        d->sym_prev[c] = (int8_t)s->cell[c].sym_prev;
    }
}

/* The program of a goal state: NAND i reads its operand, an RR value needed later is stored
   right after it appears (scratch cells t1, t2, ... in order), outputs right after the NAND that
   made their value (src/super.c:732-767). */
static void program_of(const SuperSpec *sp, const SpState *x, SuperProg *p)
{
    int temp[SP_LEN + 1], ntemps = 0;
    p->len = 0;
    for (int j = 0; j <= x->n; j++)
        temp[j] = x->stored[j] ? ++ntemps : 0;
#define PUT(o, ...)                                                                                \
    do {                                                                                           \
        p->code[p->len].op = (uint8_t)(o);                                                         \
        snprintf(p->code[p->len].cell, SUPER_NAME, __VA_ARGS__);                                   \
        p->len++;                                                                                  \
    } while (0)
    for (int i = 0; i <= x->n; i++) {
        if (i > 0) {
            int k = x->op_kind[i], r = x->op_ref[i];
            if (k == SK_ZERO)
                PUT(OP_NAND, "ZERO");
            else if (k == SK_ONE)
                PUT(OP_NAND, "ONE");
            else if (k == SK_CELL)
                PUT(OP_NAND, "%s", sp->cell[r].name);
            else
                PUT(OP_NAND, "_t%d", temp[r]);
        }
        if (x->stored[i])
            PUT(OP_STO, "_t%d", temp[i]);
        for (int c = 0; c < sp->ncells; c++)
            if (x->out_at[c] == i)
                PUT(OP_STO, "%s", sp->cell[c].name);
    }
#undef PUT
}

int cuda_super_search(const SuperSpec *sp, const SuperOpts *o, SuperResult *r, char *err,
                      size_t errlen)
{
    memset(r, 0, sizeof *r);
    if (o->parts > 1)
        return tc_fail(err, errlen, "the GPU search runs the whole tree; --part is for CPUs");
    SpSpec d;
    to_device_spec(sp, &d);
    SpState root, sol;
    sp_reset(&d, &root);
    int lb = sp_lower_bound(&d, &root);
    int found = 0, cost = 0, below = lb;
    unsigned long long nodes = 0;
    double seconds = 0;
    if (!tc_super_run(&d, o->max_cost, lb, &found, &cost, &below, &sol, &nodes, &seconds, o->quiet,
                      err, errlen))
        return 0;
    r->found = found;
    r->cost = cost;
    r->below = below;
    r->nodes = nodes;
    r->seconds = seconds;
    if (found)
        program_of(sp, &sol, &r->prog);
    r->contradiction = found && cost != below;
    return 1;
}


/* ---- checking a program ---------------------------------------------------------------------- */

#define CHECK_EXACT_BITS 16   /* garbage bits enumerated in full; beyond, seeded random trials */
#define CHECK_TRIALS     4096

/* p against the specification (the contract of super_check, src/super.h:70-72): for every way
   the outputs may take the cells of their {inputs} (two outputs never in one cell), every input
   row and every garbage -- RR when it is not an input, output and scratch cells before they are
   written -- each output must end with its target, each input that no output took must keep its
   value, and RR must end with its target when it has one.  Instructions name the spec's cells,
   ZERO, ONE (never stored to) or scratch cells (any other name).

   The check is exact.  Rows do not interact (every operation is bitwise over the truth table's
   rows), so giving each garbage bit one value in all rows at once and trying every combination
   covers every garbage of every row; and only garbage that is read before it is overwritten
   matters: the first read of RR, a read of a cell not yet written, an output or input never
   written and compared at the end.  Up to CHECK_EXACT_BITS such bits are enumerated in full;
   past that (no program of the search comes near), CHECK_TRIALS seeded random garbages are
   tried instead.  Messages are the reference's. */
int cuda_super_check(const SuperSpec *sp, const SuperProg *p, char *err, size_t errlen)
{
    enum { ZERO_REF = -1, ONE_REF = -2 };
    char scratch[SUPER_LEN][SUPER_NAME];
    int nscratch = 0, ref[SUPER_LEN], ncells;
    for (int i = 0; i < p->len; i++) {
        const char *n = p->code[i].cell;
        int constant = !strcmp(n, "ZERO") ? ZERO_REF : !strcmp(n, "ONE") ? ONE_REF : 0;
        if (constant && p->code[i].op == OP_STO)
            return tc_fail(err, errlen, "instruction %d stores to a constant", i);
        if (constant) {
            ref[i] = constant;
            continue;
        }
        int c = spec_cell(sp, n);
        if (c < 0) {
            int k = 0;
            while (k < nscratch && strcmp(scratch[k], n))
                k++;
            if (k == nscratch)
                snprintf(scratch[nscratch++], SUPER_NAME, "%s", n);
            c = sp->ncells + k;
        }
        ref[i] = c;
    }
    ncells = sp->ncells + nscratch;

    int outs[SUPER_CELLS], nout = 0, choices[SUPER_CELLS], pick[SUPER_CELLS];
    for (int c = 0; c < sp->ncells; c++)
        if (sp->cell[c].out && !sp->cell[c].in) {
            choices[nout] = __builtin_popcount(sp->cell[c].alias);
            pick[nout] = 0;
            outs[nout++] = c;
        }
    uint64_t seed = 0x5ca1ab1e;
    for (;;) {  /* the sharings, pick[0] fastest: 0 = the output's own cell, k = its k-th input */
        int home[SUPER_CELLS + SUPER_LEN], clash = 0, taken[SUPER_CELLS] = {0};
        for (int c = 0; c < ncells; c++)
            home[c] = c;
        for (int i = 0; i < nout; i++) {
            uint32_t a = sp->cell[outs[i]].alias;
            for (int k = 1; k < pick[i]; k++)
                a &= a - 1;
            if (pick[i])
                home[outs[i]] = __builtin_ctz(a);
        }
        for (int i = 0; i < nout; i++)
            for (int j = i + 1; j < nout; j++)
                clash |= home[outs[i]] == home[outs[j]];
        for (int i = 0; i < nout; i++)
            if (home[outs[i]] != outs[i])
                taken[home[outs[i]]] = 1;

        /* the garbage bits this sharing can observe: garbage[g] is a cell, or -1 for RR */
        int garbage[1 + SUPER_CELLS + SUPER_LEN], ng = 0, written[SUPER_CELLS + SUPER_LEN] = {0};
        for (int c = 0; c < sp->ncells; c++)
            written[c] = sp->cell[c].in;  /* inputs hold known values */
        if (!sp->rr_in && (p->len || sp->rr_out))
            garbage[ng++] = -1;
        for (int i = 0; i < p->len; i++) {
            int c = ref[i] >= 0 ? home[ref[i]] : -1;
            if (c >= 0 && p->code[i].op == OP_NAND && !written[c])
                garbage[ng++] = c, written[c] = 1;
            if (c >= 0 && p->code[i].op == OP_STO)
                written[c] = 1;
        }
        for (int c = 0; c < sp->ncells; c++)
            if (!written[home[c]])
                garbage[ng++] = home[c], written[home[c]] = 1;

        uint64_t combos = ng <= CHECK_EXACT_BITS ? 1ull << ng : CHECK_TRIALS;
        for (uint64_t g = 0; g < combos && !clash; g++) {
            uint64_t val[SUPER_CELLS + SUPER_LEN] = {0}, rr = 0;
            for (int c = 0; c < sp->ncells; c++)
                if (sp->cell[c].in)
                    val[c] = sp->cell[c].init;
            if (sp->rr_in)
                rr = sp_var_table(0) & sp->mask;
            for (int k = 0; k < ng; k++) {
                uint64_t bits = ng <= CHECK_EXACT_BITS ? (g >> k & 1 ? ~0ull : 0)
                                                       : tc_splitmix64(&seed);
                if (garbage[k] < 0)
                    rr = bits & sp->mask;
                else
                    val[garbage[k]] = bits & sp->mask;
            }
            for (int i = 0; i < p->len; i++) {
                int c = ref[i] >= 0 ? home[ref[i]] : ref[i];
                if (p->code[i].op == OP_STO)
                    val[c] = rr;
                else
                    rr = ~(rr & (c == ZERO_REF ? 0 : c == ONE_REF ? sp->mask : val[c])) & sp->mask;
            }
            for (int c = 0; c < sp->ncells; c++) {
                if (sp->cell[c].in && !sp->cell[c].out && taken[c])
                    continue;  /* an output took this input's cell: its value may change */
                uint64_t want = sp->cell[c].out ? sp->cell[c].target : sp->cell[c].init;
                if (val[home[c]] != want)
                    return tc_fail(err, errlen, "%s %s (cells shared: variant %d)",
                                   sp->cell[c].name,
                                   sp->cell[c].out ? "does not get its value" : "is not kept",
                                   nout ? pick[0] : 0);
            }
            if (sp->rr_out && rr != sp->rr_target)
                return tc_fail(err, errlen, "RR does not end with its value");
        }
        int i = 0;
        while (i < nout && ++pick[i] > choices[i])
            pick[i++] = 0;
        if (i == nout)
            break;
    }
    return 1;
}
