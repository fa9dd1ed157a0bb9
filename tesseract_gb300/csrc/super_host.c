/* The superoptimizer's host side: the specification language, the drop-in entry points and the
   program check.

   Specifications (src/super.h:1-16): statements "name [{a,b}] = expr" or "name := expr" (a given
   cell), separated by ';'.  Names on the left are written (RR or cells), every other name read is
   an input; a cell on both sides starts with its input value and ends with its output value;
   "{a,b}" lets an output share its cell with those inputs.  Expressions: names, 0, 1, ! ~ & ^ |
   ?: and parentheses, evaluated on truth tables (row r of input variable i is bit i of r).  The
   variables are RR first when it is read, then the names read, in order; given cells are not
   variables.  Interchangeable inputs (swapping them leaves every target, given cell and sharing
   unchanged) are found so the search reads them in order.  The parsed form is the reference's
   SuperSpec (src/super.h:24-40), so its parser's output can be passed in as well. */
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

typedef struct {
    const char *s;
    SuperSpec  *sp;
    char       *err;
    size_t      errlen;
    int         failed;
    char        names[SUPER_CELLS + 1][SUPER_NAME];
    int         nnames;
} SParse;

static void sfail(SParse *p, const char *fmt, ...)
{
    if (p->failed)
        return;
    p->failed = 1;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(p->err, p->errlen, fmt, ap);
    va_end(ap);
}

static const char *blank(const char *s)
{
    while (isspace((unsigned char)*s))
        s++;
    return s;
}

static int word(const char **s, char *out)
{
    size_t n = 0;
    *s = blank(*s);
    if (!isalpha((unsigned char)**s) && **s != '_')
        return 0;
    while ((isalnum((unsigned char)**s) || **s == '_') && n + 1 < SUPER_NAME)
        out[n++] = *(*s)++;
    out[n] = '\0';
    return 1;
}

static int is_rr(const char *n)
{
    return (n[0] == 'R' || n[0] == 'r') && (n[1] == 'R' || n[1] == 'r') && !n[2];
}

static int cell_index(const SuperSpec *sp, const char *name)
{
    for (int i = 0; i < sp->ncells; i++)
        if (!strcmp(sp->cell[i].name, name))
            return i;
    return -1;
}

static uint64_t ex_ternary(SParse *p, int pass);

/* pass 1 collects the names read; pass 2 evaluates */
static uint64_t ex_atom(SParse *p, int pass)
{
    char name[SUPER_NAME];
    p->s = blank(p->s);
    if (*p->s == '(') {
        p->s++;
        uint64_t v = ex_ternary(p, pass);
        p->s = blank(p->s);
        if (*p->s++ != ')')
            sfail(p, "expected )");
        return v;
    }
    if (*p->s == '0' || *p->s == '1')
        return *p->s++ == '1' ? ~0ull : 0;
    if (*p->s == '!' || *p->s == '~') {
        p->s++;
        return ~ex_atom(p, pass);
    }
    if (!word(&p->s, name)) {
        sfail(p, "expected a name, 0, 1 or ( at \"%.20s\"", p->s);
        return 0;
    }
    if (pass == 1) {
        for (int i = 0; i < p->nnames; i++)
            if (!strcmp(p->names[i], name))
                return 0;
        if (p->nnames == SUPER_CELLS + 1) {
            sfail(p, "too many names");
            return 0;
        }
        snprintf(p->names[p->nnames++], SUPER_NAME, "%s", name);
        return 0;
    }
    if (is_rr(name))
        return sp_var_table(0);
    int c = cell_index(p->sp, name);
    if (c < 0) {
        sfail(p, "unknown name %s", name);
        return 0;
    }
    return p->sp->cell[c].init;
}

static uint64_t ex_and(SParse *p, int pass)
{
    uint64_t v = ex_atom(p, pass);
    for (p->s = blank(p->s); *p->s == '&'; p->s = blank(p->s)) {
        p->s++;
        v &= ex_atom(p, pass);
    }
    return v;
}

static uint64_t ex_xor(SParse *p, int pass)
{
    uint64_t v = ex_and(p, pass);
    for (p->s = blank(p->s); *p->s == '^'; p->s = blank(p->s)) {
        p->s++;
        v ^= ex_and(p, pass);
    }
    return v;
}

static uint64_t ex_or(SParse *p, int pass)
{
    uint64_t v = ex_xor(p, pass);
    for (p->s = blank(p->s); *p->s == '|'; p->s = blank(p->s)) {
        p->s++;
        v |= ex_xor(p, pass);
    }
    return v;
}

static uint64_t ex_ternary(SParse *p, int pass)
{
    uint64_t c = ex_or(p, pass);
    p->s = blank(p->s);
    if (*p->s != '?')
        return c;
    p->s++;
    uint64_t a = ex_ternary(p, pass);
    p->s = blank(p->s);
    if (*p->s++ != ':')
        sfail(p, "expected : in ?:");
    uint64_t b = ex_ternary(p, pass);
    return (c & a) | (~c & b);
}

/* the truth table with variables i and j exchanged */
static uint64_t exchange(uint64_t f, int i, int j, int n)
{
    uint64_t g = 0;
    for (int r = 0; r < (1 << n); r++) {
        int bi = (r >> i) & 1, bj = (r >> j) & 1;
        int q = (r & ~(1 << i) & ~(1 << j)) | bj << i | bi << j;
        if ((f >> r) & 1)
            g |= 1ull << q;
    }
    return g;
}

static void symmetries(SuperSpec *sp, const int *var_of)
{
    for (int i = 0; i < sp->ncells; i++)
        sp->cell[i].sym_prev = -1;
    for (int i = 0; i < sp->ncells; i++) {
        if (!sp->cell[i].in || sp->cell[i].out || var_of[i] < 0)
            continue;
        for (int j = i + 1; j < sp->ncells; j++) {
            if (!sp->cell[j].in || sp->cell[j].out || var_of[j] < 0 || sp->cell[j].sym_prev >= 0)
                continue;
            int vi = var_of[i], vj = var_of[j], same = 1;
            uint64_t m = sp->mask;
            if (sp->rr_out && exchange(sp->rr_target, vi, vj, sp->nvars) != sp->rr_target)
                same = 0;
            for (int c = 0; c < sp->ncells && same; c++) {
                if (sp->cell[c].out && (exchange(sp->cell[c].target, vi, vj, sp->nvars) & m) !=
                                           (sp->cell[c].target & m))
                    same = 0;
                if (sp->cell[c].in && var_of[c] < 0 &&
                    (exchange(sp->cell[c].init, vi, vj, sp->nvars) & m) != (sp->cell[c].init & m))
                    same = 0;
                uint32_t al = sp->cell[c].alias;
                if (((al >> i) & 1) != ((al >> j) & 1))
                    same = 0;
            }
            if (same) {  /* j follows the last member of i's group */
                int last = i;
                for (int k = 0; k < sp->ncells; k++)
                    if (sp->cell[k].sym_prev == last) {
                        last = k;
                        k = -1;
                    }
                sp->cell[j].sym_prev = last;
            }
        }
    }
}

typedef struct {
    char        lhs[SUPER_NAME];
    char        alias[4][SUPER_NAME];
    int         nalias, given;
    const char *rhs;
} Statement;

int cuda_super_parse(const char *text, SuperSpec *sp, char *err, size_t errlen)
{
    SParse p;
    memset(&p, 0, sizeof p);
    memset(sp, 0, sizeof *sp);
    p.sp = sp;
    p.err = err;
    p.errlen = errlen;
    if (errlen)
        err[0] = '\0';
    Statement st[SUPER_CELLS];
    int nst = 0;
    for (const char *s = text; *blank(s) && !p.failed;) {
        if (nst == SUPER_CELLS) {
            sfail(&p, "too many statements");
            break;
        }
        Statement *t = &st[nst++];
        memset(t, 0, sizeof *t);
        if (!word(&s, t->lhs)) {
            sfail(&p, "expected a name at \"%.20s\"", s);
            break;
        }
        s = blank(s);
        if (*s == '{') {
            s++;
            for (;;) {
                if (t->nalias == 4 || !word(&s, t->alias[t->nalias++])) {
                    sfail(&p, "expected names in { }");
                    break;
                }
                s = blank(s);
                if (*s == ',') {
                    s++;
                    continue;
                }
                if (*s++ != '}')
                    sfail(&p, "expected }");
                break;
            }
            s = blank(s);
        }
        if (s[0] == ':' && s[1] == '=') {
            t->given = 1;
            s += 2;
        } else if (*s == '=') {
            s++;
        } else {
            sfail(&p, "expected = after %s", t->lhs);
            break;
        }
        t->rhs = s;
        p.s = s;
        ex_ternary(&p, 1);
        s = blank(p.s);
        if (*s == ';')
            s++;
        else if (*s)
            sfail(&p, "unexpected \"%.20s\"", s);
    }
    if (p.failed)
        return 0;
    int var_of[SUPER_CELLS];
    for (int i = 0; i < SUPER_CELLS; i++)
        var_of[i] = -1;
    for (int i = 0; i < p.nnames; i++)
        if (is_rr(p.names[i]))
            sp->rr_in = 1;
    sp->nvars = sp->rr_in;
    for (int i = 0; i < p.nnames && !p.failed; i++) {
        if (is_rr(p.names[i]))
            continue;
        int given = 0;
        for (int k = 0; k < nst; k++)
            given |= st[k].given && !strcmp(st[k].lhs, p.names[i]);
        if (given)
            continue;
        if (sp->nvars == SUPER_VARS) {
            sfail(&p, "more than %d inputs", SUPER_VARS);
            break;
        }
        int c = sp->ncells++;
        snprintf(sp->cell[c].name, SUPER_NAME, "%s", p.names[i]);
        sp->cell[c].in = 1;
        var_of[c] = sp->nvars;
        sp->cell[c].init = sp_var_table(sp->nvars++);
    }
    sp->mask = sp->nvars == 6 ? ~0ull : (1ull << (1 << sp->nvars)) - 1;
    for (int pass = 0; pass < 2 && !p.failed; pass++)
        for (int k = 0; k < nst && !p.failed; k++) {
            Statement *t = &st[k];
            if (t->given != (pass == 0))
                continue;
            p.s = t->rhs;
            uint64_t v = ex_ternary(&p, 2) & sp->mask;
            if (is_rr(t->lhs)) {
                if (t->given || sp->rr_out || t->nalias)
                    sfail(&p, "RR is set once, with =");
                sp->rr_out = 1;
                sp->rr_target = v;
                continue;
            }
            int c = cell_index(sp, t->lhs);
            if (t->given) {
                if (c >= 0) {
                    sfail(&p, "%s is defined twice", t->lhs);
                    break;
                }
                c = sp->ncells++;
                snprintf(sp->cell[c].name, SUPER_NAME, "%s", t->lhs);
                sp->cell[c].in = 1;
                sp->cell[c].init = v;
                continue;
            }
            if (c >= 0 && sp->cell[c].out) {
                sfail(&p, "%s is set twice", t->lhs);
                break;
            }
            if (c < 0) {
                if (sp->ncells == SUPER_CELLS) {
                    sfail(&p, "too many cells");
                    break;
                }
                c = sp->ncells++;
                snprintf(sp->cell[c].name, SUPER_NAME, "%s", t->lhs);
            }
            if (var_of[c] < 0 && sp->cell[c].in) {
                sfail(&p, "%s is a given cell", t->lhs);
                break;
            }
            sp->cell[c].out = 1;
            sp->cell[c].target = v;
            for (int a = 0; a < t->nalias; a++) {
                int ac = cell_index(sp, t->alias[a]);
                if (ac < 0 || !sp->cell[ac].in || ac == c)
                    sfail(&p, "%s{%s}: %s must be another input", t->lhs, t->alias[a],
                          t->alias[a]);
                else
                    sp->cell[c].alias |= 1u << ac;
            }
        }
    for (int c = 0; c < sp->ncells && !p.failed; c++)
        if (sp->cell[c].out)
            for (int a = 0; a < sp->ncells; a++)
                if (((sp->cell[c].alias >> a) & 1) && sp->cell[a].out)
                    sfail(&p, "%s may share a cell only with inputs that are not written",
                          sp->cell[c].name);
    if (!p.failed && !sp->rr_out) {
        int any = 0;
        for (int c = 0; c < sp->ncells; c++)
            any |= sp->cell[c].out;
        if (!any)
            sfail(&p, "nothing to compute: no RR = ... and no cell = ...");
    }
    if (p.failed)
        return 0;
    symmetries(sp, var_of);
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

/* ---- checking a program (src/super.c:908-1001) ----------------------------------------------- */

static uint64_t garbage(uint64_t *s)
{
    return tc_splitmix64(s);
}

/* Runs p with random garbage in RR (unless it is an input), scratch and output cells, for every
   way outputs may share a cell with their {inputs}; 1 if every output gets its target and every
   other input keeps its value each time. */
int cuda_super_check(const SuperSpec *sp, const SuperProg *p, char *err, size_t errlen)
{
    char names[SUPER_CELLS + SUPER_LEN][SUPER_NAME];
    int ncells = sp->ncells, ref[SUPER_LEN];
    for (int c = 0; c < sp->ncells; c++)
        snprintf(names[c], SUPER_NAME, "%s", sp->cell[c].name);
    for (int i = 0; i < p->len; i++) {
        const char *n = p->code[i].cell;
        if (!strcmp(n, "ZERO") || !strcmp(n, "ONE")) {
            if (p->code[i].op == OP_STO)
                return tc_fail(err, errlen, "instruction %d stores to a constant", i);
            ref[i] = !strcmp(n, "ZERO") ? -1 : -2;
            continue;
        }
        int k = 0;
        while (k < ncells && strcmp(names[k], n))
            k++;
        if (k == ncells)
            snprintf(names[ncells++], SUPER_NAME, "%s", n);
        ref[i] = k;
    }
    int outs[SUPER_CELLS], nout = 0, choice[SUPER_CELLS];
    for (int c = 0; c < sp->ncells; c++)
        if (sp->cell[c].out && !sp->cell[c].in)
            outs[nout++] = c;
    memset(choice, 0, sizeof choice);
    uint64_t seed = 12345;
    for (;;) {
        int home[SUPER_CELLS + SUPER_LEN], clash = 0;
        for (int c = 0; c < ncells; c++)
            home[c] = c;
        for (int i = 0; i < nout; i++) {
            int c = outs[i], k = 0;
            if (choice[i])
                for (int a = 0; a < sp->ncells; a++)
                    if (((sp->cell[c].alias >> a) & 1) && ++k == choice[i])
                        home[c] = a;
        }
        for (int i = 0; i < nout; i++)
            for (int j = i + 1; j < nout; j++)
                clash |= home[outs[i]] == home[outs[j]];
        for (int trial = 0; trial < 16 && !clash; trial++) {
            uint64_t val[SUPER_CELLS + SUPER_LEN], rr;
            for (int c = 0; c < ncells; c++)
                val[c] = garbage(&seed) & sp->mask;
            for (int c = 0; c < sp->ncells; c++)
                if (sp->cell[c].in)
                    val[c] = sp->cell[c].init;
            rr = sp->rr_in ? sp_var_table(0) & sp->mask : garbage(&seed) & sp->mask;
            for (int i = 0; i < p->len; i++) {
                int c = ref[i] >= 0 ? home[ref[i]] : ref[i];
                if (p->code[i].op == OP_NAND)
                    rr = ~(rr & (c == -1 ? 0 : c == -2 ? sp->mask : val[c])) & sp->mask;
                else
                    val[c] = rr;
            }
            for (int c = 0; c < sp->ncells; c++) {
                uint64_t want = sp->cell[c].out ? sp->cell[c].target : sp->cell[c].init;
                int shared = 0;
                for (int i = 0; i < nout; i++)
                    shared |= home[outs[i]] == c && outs[i] != c;
                if (!shared && val[home[c]] != want)
                    return tc_fail(err, errlen, "%s %s (cells shared: variant %d)",
                                   sp->cell[c].name,
                                   sp->cell[c].out ? "does not get its value" : "is not kept",
                                   choice[0]);
            }
            if (sp->rr_out && rr != sp->rr_target)
                return tc_fail(err, errlen, "RR does not end with its value");
        }
        int i = 0;
        for (; i < nout; i++) {
            int n = 0;
            for (int a = 0; a < sp->ncells; a++)
                n += (sp->cell[outs[i]].alias >> a) & 1;
            if (++choice[i] <= n)
                break;
            choice[i] = 0;
        }
        if (i == nout)
            break;
    }
    return 1;
}
