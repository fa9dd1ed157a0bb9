/* Specifications for verify and search: "c:s = a + b + c".

   The language, its error messages and the parsed form are the reference's interface
   (src/spec.h:1-11): the left side joins output vectors, the first one giving the highest bits;
   the right side is a 64-bit wrapping integer expression over input vectors and numbers with
   ~ - (prefix), * (tightest), + -, << >>, &, ^, | (loosest), all binary operators left
   associative, and parentheses; input k of n is bit n-1-k of the assignment x.  The parsed form
   (TcSpec) has the memory layout of the reference's private struct (src/spec.c:20-29), RPN
   included, so a Spec from either parser can be handed to the engine or to the other's
   evaluator.

   The parser here is an operator-precedence translator: one left-to-right scan of the text that
   alternates between wanting an operand and wanting an operator, with an explicit stack of
   pending operators and open parentheses, and a table of the binary operators.  An operator
   leaves the stack for the RPN when one of no higher precedence arrives or its group closes, so
   the RPN (and the stack depth it needs) is the one a recursive-descent reading of the grammar
   gives, and the first error met in the scan is the one reported.

   On the device the expression is not interpreted: the code generator turns the RPN into
   straight-line CUDA (codegen.c). */
#include <ctype.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include "tc_host.h"

/* ---- vectors of cells ------------------------------------------------------------------------ */

/* The bit index spelled by the digits after a vector's base name: -1 when the rest is not a plain
   decimal index (empty, a non-digit, or a leading zero before more digits), 64 for any index of
   64 or more. */
static int bit_index(const char *d)
{
    if (!*d || (d[0] == '0' && d[1]))
        return -1;
    int v = 0;
    for (; *d; d++) {
        if (*d < '0' || *d > '9')
            return -1;
        if (v < 64)
            v = v * 10 + (*d - '0');
    }
    return v < 64 ? v : 64;
}

/* Vector `name` among cells list[0..n): a cell called exactly `name` (case ignored) is a vector
   of width 1 and wins; otherwise the cells name0, name1, ... are its bits (idx[b] = position in
   list of bit b).  Returns the width, 0 when there is no such vector, -1 when its bits have a gap
   or one of them is 64 or more.  The interface of vec_resolve, src/spec.h:31-33. */
int tc_vec_resolve(const Program *p, const uint32_t *list, size_t n, const char *name, int *idx)
{
    for (size_t i = 0; i < n; i++)
        if (tc_same_name(p->cell_names[list[i]], name)) {
            idx[0] = (int)i;
            return 1;
        }
    size_t base = strlen(name);
    uint64_t bits = 0;
    int top = -1;
    for (size_t i = 0; i < n; i++) {
        const char *c = p->cell_names[list[i]];
        if (strncasecmp(c, name, base) != 0)
            continue;
        int b = bit_index(c + base);
        if (b < 0)
            continue;
        if (b == 64)
            return -1;
        idx[b] = (int)i;
        bits |= 1ull << b;
        top = b > top ? b : top;
    }
    if (top < 0)
        return 0;
    uint64_t all = top == 63 ? ~0ull : (1ull << (top + 1)) - 1;
    return bits == all ? top + 1 : -1;
}

/* "a=0x1f b=0x3 c=1": cells list[0..n) with values val[], in list order, the bits of a vector
   of two or more (cells base0, base1, ...) printed once as one hexadecimal number under its base
   name where its first bit appears; other cells one by one.  The interface of vec_format,
   src/spec.h:35-37.  Output stops at len - 1 characters. */
void tc_vec_format(const Program *p, const uint32_t *list, size_t n, const uint8_t *val,
                   char *buf, size_t len)
{
    size_t at = 0;
    if (!len)
        return;
    buf[0] = '\0';
    uint8_t *printed = tc_xcalloc(n + 1, 1);
    for (size_t i = 0; i < n && at < len; i++) {
        if (printed[i])
            continue;
        const char *c = p->cell_names[list[i]];
        size_t full = strlen(c), base = full;
        while (base && isdigit((unsigned char)c[base - 1]))
            base--;
        char stem[64];
        int idx[64], w = 0;
        if (base && base < full && base < sizeof stem) {
            memcpy(stem, c, base);
            stem[base] = '\0';
            w = tc_vec_resolve(p, list, n, stem, idx);
        }
        const char *sep = at ? " " : "";
        int wrote;
        if (w >= 2) {
            unsigned long long v = 0;
            for (int b = w - 1; b >= 0; b--) {
                v = v << 1 | (val[idx[b]] & 1u);
                printed[idx[b]] = 1;
            }
            wrote = snprintf(buf + at, len - at, "%s%s=0x%llx", sep, stem, v);
        } else {
            printed[i] = 1;
            wrote = snprintf(buf + at, len - at, "%s%s=%u", sep, c, (unsigned)val[i]);
        }
        at += wrote > 0 ? (size_t)wrote : 0;
    }
    free(printed);
}

/* ---- the parser ------------------------------------------------------------------------------ */

/* Binary operators: spelling, RPN item, precedence (higher binds tighter). */
static const struct {
    char    c0, c1;
    uint8_t op, prec;
} INFIX[] = {
    {'*', 0, TS_MUL, 6},   {'+', 0, TS_ADD, 5}, {'-', 0, TS_SUB, 5}, {'<', '<', TS_SHL, 4},
    {'>', '>', TS_SHR, 4}, {'&', 0, TS_AND, 3}, {'^', 0, TS_XOR, 2}, {'|', 0, TS_OR, 1},
};
#define PREFIX_PREC 7   /* ~ and - in front of an operand bind tighter than every operator */
#define OPEN_PAREN  -1  /* a pending '(' on the operator stack */

typedef struct {
    int op, prec;
} Pending;

typedef struct {
    const char    *at;
    const Program *p;
    TcSpec        *s;
    int            inputs_allowed;
    char          *err;
    size_t         errlen;
    int            bad;
    Pending       *ops;
    int            nops, capops;
} Parser;

static void fail(Parser *ps, const char *fmt, ...)
{
    if (ps->bad++)
        return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(ps->err, ps->errlen, fmt, ap);
    va_end(ap);
}

static void skip_blanks(Parser *ps)
{
    ps->at += strspn(ps->at, " \t");
}

/* The binary operator spelled at s: its INFIX entry, or -1. */
static int infix_at(const char *s)
{
    for (int i = 0; i < (int)(sizeof INFIX / sizeof INFIX[0]); i++)
        if (s[0] == INFIX[i].c0 && (!INFIX[i].c1 || s[1] == INFIX[i].c1))
            return i;
    return -1;
}

/* Appends one RPN item.  The evaluation stack's depth moves by +1 for an operand, 0 for a prefix
   operator, -1 for a binary one; more than TS_MAX_RPN items or a depth beyond TS_MAX_STACK is an
   error at the item that causes it. */
static void emit(Parser *ps, int op, uint64_t v)
{
    TcSpec *s = ps->s;
    if (s->nrpn >= TS_MAX_RPN) {
        fail(ps, "the expression is too long");
        return;
    }
    s->rpn[s->nrpn].op = op;
    s->rpn[s->nrpn].v = v;
    s->nrpn++;
    s->depth += op == TS_NUM || op == TS_VAR ? 1 : op == TS_NOT || op == TS_NEG ? 0 : -1;
    if (s->depth > s->max_depth)
        s->max_depth = s->depth;
    if (s->max_depth > TS_MAX_STACK)
        fail(ps, "the expression is nested too deeply");
}

static void push_op(Parser *ps, int op, int prec)
{
    if (ps->nops == ps->capops) {
        ps->capops = ps->capops ? 2 * ps->capops : 32;
        ps->ops = tc_xrealloc(ps->ops, (size_t)ps->capops * sizeof *ps->ops);
    }
    ps->ops[ps->nops].op = op;
    ps->ops[ps->nops].prec = prec;
    ps->nops++;
}

/* Moves pending operators of precedence >= prec to the RPN, down to the innermost open '('. */
static void release(Parser *ps, int prec)
{
    while (!ps->bad && ps->nops && ps->ops[ps->nops - 1].op != OPEN_PAREN &&
           ps->ops[ps->nops - 1].prec >= prec) {
        ps->nops--;
        emit(ps, ps->ops[ps->nops].op, 0);
    }
}

/* Reads an identifier ([A-Za-z_][A-Za-z0-9_]*) into buf, cut to len - 1 characters; 0 if none. */
static int identifier(Parser *ps, char *buf, size_t len)
{
    const char *b = ps->at;
    if (!isalpha((unsigned char)*b) && *b != '_')
        return 0;
    const char *e = b;
    while (isalnum((unsigned char)*e) || *e == '_')
        e++;
    size_t n = (size_t)(e - b) < len - 1 ? (size_t)(e - b) : len - 1;
    memcpy(buf, b, n);
    buf[n] = '\0';
    ps->at = e;
    return 1;
}

/* The variable number of input vector `name`, adding it on first use; -1 after an error. */
static int variable(Parser *ps, const char *name)
{
    TcSpec *s = ps->s;
    for (int k = 0; k < s->nvars; k++)
        if (tc_same_name(s->var_name[k], name))
            return k;
    if (!ps->inputs_allowed) {
        fail(ps, "'%s': the right side must be a number here", name);
        return -1;
    }
    if (s->nvars == TS_MAX_VARS) {
        fail(ps, "too many input vectors");
        return -1;
    }
    int idx[64];
    int w = tc_vec_resolve(ps->p, ps->p->inputs, ps->p->ninputs, name, idx);
    if (w == 0)
        fail(ps, "no input called %s", name);
    if (w < 0)
        fail(ps, "input vector %s has missing bits or more than 64", name);
    if (w <= 0)
        return -1;
    int k = s->nvars++;
    snprintf(s->var_name[k], sizeof s->var_name[k], "%s", name);
    s->var_bits[k] = w;
    for (int b = 0; b < w; b++)   /* input k of n is bit n-1-k of x */
        s->var_pos[k][b] = (int)ps->p->ninputs - 1 - idx[b];
    return k;
}

/* A number or an input vector at the scan position; 0 after an error. */
static int operand(Parser *ps)
{
    char c = *ps->at, name[64];
    if (isdigit((unsigned char)c)) {
        char *end;
        uint64_t v = strtoull(ps->at, &end, 0);  /* decimal, 0x hexadecimal or 0 octal */
        ps->at = end;
        emit(ps, TS_NUM, v);
    } else if (identifier(ps, name, sizeof name)) {
        int k = variable(ps, name);
        if (k >= 0)
            emit(ps, TS_VAR, (uint64_t)k);
    } else if (c) {
        fail(ps, "unexpected '%c'", c);
    } else {
        fail(ps, "the expression ends too early");
    }
    return !ps->bad;
}

/* The right side, up to the first character that cannot continue it. */
static void expression(Parser *ps)
{
    int want_operand = 1;
    while (!ps->bad) {
        skip_blanks(ps);
        if (want_operand) {
            char c = *ps->at;
            if (c == '~' || c == '-' || c == '(') {
                push_op(ps, c == '(' ? OPEN_PAREN : c == '~' ? TS_NOT : TS_NEG, PREFIX_PREC);
                ps->at++;
            } else if (operand(ps)) {
                want_operand = 0;
            }
            continue;
        }
        /* an operand is complete: the prefix operators written just before it apply first */
        while (!ps->bad && ps->nops && ps->ops[ps->nops - 1].op != OPEN_PAREN &&
               ps->ops[ps->nops - 1].prec == PREFIX_PREC)
            emit(ps, ps->ops[--ps->nops].op, 0);
        int i = infix_at(ps->at);
        if (i >= 0) {
            release(ps, INFIX[i].prec);  /* left associative: equal precedence goes first */
            push_op(ps, INFIX[i].op, INFIX[i].prec);
            ps->at += INFIX[i].c1 ? 2 : 1;
            want_operand = 1;
            continue;
        }
        release(ps, 0);  /* the innermost group (or the whole side) ends here */
        if (ps->bad || !ps->nops)
            return;
        if (*ps->at != ')') {
            fail(ps, "expected )");
            return;
        }
        ps->nops--;  /* the '(' */
        ps->at++;
    }
}

/* The left side: output vectors joined by ':' (at most 64 of them), the first one giving the
   highest bits of the result. */
static void outputs(Parser *ps)
{
    const Program *p = ps->p;
    int bits[64][64], width[64], nvec = 0, total = 0;
    do {
        char name[64];
        skip_blanks(ps);
        if (!identifier(ps, name, sizeof name)) {
            fail(ps, "expected an output name before =");
            return;
        }
        int w = tc_vec_resolve(p, p->outputs, p->noutputs, name, bits[nvec]);
        if (w <= 0) {
            fail(ps, w ? "output vector %s has missing bits or more than 64"
                       : "no output called %s", name);
            return;
        }
        width[nvec++] = w;
        total += w;
        skip_blanks(ps);
    } while (nvec < 64 && *ps->at == ':' && ps->at++);
    if (total > 64) {
        fail(ps, "the left side has %d bits, at most 64 work", total);
        return;
    }
    TcSpec *s = ps->s;
    for (int k = nvec - 1; k >= 0; k--)   /* the last vector is the lowest */
        for (int b = 0; b < width[k]; b++)
            s->out[s->width++] = p->outputs[bits[k][b]];
}

Spec *cuda_spec_parse(const char *text, const Program *p, int inputs_allowed, char *err,
                      size_t errlen)
{
    TcSpec *s = calloc(1, sizeof *s);
    if (!s) {
        snprintf(err, errlen, "out of memory");
        return NULL;
    }
    Parser ps;
    memset(&ps, 0, sizeof ps);
    ps.at = text;
    ps.p = p;
    ps.s = s;
    ps.inputs_allowed = inputs_allowed;
    ps.err = err;
    ps.errlen = errlen;
    outputs(&ps);
    if (!ps.bad) {
        skip_blanks(&ps);
        if (*ps.at == '=')
            ps.at++;
        else
            fail(&ps, "expected = after the outputs");
    }
    if (!ps.bad)
        expression(&ps);
    if (!ps.bad) {
        skip_blanks(&ps);
        if (*ps.at)
            fail(&ps, "unexpected '%c'", *ps.at);
    }
    free(ps.ops);
    if (ps.bad) {
        free(s);
        return NULL;
    }
    return (Spec *)s;
}

void cuda_spec_free(Spec *s)
{
    free(s);
}

int cuda_spec_width(const Spec *s)
{
    return ((const TcSpec *)s)->width;
}

uint32_t cuda_spec_out_cell(const Spec *s, int bit)
{
    return ((const TcSpec *)s)->out[bit];
}

/* ---- evaluation on the host (reports and the CLI; the device has generated code) ------------- */

static uint64_t binary(int op, uint64_t l, uint64_t r)
{
    if (op == TS_ADD) return l + r;
    if (op == TS_SUB) return l - r;
    if (op == TS_MUL) return l * r;
    if (op == TS_AND) return l & r;
    if (op == TS_OR)  return l | r;
    if (op == TS_XOR) return l ^ r;
    if (op == TS_SHL) return r < 64 ? l << r : 0;  /* shifts of 64 or more give 0 */
    return r < 64 ? l >> r : 0;                    /* TS_SHR */
}

/* The right side for assignment x, cut to the left side's width. */
uint64_t cuda_spec_value(const Spec *spec, uint64_t x)
{
    const TcSpec *s = (const TcSpec *)spec;
    uint64_t var[TS_MAX_VARS], st[TS_MAX_STACK + 1];
    for (int k = 0; k < s->nvars; k++) {
        var[k] = 0;
        for (int b = s->var_bits[k] - 1; b >= 0; b--)
            var[k] = var[k] << 1 | (x >> s->var_pos[k][b] & 1);
    }
    int n = 0;
    for (const TcSpecItem *it = s->rpn; it < s->rpn + s->nrpn; it++) {
        switch (it->op) {
        case TS_NUM: st[n++] = it->v; break;
        case TS_VAR: st[n++] = var[it->v]; break;
        case TS_NOT: st[n - 1] = ~st[n - 1]; break;
        case TS_NEG: st[n - 1] = 0 - st[n - 1]; break;
        default:     n--; st[n - 1] = binary(it->op, st[n - 1], st[n]); break;
        }
    }
    uint64_t mask = s->width >= 64 ? ~0ull : (1ull << s->width) - 1;
    return st[0] & mask;
}
