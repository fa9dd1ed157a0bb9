/* Specifications for verify and search: "c:s = a + b + c".  The grammar, the error messages and
   the parsed form are the reference's (src/spec.h, src/spec.c:42-377): the left side joins output
   vectors, the first one highest; the right side is a 64-bit integer expression over input
   vectors, kept as reverse Polish notation; input k of n is bit n-1-k of the assignment x.

   The parsed form (TcSpec) has the reference's memory layout, so either parser's result can be
   handed to the engine.  On the device the expression is not interpreted: the code generator
   turns the RPN into straight-line CUDA (codegen.c). */
#include <ctype.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include "tc_host.h"

typedef struct {
    const char    *s;
    const Program *p;
    TcSpec        *spec;
    int            inputs_allowed;
    char          *err;
    size_t         errlen;
    int            failed;
} Parse;

static int prefix_nocase(const char *a, const char *b, size_t n)
{
    for (size_t i = 0; i < n; i++)
        if (tolower((unsigned char)a[i]) != tolower((unsigned char)b[i]))
            return 0;
    return 1;
}

/* Vector `name` among cells list[0..n): a cell called exactly `name` (width 1), or the cells
   name0, name1, ... (idx[i] = position of bit i).  Returns the width, 0 if absent, -1 for gaps or
   more than 64 bits.  src/spec.h:31-33. */
int tc_vec_resolve(const Program *p, const uint32_t *list, size_t n, const char *name, int *idx)
{
    size_t len = strlen(name);
    for (size_t i = 0; i < n; i++) {
        const char *c = p->cell_names[list[i]];
        if (strlen(c) == len && prefix_nocase(c, name, len)) {
            idx[0] = (int)i;
            return 1;
        }
    }
    int width = 0;
    uint64_t seen = 0;
    for (size_t i = 0; i < n; i++) {
        const char *c = p->cell_names[list[i]];
        if (strlen(c) <= len || !prefix_nocase(c, name, len))
            continue;
        const char *d = c + len;
        if (!isdigit((unsigned char)d[0]) || (d[0] == '0' && d[1]))
            continue;
        char *end;
        unsigned long bit = strtoul(d, &end, 10);
        if (*end)
            continue;
        if (bit >= 64)
            return -1;
        idx[bit] = (int)i;
        seen |= 1ull << bit;
        if ((int)bit + 1 > width)
            width = (int)bit + 1;
    }
    if (width && seen != (width == 64 ? ~0ull : (1ull << width) - 1))
        return -1;
    return width;
}

static void fail(Parse *ps, const char *fmt, ...)
{
    if (ps->failed)
        return;
    ps->failed = 1;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(ps->err, ps->errlen, fmt, ap);
    va_end(ap);
}

static void blanks(Parse *ps)
{
    while (*ps->s == ' ' || *ps->s == '\t')
        ps->s++;
}

static void emit(Parse *ps, int op, uint64_t v)
{
    TcSpec *s = ps->spec;
    if (s->nrpn == TS_MAX_RPN) {
        fail(ps, "the expression is too long");
        return;
    }
    s->rpn[s->nrpn].op = op;
    s->rpn[s->nrpn++].v = v;
    if (op == TS_NUM || op == TS_VAR)
        s->depth++;
    else if (op != TS_NOT && op != TS_NEG)
        s->depth--;
    if (s->depth > s->max_depth)
        s->max_depth = s->depth;
    if (s->max_depth > TS_MAX_STACK)
        fail(ps, "the expression is nested too deeply");
}

static int word(Parse *ps, char *buf, size_t len)
{
    size_t n = 0;
    if (!isalpha((unsigned char)*ps->s) && *ps->s != '_')
        return 0;
    while (isalnum((unsigned char)*ps->s) || *ps->s == '_') {
        if (n + 1 < len)
            buf[n++] = *ps->s;
        ps->s++;
    }
    buf[n] = '\0';
    return 1;
}

static int input_vector(Parse *ps, const char *name)
{
    TcSpec *s = ps->spec;
    size_t len = strlen(name);
    for (int k = 0; k < s->nvars; k++)
        if (strlen(s->var_name[k]) == len && prefix_nocase(s->var_name[k], name, len))
            return k;
    if (!ps->inputs_allowed) {
        fail(ps, "'%s': the right side must be a number here", name);
        return -1;
    }
    if (s->nvars == TS_MAX_VARS) {
        fail(ps, "too many input vectors");
        return -1;
    }
    int idx[64], w = tc_vec_resolve(ps->p, ps->p->inputs, ps->p->ninputs, name, idx);
    if (w <= 0) {
        fail(ps, w < 0 ? "input vector %s has missing bits or more than 64" : "no input called %s",
             name);
        return -1;
    }
    int k = s->nvars++;
    snprintf(s->var_name[k], sizeof s->var_name[k], "%s", name);
    s->var_bits[k] = w;
    for (int b = 0; b < w; b++)
        s->var_pos[k][b] = (int)ps->p->ninputs - 1 - idx[b];
    return k;
}

static void expression(Parse *ps, int min_prec);

static void operand(Parse *ps)
{
    blanks(ps);
    char name[64];
    if (*ps->s == '(') {
        ps->s++;
        expression(ps, 0);
        blanks(ps);
        if (*ps->s != ')')
            fail(ps, "expected )");
        else
            ps->s++;
    } else if (isdigit((unsigned char)*ps->s)) {
        char *end;
        unsigned long long v = strtoull(ps->s, &end, 0);
        ps->s = end;
        emit(ps, TS_NUM, v);
    } else if (word(ps, name, sizeof name)) {
        int k = input_vector(ps, name);
        if (k >= 0)
            emit(ps, TS_VAR, (uint64_t)k);
    } else {
        fail(ps, *ps->s ? "unexpected '%c'" : "the expression ends too early", *ps->s);
    }
}

static void prefix(Parse *ps)
{
    blanks(ps);
    if (*ps->s == '~' || *ps->s == '-') {
        int op = *ps->s == '~' ? TS_NOT : TS_NEG;
        ps->s++;
        prefix(ps);
        emit(ps, op, 0);
    } else {
        operand(ps);
    }
}

/* The binary operator at s, its precedence (higher binds tighter) and its length. */
static int infix(const char *s, int *prec, int *len)
{
    *len = 1;
    switch (*s) {
    case '|': *prec = 1; return TS_OR;
    case '^': *prec = 2; return TS_XOR;
    case '&': *prec = 3; return TS_AND;
    case '<': *len = 2; *prec = 4; return s[1] == '<' ? TS_SHL : 0;
    case '>': *len = 2; *prec = 4; return s[1] == '>' ? TS_SHR : 0;
    case '+': *prec = 5; return TS_ADD;
    case '-': *prec = 5; return TS_SUB;
    case '*': *prec = 6; return TS_MUL;
    default:  return 0;
    }
}

static void expression(Parse *ps, int min_prec)
{
    prefix(ps);
    while (!ps->failed) {
        blanks(ps);
        int prec, len, op = infix(ps->s, &prec, &len);
        if (!op || prec < min_prec)
            break;
        ps->s += len;
        expression(ps, prec + 1);
        emit(ps, op, 0);
    }
}

Spec *cuda_spec_parse(const char *text, const Program *p, int inputs_allowed, char *err,
                      size_t errlen)
{
    TcSpec *s = calloc(1, sizeof *s);
    if (!s) {
        snprintf(err, errlen, "out of memory");
        return NULL;
    }
    Parse ps = {text, p, s, inputs_allowed, err, errlen, 0};
    int outs[64][64], widths[64], nout = 0, total = 0;
    for (;;) {
        char name[64];
        blanks(&ps);
        if (!word(&ps, name, sizeof name)) {
            fail(&ps, "expected an output name before =");
            break;
        }
        int w = tc_vec_resolve(p, p->outputs, p->noutputs, name, outs[nout]);
        if (w <= 0) {
            fail(&ps, w < 0 ? "output vector %s has missing bits or more than 64"
                            : "no output called %s", name);
            break;
        }
        widths[nout++] = w;
        total += w;
        blanks(&ps);
        if (*ps.s != ':' || nout == 64)
            break;
        ps.s++;
    }
    if (!ps.failed && total > 64)
        fail(&ps, "the left side has %d bits, at most 64 work", total);
    if (!ps.failed) {
        for (int k = nout - 1; k >= 0; k--)
            for (int b = 0; b < widths[k]; b++)
                s->out[s->width++] = p->outputs[outs[k][b]];
        blanks(&ps);
        if (*ps.s != '=')
            fail(&ps, "expected = after the outputs");
        else
            ps.s++;
    }
    if (!ps.failed)
        expression(&ps, 0);
    if (!ps.failed) {
        blanks(&ps);
        if (*ps.s)
            fail(&ps, "unexpected '%c'", *ps.s);
    }
    if (ps.failed) {
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

/* The right side for assignment x, on the host (for reports; the device has its own code). */
uint64_t cuda_spec_value(const Spec *spec, uint64_t x)
{
    const TcSpec *s = (const TcSpec *)spec;
    uint64_t var[TS_MAX_VARS], st[TS_MAX_STACK + 1];
    for (int k = 0; k < s->nvars; k++) {
        uint64_t v = 0;
        for (int b = 0; b < s->var_bits[k]; b++)
            v |= ((x >> s->var_pos[k][b]) & 1) << b;
        var[k] = v;
    }
    int sp = 0;
    for (int i = 0; i < s->nrpn; i++) {
        const TcSpecItem *it = &s->rpn[i];
        if (it->op == TS_NUM) {
            st[sp++] = it->v;
        } else if (it->op == TS_VAR) {
            st[sp++] = var[it->v];
        } else if (it->op == TS_NOT) {
            st[sp - 1] = ~st[sp - 1];
        } else if (it->op == TS_NEG) {
            st[sp - 1] = 0 - st[sp - 1];
        } else {
            uint64_t b = st[--sp], *a = &st[sp - 1];
            switch (it->op) {
            case TS_ADD: *a += b; break;
            case TS_SUB: *a -= b; break;
            case TS_MUL: *a *= b; break;
            case TS_AND: *a &= b; break;
            case TS_OR:  *a |= b; break;
            case TS_XOR: *a ^= b; break;
            case TS_SHL: *a = b < 64 ? *a << b : 0; break;
            case TS_SHR: *a = b < 64 ? *a >> b : 0; break;
            }
        }
    }
    return s->width == 64 ? st[0] : st[0] & ((1ull << s->width) - 1);
}
