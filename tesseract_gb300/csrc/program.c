/* Program utilities: freeing, cell lookup, read-only cells, link resolution, the cube's
   dimensions, and printing as assembly.  Semantics follow src/isa.h:48-62 and src/asm.c:767-801;
   the printed form follows src/build.c:417-444 so that it assembles back into the same program. */
#include <ctype.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include "tc_host.h"

void *tc_xmalloc(size_t n)
{
    void *p = malloc(n ? n : 1);
    if (!p) {
        fputs("out of memory\n", stderr);
        exit(1);
    }
    return p;
}

void *tc_xcalloc(size_t n, size_t k)
{
    void *p = calloc(n ? n : 1, k ? k : 1);
    if (!p) {
        fputs("out of memory\n", stderr);
        exit(1);
    }
    return p;
}

void *tc_xrealloc(void *p, size_t n)
{
    void *q = realloc(p, n ? n : 1);
    if (!q) {
        fputs("out of memory\n", stderr);
        exit(1);
    }
    return q;
}

char *tc_xstrdup(const char *s)
{
    size_t n = strlen(s) + 1;
    return memcpy(tc_xmalloc(n), s, n);
}

int tc_same_name(const char *a, const char *b)
{
    return strcasecmp(a, b) == 0;
}

uint64_t tc_splitmix64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void tc_program_free(Program *p)
{
    if (!p)
        return;
    for (uint32_t i = 0; p->cell_names && i < p->ncells; i++)
        free(p->cell_names[i]);
    free(p->cell_names);
    free(p->code);
    free(p->inputs);
    free(p->outputs);
    free(p->special);
    memset(p, 0, sizeof *p);
}

int tc_program_find_cell(const Program *p, const char *name, uint32_t *addr)
{
    for (uint32_t i = 0; i < p->ncells; i++)
        if (tc_same_name(p->cell_names[i], name)) {
            *addr = i;
            return 1;
        }
    return 0;
}

int tc_program_readonly(const Program *p, uint32_t cell)
{
    return cell < CELL_FIRST_FREE || (p->special && p->special[cell].kind != CK_PLAIN);
}

uint32_t tc_program_resolve(const Program *p, uint32_t cell, unsigned *mask)
{
    unsigned m = 0;
    while (p->special && p->special[cell].kind == CK_LINK) {
        m ^= 1u << p->special[cell].dim;
        cell = p->special[cell].src;
    }
    *mask = m;
    return cell;
}

unsigned tc_program_dims(const Program *p)
{
    unsigned dims = CUBE_DIMS;
    if (!p->special)
        return dims;
    for (uint32_t c = 0; c < p->ncells; c++)
        if (p->special[c].kind != CK_PLAIN && p->special[c].dim + 1u > dims)
            dims = p->special[c].dim + 1u;
    return dims;
}

int tc_program_id_name(const char *name)
{
    if (tolower((unsigned char)name[0]) != 'i' || tolower((unsigned char)name[1]) != 'd')
        return -1;
    const char *d = name + 2;
    if (!isdigit((unsigned char)d[0]) || (d[0] == '0' && d[1]))
        return -1;
    int v = d[0] - '0';
    if (d[1]) {
        if (!isdigit((unsigned char)d[1]) || d[2])
            return -1;
        v = 10 * v + (d[1] - '0');
    }
    return v < CUBE_MAX_DIMS ? v : -1;
}

int tc_program_copy(const Program *s, Program *d)
{
    memset(d, 0, sizeof *d);
    d->len = s->len;
    d->ncells = s->ncells;
    d->ninputs = s->ninputs;
    d->noutputs = s->noutputs;
    d->code = tc_xmalloc(s->len * sizeof *d->code);
    memcpy(d->code, s->code, s->len * sizeof *d->code);
    d->cell_names = tc_xmalloc(s->ncells * sizeof *d->cell_names);
    for (uint32_t i = 0; i < s->ncells; i++)
        d->cell_names[i] = tc_xstrdup(s->cell_names[i]);
    d->inputs = tc_xmalloc(s->ninputs * sizeof *d->inputs);
    memcpy(d->inputs, s->inputs, s->ninputs * sizeof *d->inputs);
    d->outputs = tc_xmalloc(s->noutputs * sizeof *d->outputs);
    memcpy(d->outputs, s->outputs, s->noutputs * sizeof *d->outputs);
    if (s->special) {
        d->special = tc_xmalloc(s->ncells * sizeof *d->special);
        memcpy(d->special, s->special, s->ncells * sizeof *d->special);
    }
    return 1;
}

/* ---- printing ------------------------------------------------------------------------------ */

typedef struct {
    char  *buf;
    size_t len, at;
} Out;

static void put(Out *o, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    size_t room = o->at < o->len ? o->len - o->at : 0;
    int k = vsnprintf(o->buf ? o->buf + o->at : NULL, room, fmt, ap);
    va_end(ap);
    if (k > 0)
        o->at += (size_t)k;
}

static void put_list(Out *o, const char *directive, const Program *p, const uint32_t *cells,
                     size_t n)
{
    for (size_t i = 0; i < n; i++) {
        if (i % 16 == 0)
            put(o, "%s%s", i ? "\n" : "", directive);
        else
            put(o, " ");
        put(o, "%s", p->cell_names[cells[i]]);
    }
    if (n)
        put(o, "\n");
}

size_t tc_program_print(const Program *p, char *buf, size_t len)
{
    Out o = {buf, len, 0};
    put_list(&o, ".in  ", p, p->inputs, p->ninputs);
    put_list(&o, ".out ", p, p->outputs, p->noutputs);
    for (uint32_t c = 0; p->special && c < p->ncells; c++)
        if (p->special[c].kind == CK_LINK)
            put(&o, ".link %s = %s @ %u\n", p->cell_names[c], p->cell_names[p->special[c].src],
                (unsigned)p->special[c].dim);
    put(&o, "\n");
    for (size_t i = 0; i < p->len; i++)
        put(&o, "    %-4s %s\n", p->code[i].op == OP_NAND ? "NAND" : "STO",
            p->cell_names[p->code[i].addr]);
    return o.at;
}

char *tc_program_text(const Program *p, size_t *len)
{
    size_t n = tc_program_print(p, NULL, 0);
    char *b = tc_xmalloc(n + 1);
    tc_program_print(p, b, n + 1);
    if (len)
        *len = n;
    return b;
}
