/* The assembler: source text to Program.  The language is the reference's (docs/ISA.md,
   "Assembly language"): .in/.out/.link/.include/.macro directives, NAND and STO, macros with
   parameters, '#' name joining and @locals.  Cells are numbered in order of first appearance and
   macro locals are named "@<call>:<name>", exactly as src/asm.c does, so both assemblers give the
   same Program for the same text.  Cell lookup is a hash table here (the programs that matter on
   the GPU have hundreds of thousands of instructions). */
#include <ctype.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include "tc_host.h"

enum { NEST_LIMIT = 64, TOKEN_LIMIT = 128 };

typedef struct {
    char  *name;
    char **params;
    int    nparams;
    char **lines;
    int   *line_no;
    int    nlines;
    char  *file, *dir;
} Macro;

typedef struct {
    /* the program being built */
    Instr    *code;
    size_t    len, cap;
    char    **names;
    CellInfo *info;
    uint32_t  ncells, capcells;
    uint32_t *slots;  /* open addressing: cell + 1, 0 = empty */
    size_t    nslots;
    uint32_t *in, *out;
    size_t    nin, capin, nout, capout;
    int       special;
    Macro    *macros;
    int       nmacros, capmacros;
    unsigned  calls;  /* macro calls so far: numbers the @locals */
    char     *err;
    size_t    errlen;
    int       failed;
} Asm;

typedef struct {
    const char *file, *dir;
    const char *from;  /* "file:line" of the outermost macro call, or NULL */
    int         depth;
    int         in_macro;
} Where;

typedef struct {
    char *copy;
    char *t[TOKEN_LIMIT];
    int   n;
} Toks;

static void assemble_lines(Asm *a, const Where *w, char **lines, const int *nos, int n);

static void error(Asm *a, const Where *w, int line, const char *fmt, ...)
{
    if (a->failed)
        return;
    a->failed = 1;
    if (!a->errlen)
        return;
    size_t at = 0;
    int k = snprintf(a->err, a->errlen, "%s:%d: ", w->file, line);
    at = k > 0 ? (size_t)k : 0;
    if (at < a->errlen) {
        va_list ap;
        va_start(ap, fmt);
        k = vsnprintf(a->err + at, a->errlen - at, fmt, ap);
        va_end(ap);
        if (k > 0)
            at += (size_t)k;
    }
    if (w->from && at < a->errlen)
        snprintf(a->err + at, a->errlen - at, " (in macro called at %s)", w->from);
}

/* ---- tokens ------------------------------------------------------------------------------- */

static int is_sep(char c)
{
    return c == ' ' || c == '\t' || c == ',' || c == '\r';
}

/* Splits a line: separators are blanks and commas, ';' starts a comment, "..." is one token.
   Returns NULL or an error message. */
static const char *split(const char *line, Toks *t)
{
    char *p = t->copy = tc_xstrdup(line);
    t->n = 0;
    for (;;) {
        while (is_sep(*p))
            p++;
        if (!*p || *p == ';')
            return NULL;
        if (t->n == TOKEN_LIMIT)
            return "too many tokens on one line";
        if (*p == '"') {
            t->t[t->n++] = ++p;
            char *q = strchr(p, '"');
            if (!q)
                return "unterminated string";
            *q = '\0';
            p = q + 1;
            continue;
        }
        t->t[t->n++] = p;
        while (*p && !is_sep(*p) && *p != ';')
            p++;
        if (*p == ';') {
            *p = '\0';
            return NULL;
        }
        if (*p)
            *p++ = '\0';
    }
}

static int identifier(const char *s)
{
    if (!isalpha((unsigned char)*s) && *s != '_')
        return 0;
    while (*++s)
        if (!isalnum((unsigned char)*s) && *s != '_')
            return 0;
    return 1;
}

static int instruction_name(const char *s)
{
    return tc_same_name(s, "NAND") || tc_same_name(s, "STO");
}

/* ---- cells --------------------------------------------------------------------------------- */

static uint64_t name_hash(const char *s)
{
    uint64_t h = 0xcbf29ce484222325ull;
    for (; *s; s++)
        h = (h ^ (uint64_t)(unsigned char)tolower((unsigned char)*s)) * 0x100000001b3ull;
    return h;
}

static size_t slot_of(const Asm *a, const char *name)
{
    size_t i = (size_t)name_hash(name) & (a->nslots - 1);
    while (a->slots[i] && !tc_same_name(a->names[a->slots[i] - 1], name))
        i = (i + 1) & (a->nslots - 1);
    return i;
}

static void grow_slots(Asm *a)
{
    free(a->slots);
    a->nslots = a->nslots ? 2 * a->nslots : 256;
    a->slots = tc_xcalloc(a->nslots, sizeof *a->slots);
    for (uint32_t c = 0; c < a->ncells; c++)
        a->slots[slot_of(a, a->names[c])] = c + 1;
}

static int lookup(const Asm *a, const char *name)
{
    size_t i = slot_of(a, name);
    return a->slots[i] ? (int)a->slots[i] - 1 : -1;
}

static uint32_t cell(Asm *a, const char *name)
{
    size_t i = slot_of(a, name);
    if (a->slots[i])
        return a->slots[i] - 1;
    if (a->ncells == a->capcells) {
        a->capcells = a->capcells ? 2 * a->capcells : 64;
        a->names = tc_xrealloc(a->names, a->capcells * sizeof *a->names);
        a->info = tc_xrealloc(a->info, a->capcells * sizeof *a->info);
    }
    uint32_t c = a->ncells++;
    a->names[c] = tc_xstrdup(name);
    memset(&a->info[c], 0, sizeof a->info[c]);
    int d = tc_program_id_name(name);
    if (d >= 0) {
        a->info[c].kind = CK_ID;
        a->info[c].dim = (uint8_t)d;
        a->special = 1;
    }
    a->slots[i] = c + 1;
    if (2 * (size_t)a->ncells > a->nslots)
        grow_slots(a);
    return c;
}

static int readonly(const Asm *a, uint32_t c)
{
    return c < CELL_FIRST_FREE || a->info[c].kind != CK_PLAIN;
}

static const char *kind_text(const Asm *a, uint32_t c)
{
    return c < CELL_FIRST_FREE ? "constant" : a->info[c].kind == CK_ID ? "lane-id" : "link";
}

static int name_ok(Asm *a, const Where *w, int line, const char *tok)
{
    if (tok[0] == '@') {
        if (w->in_macro)
            return 1;
        error(a, w, line, "'%s': @names are only allowed inside macros", tok);
        return 0;
    }
    if (identifier(tok))
        return 1;
    error(a, w, line, "'%s' is not a valid cell name", tok);
    return 0;
}

static void io_list(Asm *a, const Where *w, int line, const Toks *t, uint32_t **list, size_t *n,
                    size_t *cap)
{
    if (t->n < 2) {
        error(a, w, line, "%s expects at least one cell name", t->t[0]);
        return;
    }
    for (int i = 1; i < t->n; i++) {
        if (!name_ok(a, w, line, t->t[i]))
            return;
        uint32_t c = cell(a, t->t[i]);
        if (readonly(a, c)) {
            error(a, w, line, "%s is a %s cell", t->t[i], kind_text(a, c));
            return;
        }
        for (size_t k = 0; k < *n; k++)
            if ((*list)[k] == c) {
                error(a, w, line, "%s is declared twice", t->t[i]);
                return;
            }
        if (*n == *cap) {
            *cap = *cap ? 2 * *cap : 16;
            *list = tc_xrealloc(*list, *cap * sizeof **list);
        }
        (*list)[(*n)++] = c;
    }
}

/* .link y = x @ d, spaces optional: the tokens are joined first. */
static void link_line(Asm *a, const Where *w, int line, const Toks *t)
{
    char buf[512];
    size_t n = 0;
    for (int i = 1; i < t->n; i++) {
        size_t k = strlen(t->t[i]);
        if (n + k + 1 > sizeof buf) {
            error(a, w, line, ".link line too long");
            return;
        }
        memcpy(buf + n, t->t[i], k);
        n += k;
    }
    buf[n] = '\0';
    char *eq = strchr(buf, '=');
    char *at = eq ? strrchr(eq + 1, '@') : NULL;
    if (!eq || !at) {
        error(a, w, line, ".link expects: .link name = cell @ dimension");
        return;
    }
    *eq = '\0';
    *at = '\0';
    const char *name = buf, *src = eq + 1, *dim = at + 1;
    char *end;
    long d = strtol(dim, &end, 10);
    if (!*dim || *end || d < 0 || d >= CUBE_MAX_DIMS) {
        error(a, w, line, "the dimension must be 0 to %d, got '%s'", CUBE_MAX_DIMS - 1, dim);
        return;
    }
    if (!name_ok(a, w, line, name) || !name_ok(a, w, line, src))
        return;
    if (lookup(a, name) >= 0) {
        error(a, w, line, "%s is already a cell: declare a link before its first use", name);
        return;
    }
    if (tc_program_id_name(name) >= 0) {
        error(a, w, line, "%s is a lane-id cell", name);
        return;
    }
    if (tc_same_name(name, src)) {
        error(a, w, line, "a link cannot read itself");
        return;
    }
    uint32_t s = cell(a, src), y = cell(a, name);
    a->info[y].kind = CK_LINK;
    a->info[y].dim = (uint8_t)d;
    a->info[y].src = s;
    a->special = 1;
}

/* ---- files --------------------------------------------------------------------------------- */

/* UTF-16 (with a byte order mark) becomes 8-bit text, a UTF-8 byte order mark is dropped. */
static size_t normalize(char *buf, size_t len)
{
    unsigned char *b = (unsigned char *)buf;
    if (len >= 2 && ((b[0] == 0xFF && b[1] == 0xFE) || (b[0] == 0xFE && b[1] == 0xFF))) {
        int little = b[0] == 0xFF;
        size_t n = 0;
        for (size_t i = 2; i + 1 < len; i += 2) {
            unsigned c = little ? (unsigned)b[i] | (unsigned)b[i + 1] << 8
                                : (unsigned)b[i] << 8 | (unsigned)b[i + 1];
            b[n++] = (unsigned char)(c < 128 ? c : '?');
        }
        b[n] = '\0';
        return n;
    }
    if (len >= 3 && b[0] == 0xEF && b[1] == 0xBB && b[2] == 0xBF) {
        memmove(b, b + 3, len - 2);
        return len - 3;
    }
    return len;
}

static char *slurp(const char *path)
{
    FILE *f = fopen(path, "rb");
    if (!f)
        return NULL;
    size_t len = 0, cap = 1 << 16;
    char *buf = tc_xmalloc(cap);
    for (;;) {
        size_t got = fread(buf + len, 1, cap - len - 1, f);
        if (!got)
            break;
        len += got;
        if (len + 1 == cap) {
            cap *= 2;
            buf = tc_xrealloc(buf, cap);
        }
    }
    fclose(f);
    buf[len] = '\0';
    normalize(buf, len);
    return buf;
}

static char *directory(const char *path)
{
    const char *slash = NULL;
    for (const char *p = path; *p; p++)
        if (*p == '/' || *p == '\\')
            slash = p;
    if (!slash)
        return tc_xstrdup(".");
    size_t n = slash == path ? 1 : (size_t)(slash - path);
    char *d = tc_xmalloc(n + 1);
    memcpy(d, path, n);
    d[n] = '\0';
    return d;
}

static void assemble_text(Asm *a, char *text, const char *file, const char *dir,
                          const char *from, int depth)
{
    if ((unsigned char)text[0] == 0xEF && (unsigned char)text[1] == 0xBB &&
        (unsigned char)text[2] == 0xBF)
        text += 3;
    int n = 1;
    for (const char *p = text; *p; p++)
        n += *p == '\n';
    char **lines = tc_xmalloc((size_t)n * sizeof *lines);
    int k = 0;
    lines[k++] = text;
    for (char *p = text; *p; p++)
        if (*p == '\n') {
            *p = '\0';
            lines[k++] = p + 1;
        }
    Where w = {file, dir, from, depth, 0};
    assemble_lines(a, &w, lines, NULL, n);
    free(lines);
}

static void include(Asm *a, const Where *w, int line, const char *name)
{
    if (w->depth >= NEST_LIMIT) {
        error(a, w, line, "includes nested too deeply");
        return;
    }
    char path[1024];
    int absolute = name[0] == '/' || name[0] == '\\' || (name[0] && name[1] == ':');
    if (absolute)
        snprintf(path, sizeof path, "%s", name);
    else
        snprintf(path, sizeof path, "%s/%s", w->dir, name);
    char *text = slurp(path);
    if (!text) {
        error(a, w, line, "cannot open include file '%s'", path);
        return;
    }
    char *dir = directory(path);
    assemble_text(a, text, path, dir, w->from, w->depth + 1);
    free(dir);
    free(text);
}

/* ---- macros -------------------------------------------------------------------------------- */

static Macro *find_macro(Asm *a, const char *name)
{
    for (int i = 0; i < a->nmacros; i++)
        if (tc_same_name(a->macros[i].name, name))
            return &a->macros[i];
    return NULL;
}

static int param(const Macro *m, const char *tok)
{
    for (int i = 0; i < m->nparams; i++)
        if (tc_same_name(m->params[i], tok))
            return i;
    return -1;
}

/* Reads the body of a .macro starting at lines[start]; returns the index of its .endm. */
static int define_macro(Asm *a, const Where *w, const Toks *head, char **lines, const int *nos,
                        int start, int n)
{
    int line = nos ? nos[start] : start + 1, end;
    for (end = start + 1; end < n; end++) {
        Toks t;
        const char *e = split(lines[end], &t);
        int is_end = !e && t.n > 0 && tc_same_name(t.t[0], ".endm");
        int nested = !e && t.n > 0 && tc_same_name(t.t[0], ".macro");
        free(t.copy);
        if (nested) {
            error(a, w, nos ? nos[end] : end + 1, "macros cannot be defined inside macros");
            return n;
        }
        if (is_end)
            break;
    }
    if (end == n) {
        error(a, w, line, "missing .endm for macro %s", head->n > 1 ? head->t[1] : "");
        return n;
    }
    if (head->n < 2 || !identifier(head->t[1])) {
        error(a, w, line, ".macro expects a name");
        return end;
    }
    const char *name = head->t[1];
    if (instruction_name(name)) {
        error(a, w, line, "cannot redefine instruction %s", name);
        return end;
    }
    if (find_macro(a, name)) {
        error(a, w, line, "macro %s is already defined", name);
        return end;
    }
    for (int i = 2; i < head->n; i++) {
        if (!identifier(head->t[i]) || instruction_name(head->t[i])) {
            error(a, w, line, "'%s' is not a valid parameter name", head->t[i]);
            return end;
        }
        for (int k = 2; k < i; k++)
            if (tc_same_name(head->t[k], head->t[i])) {
                error(a, w, line, "parameter %s is listed twice", head->t[i]);
                return end;
            }
    }
    if (a->nmacros == a->capmacros) {
        a->capmacros = a->capmacros ? 2 * a->capmacros : 16;
        a->macros = tc_xrealloc(a->macros, (size_t)a->capmacros * sizeof *a->macros);
    }
    Macro *m = &a->macros[a->nmacros++];
    m->name = tc_xstrdup(name);
    m->nparams = head->n - 2;
    m->params = tc_xmalloc((size_t)(m->nparams + 1) * sizeof *m->params);
    for (int i = 0; i < m->nparams; i++)
        m->params[i] = tc_xstrdup(head->t[i + 2]);
    m->nlines = end - start - 1;
    m->lines = tc_xmalloc((size_t)(m->nlines + 1) * sizeof *m->lines);
    m->line_no = tc_xmalloc((size_t)(m->nlines + 1) * sizeof *m->line_no);
    for (int i = 0; i < m->nlines; i++) {
        m->lines[i] = tc_xstrdup(lines[start + 1 + i]);
        m->line_no[i] = nos ? nos[start + 1 + i] : start + 2 + i;
    }
    m->file = tc_xstrdup(w->file);
    m->dir = tc_xstrdup(w->dir);
    return end;
}

typedef struct {
    char  *s;
    size_t len, cap;
} Buf;

static void buf_add(Buf *b, const char *s)
{
    size_t n = strlen(s);
    if (b->len + n + 1 > b->cap) {
        b->cap = 2 * (b->len + n + 1);
        b->s = tc_xrealloc(b->s, b->cap);
    }
    memcpy(b->s + b->len, s, n + 1);
    b->len += n;
}

/* One macro call: parameters substituted, pieces joined at '#', every @local renamed to
   "@<call>:<name>" (names that already hold ':' belong to an outer call), then the body is
   assembled in the macro's own file context. */
static void call_macro(Asm *a, const Where *w, int line, const Macro *m, char *const *args)
{
    if (w->depth >= NEST_LIMIT) {
        error(a, w, line, "macros nested too deeply (does %s call itself?)", m->name);
        return;
    }
    for (int i = 0; i < m->nparams; i++) {
        size_t digits = strspn(args[i], "0123456789");
        if (!(digits > 0 && !args[i][digits]) && !name_ok(a, w, line, args[i]))
            return;
    }
    unsigned id = ++a->calls;
    char from[512];
    if (!w->from)
        snprintf(from, sizeof from, "%s:%d", w->file, line);
    Where sub = {m->file, m->dir, w->from ? w->from : from, w->depth + 1, 1};

    int n = m->nlines;
    const int *nos = m->line_no;
    char **body = tc_xmalloc((size_t)(n + 1) * sizeof *body);
    for (int b = 0; b < n; b++) {
        Toks t;
        Buf out = {0};
        buf_add(&out, "");
        const char *e = split(m->lines[b], &t);
        if (e)
            error(a, &sub, nos[b], "%s", e);
        for (int i = 0; !e && i < t.n; i++) {
            const char *tok = t.t[i];
            char joined[300], local[320];
            if (strchr(tok, '#')) {
                size_t at = 0;
                const char *s = tok;
                for (;;) {
                    const char *h = strchr(s, '#');
                    size_t len = h ? (size_t)(h - s) : strlen(s);
                    char piece[300];
                    snprintf(piece, sizeof piece, "%.*s", (int)len, s);
                    int p = param(m, piece);
                    at += (size_t)snprintf(joined + at, sizeof joined - at, "%s",
                                           p >= 0 ? args[p] : piece);
                    if (!h || at >= sizeof joined)
                        break;
                    s = h + 1;
                }
                tok = joined;
            } else {
                int p = param(m, tok);
                if (p >= 0)
                    tok = args[p];
            }
            if (tok[0] == '@' && tok[1] && !strchr(tok, ':')) {
                if (!identifier(tok + 1)) {
                    error(a, &sub, nos[b], "'%s' is not a valid local name", tok);
                    break;
                }
                snprintf(local, sizeof local, "@%u:%s", id, tok + 1);
                tok = local;
            }
            int quote = !*tok || strchr(tok, ' ');
            if (i)
                buf_add(&out, " ");
            if (quote)
                buf_add(&out, "\"");
            buf_add(&out, tok);
            if (quote)
                buf_add(&out, "\"");
        }
        free(t.copy);
        body[b] = out.s;
    }
    if (!a->failed)
        assemble_lines(a, &sub, body, nos, n);
    for (int b = 0; b < n; b++)
        free(body[b]);
    free(body);
}

/* ---- lines --------------------------------------------------------------------------------- */

static void one_line(Asm *a, const Where *w, int line, const Toks *t)
{
    const char *op = t->t[0];
    if (op[0] == '.') {
        if (tc_same_name(op, ".in"))
            io_list(a, w, line, t, &a->in, &a->nin, &a->capin);
        else if (tc_same_name(op, ".out"))
            io_list(a, w, line, t, &a->out, &a->nout, &a->capout);
        else if (tc_same_name(op, ".link"))
            link_line(a, w, line, t);
        else if (tc_same_name(op, ".include") && t->n == 2)
            include(a, w, line, t->t[1]);
        else if (tc_same_name(op, ".include"))
            error(a, w, line, ".include expects one file name");
        else if (tc_same_name(op, ".endm"))
            error(a, w, line, ".endm without .macro");
        else
            error(a, w, line, "unknown directive %s", op);
        return;
    }
    if (instruction_name(op)) {
        if (t->n != 2) {
            error(a, w, line, "%s expects exactly one cell", op);
            return;
        }
        if (!name_ok(a, w, line, t->t[1]))
            return;
        uint32_t c = cell(a, t->t[1]);
        int sto = tc_same_name(op, "STO");
        if (sto && readonly(a, c)) {
            error(a, w, line, "cannot store to %s cell %s", kind_text(a, c), t->t[1]);
            return;
        }
        if (a->len == a->cap) {
            a->cap = a->cap ? 2 * a->cap : 256;
            a->code = tc_xrealloc(a->code, a->cap * sizeof *a->code);
        }
        a->code[a->len].op = (uint8_t)(sto ? OP_STO : OP_NAND);
        a->code[a->len].addr = c;
        a->len++;
        return;
    }
    const Macro *m = find_macro(a, op);
    if (!m) {
        error(a, w, line, "unknown instruction or macro '%s'", op);
        return;
    }
    if (t->n - 1 != m->nparams) {
        error(a, w, line, "macro %s expects %d argument%s, got %d", m->name, m->nparams,
              m->nparams == 1 ? "" : "s", t->n - 1);
        return;
    }
    call_macro(a, w, line, m, t->t + 1);
}

static void assemble_lines(Asm *a, const Where *w, char **lines, const int *nos, int n)
{
    for (int i = 0; i < n && !a->failed; i++) {
        int line = nos ? nos[i] : i + 1;
        Toks t;
        const char *e = split(lines[i], &t);
        if (e)
            error(a, w, line, "%s", e);
        else if (t.n > 0 && tc_same_name(t.t[0], ".macro"))
            i = define_macro(a, w, &t, lines, nos, i, n);
        else if (t.n > 0)
            one_line(a, w, line, &t);
        free(t.copy);
    }
}

/* ---- entry points -------------------------------------------------------------------------- */

static void start(Asm *a, char *err, size_t errlen)
{
    memset(a, 0, sizeof *a);
    a->err = err;
    a->errlen = errlen;
    if (errlen)
        err[0] = '\0';
    grow_slots(a);
    cell(a, "ZERO");
    cell(a, "ONE");
}

static int finish(Asm *a, Program *out)
{
    for (int i = 0; i < a->nmacros; i++) {
        Macro *m = &a->macros[i];
        for (int k = 0; k < m->nparams; k++)
            free(m->params[k]);
        for (int k = 0; k < m->nlines; k++)
            free(m->lines[k]);
        free(m->name);
        free(m->params);
        free(m->lines);
        free(m->line_no);
        free(m->file);
        free(m->dir);
    }
    free(a->macros);
    free(a->slots);
    Program p;
    memset(&p, 0, sizeof p);
    p.code = a->code;
    p.len = a->len;
    p.ncells = a->ncells;
    p.cell_names = a->names;
    p.inputs = a->in;
    p.ninputs = a->nin;
    p.outputs = a->out;
    p.noutputs = a->nout;
    p.special = a->info;
    if (!a->special) {
        free(a->info);
        p.special = NULL;
    }
    if (a->failed) {
        tc_program_free(&p);
        memset(out, 0, sizeof *out);
        return 0;
    }
    *out = p;
    return 1;
}

int tc_asm_string(const char *src, const char *name, const char *base_dir, Program *out,
                  char *err, size_t errlen)
{
    Asm a;
    start(&a, err, errlen);
    char *text = tc_xstrdup(src);
    assemble_text(&a, text, name ? name : "<string>", base_dir ? base_dir : ".", NULL, 0);
    free(text);
    return finish(&a, out);
}

int tc_asm_file(const char *path, Program *out, char *err, size_t errlen)
{
    char *text = slurp(path);
    if (!text) {
        memset(out, 0, sizeof *out);
        snprintf(err, errlen, "%s: cannot open file", path);
        return 0;
    }
    Asm a;
    start(&a, err, errlen);
    char *dir = directory(path);
    assemble_text(&a, text, path, dir, NULL, 0);
    free(dir);
    free(text);
    return finish(&a, out);
}
