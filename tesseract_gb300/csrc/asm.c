/* The assembler: source text -> Program.

   The language is the reference's program format (its docs/ISA.md, src/asm.h:7-17), and the
   Program it yields must be the reference's cell for cell: cells are numbered by first
   appearance (ZERO, ONE, then every name as met in .in/.out/.link lines, instructions and macro
   bodies), names keep the spelling of their first appearance, each macro call numbers its @local
   names @<call>:<name>, and errors read "file:line: message", with " (in macro called at
   file:line)" naming the outermost call when the line came from a macro body.  Macro expansion
   in that language is textual: a call rewrites each body line (parameters replaced, '#' pieces
   joined, @locals renamed, tokens with blanks quoted) into a line that is then read like any
   other, so this assembler does the same.

   The design here: one driver loop pulls lines from an explicit stack of frames -- the source
   text, each included file, each macro call's rewritten body -- instead of recursing into
   includes and calls; a macro definition is cut out of the frame it appears in; cells and macros
   live in hash tables keyed by their case-folded names. */
#include <ctype.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include "tc_host.h"

#define NEST_LIMIT  64   /* frames above the source: macro calls and includes together */
#define LINE_TOKENS 128  /* tokens on one line */

/* ---- names ----------------------------------------------------------------------------------- */

static int name_char(int c)
{
    return isalnum(c) || c == '_';
}

/* A name: letters, digits and '_', not starting with a digit. */
static int is_name(const char *s)
{
    if (!isalpha((unsigned char)*s) && *s != '_')
        return 0;
    while (*++s)
        if (!name_char((unsigned char)*s))
            return 0;
    return 1;
}

static int is_opcode(const char *s)
{
    return tc_same_name(s, "NAND") || tc_same_name(s, "STO");
}

/* An open-addressing table from case-folded names to indices. */
typedef struct {
    uint32_t *slot;  /* index + 1, 0 = empty */
    size_t    cap;   /* a power of two */
} NameTable;

static uint64_t fold_hash(const char *s)
{
    uint64_t h = 0x9ae16a3b2f90404full;
    for (; *s; s++)
        h = (h ^ (uint64_t)tolower((unsigned char)*s)) * 0x100000001b3ull;
    return h ^ (h >> 32);
}

/* The index of `name` (case ignored) among names[] through the table, or -1. */
static long table_find(const NameTable *t, char *const *names, const char *name)
{
    if (!t->cap)
        return -1;
    for (size_t i = fold_hash(name) & (t->cap - 1);; i = (i + 1) & (t->cap - 1)) {
        if (!t->slot[i])
            return -1;
        if (tc_same_name(names[t->slot[i] - 1], name))
            return (long)t->slot[i] - 1;
    }
}

/* Records names[index] (not yet present); keeps the table at most half full. */
static void table_add(NameTable *t, char *const *names, uint32_t index)
{
    if (2 * (size_t)(index + 1) > t->cap) {
        size_t cap = t->cap ? 2 * t->cap : 64;
        free(t->slot);
        t->slot = tc_xcalloc(cap, sizeof *t->slot);
        t->cap = cap;
        for (uint32_t k = 0; k < index; k++)
            table_add(t, names, k);
    }
    size_t i = fold_hash(names[index]) & (t->cap - 1);
    while (t->slot[i])
        i = (i + 1) & (t->cap - 1);
    t->slot[i] = index + 1;
}

/* ---- text ------------------------------------------------------------------------------------ */

typedef struct {
    char *s;
    size_t n, cap;
} Text;

static void text_put(Text *t, const char *s, size_t n)
{
    if (t->n + n + 1 > t->cap) {
        t->cap = 2 * (t->n + n + 1);
        t->s = tc_xrealloc(t->s, t->cap);
    }
    memcpy(t->s + t->n, s, n);
    t->n += n;
    t->s[t->n] = '\0';
}

static void text_puts(Text *t, const char *s)
{
    text_put(t, s, strlen(s));
}

/* The tokens of one line, cut out of a private copy of it.  Blanks, tabs, carriage returns and
   commas separate tokens; ';' ends the line; a token that starts with '"' runs to the next '"'
   (which it does not include) and may hold any of those.  Returns NULL or an error message. */
typedef struct {
    char *copy;
    char *tok[LINE_TOKENS];
    int   n;
} Line;

static int separator(char c)
{
    return c == ' ' || c == '\t' || c == ',' || c == '\r';
}

static const char *lex(const char *src, Line *l)
{
    char *p = l->copy = tc_xstrdup(src);
    l->n = 0;
    for (;;) {
        while (separator(*p))
            p++;
        if (!*p || *p == ';')
            return NULL;
        if (l->n == LINE_TOKENS)
            return "too many tokens on one line";
        if (*p == '"') {
            char *close = strchr(p + 1, '"');
            if (!close)
                return "unterminated string";
            *close = '\0';
            l->tok[l->n++] = p + 1;
            p = close + 1;
            continue;
        }
        l->tok[l->n++] = p;
        p += strcspn(p, " \t,\r;");
        if (*p == ';') {
            *p = '\0';
            return NULL;
        }
        if (*p)
            *p++ = '\0';
    }
}

static void line_free(Line *l)
{
    free(l->copy);
    l->copy = NULL;
}

/* UTF-16 with a byte order mark (as Windows PowerShell 5 writes files) becomes 8-bit text, each
   character beyond ASCII a '?'; a UTF-8 byte order mark is dropped.  buf[len] is 0. */
static void normalize(char *buf, size_t len)
{
    unsigned char *b = (unsigned char *)buf;
    if (len >= 2 && (b[0] == 0xFF || b[0] == 0xFE) && b[1] == (b[0] ^ 0x01)) {
        int hi_first = b[0] == 0xFE;
        size_t k = 0;
        for (size_t i = 2; i + 1 < len; i += 2) {
            unsigned c = hi_first ? (unsigned)b[i] << 8 | b[i + 1]
                                  : (unsigned)b[i + 1] << 8 | b[i];
            b[k++] = c < 0x80 ? (unsigned char)c : '?';
        }
        b[k] = '\0';
    } else if (len >= 3 && b[0] == 0xEF && b[1] == 0xBB && b[2] == 0xBF) {
        memmove(b, b + 3, len - 2);
    }
}

static char *read_text(const char *path)
{
    FILE *f = fopen(path, "rb");
    if (!f)
        return NULL;
    Text t = {0};
    char chunk[65536];
    size_t got;
    text_put(&t, "", 0);
    while ((got = fread(chunk, 1, sizeof chunk, f)) > 0)
        text_put(&t, chunk, got);
    fclose(f);
    normalize(t.s, t.n);
    return t.s;
}

/* The directory part of a path ('/' or '\\' separated), "." when it has none. */
static char *parent_dir(const char *path)
{
    const char *cut = NULL;
    for (const char *p = path; *p; p++)
        if (*p == '/' || *p == '\\')
            cut = p;
    if (!cut)
        return tc_xstrdup(".");
    size_t n = cut == path ? 1 : (size_t)(cut - path);
    char *d = tc_xmalloc(n + 1);
    memcpy(d, path, n);
    d[n] = '\0';
    return d;
}

/* ---- the assembler's state --------------------------------------------------------------------- */

typedef struct {
    char       *name;
    char      **params;
    int         nparams;
    char      **body;     /* raw lines between .macro and .endm */
    int        *body_no;  /* their line numbers */
    int         nbody;
    const char *file, *dir;  /* where it was defined */
} Macro;

/* Where lines come from: the source text, an included file, or one macro call's body. */
typedef struct {
    char      **lines;
    int        *nos;        /* line numbers (in `file`) */
    int         n, at;
    const char *file, *dir;
    const char *from;       /* the outermost macro call ("file:line"), NULL outside macros */
    int         depth;      /* frames below this one */
    int         local_ok;   /* a macro body: @names allowed */
    char       *text;       /* the buffer lines[] point into, or NULL when each line is owned */
} Frame;

typedef struct {
    /* the program */
    Instr    *code;
    size_t    len, capcode;
    char    **names;
    CellInfo *info;
    uint32_t  ncells, capcells;
    int       special;
    uint32_t *in, *out;
    size_t    nin, nout, capin, capout;
    NameTable cells;
    /* macros */
    Macro    *macros;
    char    **macro_names;
    int       nmacros, capmacros;
    NameTable macro_table;
    unsigned  calls;       /* macro calls so far: numbers the @locals */
    /* lines */
    Frame    *frames;
    int       nframes, capframes;
    char    **strings;     /* file names, directories, call sites: alive until the end */
    size_t    nstrings, capstrings;
    /* errors */
    char     *err;
    size_t    errlen;
    int       failed;
} Asm;

static const char *keep(Asm *a, char *s)  /* takes ownership of s */
{
    if (a->nstrings == a->capstrings) {
        a->capstrings = a->capstrings ? 2 * a->capstrings : 16;
        a->strings = tc_xrealloc(a->strings, a->capstrings * sizeof *a->strings);
    }
    a->strings[a->nstrings++] = s;
    return s;
}

/* Records the first error: "file:line: message", plus the outermost macro call. */
static void error(Asm *a, const Frame *f, int line, const char *fmt, ...)
{
    if (a->failed++ || !a->errlen)
        return;
    size_t at = 0, room = a->errlen;
    int k = snprintf(a->err, room, "%s:%d: ", f->file, line);
    at = k > 0 ? (size_t)k : 0;
    if (at < room) {
        va_list ap;
        va_start(ap, fmt);
        k = vsnprintf(a->err + at, room - at, fmt, ap);
        va_end(ap);
        at += k > 0 ? (size_t)k : 0;
    }
    if (f->from && at < room)
        snprintf(a->err + at, room - at, " (in macro called at %s)", f->from);
}

/* ---- cells ------------------------------------------------------------------------------------- */

/* The cell called `name`, created at the end of the numbering when new (ID0..ID15 are lane-id
   cells). */
static uint32_t cell(Asm *a, const char *name)
{
    long found = table_find(&a->cells, a->names, name);
    if (found >= 0)
        return (uint32_t)found;
    if (a->ncells == a->capcells) {
        a->capcells = a->capcells ? 2 * a->capcells : 64;
        a->names = tc_xrealloc(a->names, a->capcells * sizeof *a->names);
        a->info = tc_xrealloc(a->info, a->capcells * sizeof *a->info);
    }
    uint32_t c = a->ncells++;
    a->names[c] = tc_xstrdup(name);
    memset(&a->info[c], 0, sizeof a->info[c]);
    int bit = tc_program_id_name(name);
    if (bit >= 0) {
        a->info[c].kind = CK_ID;
        a->info[c].dim = (uint8_t)bit;
        a->special = 1;
    }
    table_add(&a->cells, a->names, c);
    return c;
}

static const char *readonly_kind(const Asm *a, uint32_t c)  /* NULL for a writable cell */
{
    if (c < CELL_FIRST_FREE)
        return "constant";
    return a->info[c].kind == CK_ID ? "lane-id" : a->info[c].kind == CK_LINK ? "link" : NULL;
}

/* A cell name in a statement: a name, or an @local (only in lines from a macro body, where the
   call has already renamed it). */
static int check_name(Asm *a, const Frame *f, int line, const char *tok)
{
    if (tok[0] == '@' && f->local_ok)
        return 1;
    if (tok[0] == '@')
        error(a, f, line, "'%s': @names are only allowed inside macros", tok);
    else if (!is_name(tok))
        error(a, f, line, "'%s' is not a valid cell name", tok);
    return !a->failed;
}

/* ---- statements -------------------------------------------------------------------------------- */

static void push_cell(uint32_t **list, size_t *n, size_t *cap, uint32_t c)
{
    if (*n == *cap) {
        *cap = *cap ? 2 * *cap : 16;
        *list = tc_xrealloc(*list, *cap * sizeof **list);
    }
    (*list)[(*n)++] = c;
}

/* .in / .out NAME... */
static void declare_io(Asm *a, const Frame *f, int line, const Line *l, int output)
{
    uint32_t **list = output ? &a->out : &a->in;
    size_t *n = output ? &a->nout : &a->nin, *cap = output ? &a->capout : &a->capin;
    if (l->n == 1)
        error(a, f, line, "%s expects at least one cell name", l->tok[0]);
    for (int i = 1; i < l->n && !a->failed; i++) {
        const char *name = l->tok[i];
        if (!check_name(a, f, line, name))
            return;
        uint32_t c = cell(a, name);
        const char *ro = readonly_kind(a, c);
        if (ro) {
            error(a, f, line, "%s is a %s cell", name, ro);
            return;
        }
        for (size_t k = 0; k < *n; k++)
            if ((*list)[k] == c) {
                error(a, f, line, "%s is declared twice", name);
                return;
            }
        push_cell(list, n, cap, c);
    }
}

/* .link NAME = SOURCE @ DIM, the tokens read as one string (blanks anywhere).  The dimension
   follows the last '@' after the '='.  NAME must be a new cell, so links never form a loop. */
static void declare_link(Asm *a, const Frame *f, int line, const Line *l)
{
    char s[512];
    size_t len = 0;
    for (int i = 1; i < l->n; i++) {
        size_t k = strlen(l->tok[i]);
        if (len + k >= sizeof s) {
            error(a, f, line, ".link line too long");
            return;
        }
        memcpy(s + len, l->tok[i], k);
        len += k;
    }
    s[len] = '\0';
    char *eq = strchr(s, '=');
    char *at = eq ? strrchr(eq, '@') : NULL;
    if (!at) {
        error(a, f, line, ".link expects: .link name = cell @ dimension");
        return;
    }
    *eq = *at = '\0';
    const char *name = s, *src = eq + 1, *dim = at + 1;
    char *end;
    long d = strtol(dim, &end, 10);
    if (end == dim || *end || d < 0 || d >= CUBE_MAX_DIMS) {
        error(a, f, line, "the dimension must be 0 to %d, got '%s'", CUBE_MAX_DIMS - 1, dim);
        return;
    }
    if (!check_name(a, f, line, name) || !check_name(a, f, line, src))
        return;
    if (table_find(&a->cells, a->names, name) >= 0)
        error(a, f, line, "%s is already a cell: declare a link before its first use", name);
    else if (tc_program_id_name(name) >= 0)
        error(a, f, line, "%s is a lane-id cell", name);
    else if (tc_same_name(name, src))
        error(a, f, line, "a link cannot read itself");
    if (a->failed)
        return;
    uint32_t from = cell(a, src);  /* the source is numbered before the link */
    uint32_t y = cell(a, name);
    a->info[y].kind = CK_LINK;
    a->info[y].dim = (uint8_t)d;
    a->info[y].src = from;
    a->special = 1;
}

/* NAND CELL / STO CELL */
static void instruction(Asm *a, const Frame *f, int line, const Line *l)
{
    if (l->n != 2) {
        error(a, f, line, "%s expects exactly one cell", l->tok[0]);
        return;
    }
    if (!check_name(a, f, line, l->tok[1]))
        return;
    uint32_t c = cell(a, l->tok[1]);
    int store = tc_same_name(l->tok[0], "STO");
    const char *ro = readonly_kind(a, c);
    if (store && ro) {
        error(a, f, line, "cannot store to %s cell %s", ro, l->tok[1]);
        return;
    }
    if (a->len == a->capcode) {
        a->capcode = a->capcode ? 2 * a->capcode : 256;
        a->code = tc_xrealloc(a->code, a->capcode * sizeof *a->code);
    }
    a->code[a->len].op = (uint8_t)(store ? OP_STO : OP_NAND);
    a->code[a->len].addr = c;
    a->len++;
}

/* ---- frames ------------------------------------------------------------------------------------ */

static Frame *push_frame(Asm *a)
{
    if (a->nframes == a->capframes) {
        a->capframes = a->capframes ? 2 * a->capframes : 8;
        a->frames = tc_xrealloc(a->frames, (size_t)a->capframes * sizeof *a->frames);
    }
    Frame *f = &a->frames[a->nframes++];
    memset(f, 0, sizeof *f);
    return f;
}

static void pop_frame(Asm *a)
{
    Frame *f = &a->frames[--a->nframes];
    if (f->text)
        free(f->text);
    else
        for (int i = 0; i < f->n; i++)
            free(f->lines[i]);
    free(f->lines);
    free(f->nos);
}

/* A frame over `text` (taken over), split at newlines, numbered from 1. */
static void push_text(Asm *a, char *text, const char *file, const char *dir, const char *from,
                      int depth)
{
    char *start = text;
    if ((unsigned char)start[0] == 0xEF && (unsigned char)start[1] == 0xBB &&
        (unsigned char)start[2] == 0xBF)
        start += 3;
    int n = 1;
    for (const char *p = start; *p; p++)
        n += *p == '\n';
    Frame *f = push_frame(a);
    f->lines = tc_xmalloc((size_t)n * sizeof *f->lines);
    f->nos = tc_xmalloc((size_t)n * sizeof *f->nos);
    char *p = start;
    for (int i = 0; i < n; i++) {
        f->lines[i] = p;
        f->nos[i] = i + 1;
        p += strcspn(p, "\n");
        if (*p)
            *p++ = '\0';
    }
    f->n = n;
    f->text = text;
    f->file = file;
    f->dir = dir;
    f->from = from;
    f->depth = depth;
}

/* .include "FILE", relative to the including file's directory unless absolute. */
static void include(Asm *a, const Frame *f, int line, const char *name)
{
    if (f->depth >= NEST_LIMIT) {
        error(a, f, line, "includes nested too deeply");
        return;
    }
    char path[1024];
    int absolute = name[0] == '/' || name[0] == '\\' || (name[0] && name[1] == ':');
    snprintf(path, sizeof path, absolute ? "%s%s" : "%s/%s", absolute ? "" : f->dir, name);
    char *text = read_text(path);
    if (!text) {
        error(a, f, line, "cannot open include file '%s'", path);
        return;
    }
    const char *file = keep(a, tc_xstrdup(path));
    const char *dir = keep(a, parent_dir(path));
    const char *from = f->from;
    int depth = f->depth + 1;
    push_text(a, text, file, dir, from, depth);  /* may move the frames: f is not used after */
}

/* ---- macros ------------------------------------------------------------------------------------ */

static long find_macro(const Asm *a, const char *name)
{
    return table_find(&a->macro_table, a->macro_names, name);
}

static int param_of(const Macro *m, const char *s)
{
    for (int i = 0; i < m->nparams; i++)
        if (tc_same_name(m->params[i], s))
            return i;
    return -1;
}

/* .macro NAME PARAM... at line index `head` of f: takes the lines up to .endm out of the frame
   and defines the macro. */
static void define_macro(Asm *a, Frame *f, const Line *head)
{
    int line = f->nos[f->at - 1], end = f->at;
    for (; end < f->n; end++) {
        Line l;
        const char *bad = lex(f->lines[end], &l);
        int is_macro = !bad && l.n && tc_same_name(l.tok[0], ".macro");
        int is_end = !bad && l.n && tc_same_name(l.tok[0], ".endm");
        line_free(&l);
        if (is_macro) {
            error(a, f, f->nos[end], "macros cannot be defined inside macros");
            return;
        }
        if (is_end)
            break;
    }
    if (end == f->n) {
        error(a, f, line, "missing .endm for macro %s", head->n > 1 ? head->tok[1] : "");
        return;
    }
    int first = f->at;
    f->at = end + 1;
    const char *name = head->n > 1 ? head->tok[1] : NULL;
    if (!name || !is_name(name)) {
        error(a, f, line, ".macro expects a name");
        return;
    }
    if (is_opcode(name)) {
        error(a, f, line, "cannot redefine instruction %s", name);
        return;
    }
    if (find_macro(a, name) >= 0) {
        error(a, f, line, "macro %s is already defined", name);
        return;
    }
    for (int i = 2; i < head->n; i++) {
        if (!is_name(head->tok[i]) || is_opcode(head->tok[i])) {
            error(a, f, line, "'%s' is not a valid parameter name", head->tok[i]);
            return;
        }
        for (int k = 2; k < i; k++)
            if (tc_same_name(head->tok[k], head->tok[i])) {
                error(a, f, line, "parameter %s is listed twice", head->tok[i]);
                return;
            }
    }
    if (a->nmacros == a->capmacros) {
        a->capmacros = a->capmacros ? 2 * a->capmacros : 16;
        a->macros = tc_xrealloc(a->macros, (size_t)a->capmacros * sizeof *a->macros);
        a->macro_names = tc_xrealloc(a->macro_names,
                                     (size_t)a->capmacros * sizeof *a->macro_names);
    }
    Macro *m = &a->macros[a->nmacros];
    m->name = tc_xstrdup(name);
    m->nparams = head->n - 2;
    m->params = tc_xmalloc((size_t)(m->nparams + 1) * sizeof *m->params);
    for (int i = 0; i < m->nparams; i++)
        m->params[i] = tc_xstrdup(head->tok[i + 2]);
    m->nbody = end - first;
    m->body = tc_xmalloc((size_t)(m->nbody + 1) * sizeof *m->body);
    m->body_no = tc_xmalloc((size_t)(m->nbody + 1) * sizeof *m->body_no);
    for (int i = 0; i < m->nbody; i++) {
        m->body[i] = tc_xstrdup(f->lines[first + i]);
        m->body_no[i] = f->nos[first + i];
    }
    m->file = f->file;
    m->dir = f->dir;
    a->macro_names[a->nmacros] = m->name;
    table_add(&a->macro_table, a->macro_names, (uint32_t)a->nmacros);
    a->nmacros++;
}

/* One token of a body line as the call rewrites it: a parameter becomes its argument; with '#',
   each piece that is a parameter becomes its argument and the pieces are joined (at most 299
   characters); an @local of this call becomes @<call>:<name>.  Returns 0 after an error. */
static int rewrite_token(Asm *a, const Frame *body, int line, const Macro *m, char *const *args,
                         unsigned call, const char *tok, Text *out)
{
    char joined[300], local[320];
    if (strchr(tok, '#')) {
        size_t at = 0;
        joined[0] = '\0';
        for (const char *piece = tok; at < sizeof joined;) {
            size_t n = strcspn(piece, "#");
            char part[300];
            snprintf(part, sizeof part, "%.*s", (int)n, piece);
            int p = param_of(m, part);
            int k = snprintf(joined + at, sizeof joined - at, "%s", p >= 0 ? args[p] : part);
            at += k > 0 ? (size_t)k : 0;
            if (!piece[n])
                break;
            piece += n + 1;
        }
        tok = joined;
    } else {
        int p = param_of(m, tok);
        if (p >= 0)
            tok = args[p];
    }
    /* a lone '@' is .link syntax; a name holding ':' is an outer call's local already */
    if (tok[0] == '@' && tok[1] && !strchr(tok, ':')) {
        if (!is_name(tok + 1)) {
            error(a, body, line, "'%s' is not a valid local name", tok);
            return 0;
        }
        snprintf(local, sizeof local, "@%u:%s", call, tok + 1);
        tok = local;
    }
    int quote = !*tok || strchr(tok, ' ');
    if (quote)
        text_puts(out, "\"");
    text_puts(out, tok);
    if (quote)
        text_puts(out, "\"");
    return 1;
}

/* A call of macro mi with the tokens after the name as arguments: the rewritten body becomes a
   new frame on top of f. */
static void call_macro(Asm *a, Frame *f, int line, long mi, char *const *args)
{
    const Macro *m = &a->macros[mi];
    if (f->depth >= NEST_LIMIT) {
        error(a, f, line, "macros nested too deeply (does %s call itself?)", m->name);
        return;
    }
    for (int i = 0; i < m->nparams; i++) {
        size_t digits = strspn(args[i], "0123456789");
        if ((!digits || args[i][digits]) && !check_name(a, f, line, args[i]))
            return;
    }
    unsigned call = ++a->calls;
    const char *from = f->from;
    if (!from) {
        char site[512];
        snprintf(site, sizeof site, "%s:%d", f->file, line);
        from = keep(a, tc_xstrdup(site));
    }
    Frame body = {0};
    body.file = m->file;
    body.dir = m->dir;
    body.from = from;
    body.depth = f->depth + 1;
    body.local_ok = 1;
    body.n = m->nbody;
    body.lines = tc_xmalloc((size_t)(m->nbody + 1) * sizeof *body.lines);
    body.nos = tc_xmalloc((size_t)(m->nbody + 1) * sizeof *body.nos);
    for (int b = 0; b < m->nbody; b++) {
        Text out = {0};
        text_put(&out, "", 0);
        Line l;
        const char *bad = lex(m->body[b], &l);
        if (bad)
            error(a, &body, m->body_no[b], "%s", bad);
        for (int i = 0; !bad && i < l.n; i++) {
            if (i)
                text_puts(&out, " ");
            if (!rewrite_token(a, &body, m->body_no[b], m, args, call, l.tok[i], &out))
                break;
        }
        line_free(&l);
        body.lines[b] = out.s;
        body.nos[b] = m->body_no[b];
    }
    *push_frame(a) = body;  /* f may have moved */
}

/* ---- the driver -------------------------------------------------------------------------------- */

static void statement(Asm *a, Frame *f, int line, Line *l)
{
    const char *op = l->tok[0];
    if (op[0] == '.') {
        if (tc_same_name(op, ".in") || tc_same_name(op, ".out"))
            declare_io(a, f, line, l, tc_same_name(op, ".out"));
        else if (tc_same_name(op, ".link"))
            declare_link(a, f, line, l);
        else if (tc_same_name(op, ".include") && l->n == 2)
            include(a, f, line, l->tok[1]);
        else if (tc_same_name(op, ".include"))
            error(a, f, line, ".include expects one file name");
        else if (tc_same_name(op, ".endm"))
            error(a, f, line, ".endm without .macro");
        else
            error(a, f, line, "unknown directive %s", op);
    } else if (is_opcode(op)) {
        instruction(a, f, line, l);
    } else {
        long mi = find_macro(a, op);
        if (mi < 0)
            error(a, f, line, "unknown instruction or macro '%s'", op);
        else if (l->n - 1 != a->macros[mi].nparams)
            error(a, f, line, "macro %s expects %d argument%s, got %d", a->macros[mi].name,
                  a->macros[mi].nparams, a->macros[mi].nparams == 1 ? "" : "s", l->n - 1);
        else
            call_macro(a, f, line, mi, l->tok + 1);
    }
}

/* Reads lines from the top frame until every frame is done or an error is recorded. */
static void drive(Asm *a)
{
    while (a->nframes && !a->failed) {
        Frame *f = &a->frames[a->nframes - 1];
        if (f->at == f->n) {
            pop_frame(a);
            continue;
        }
        int line = f->nos[f->at];
        Line l;
        const char *bad = lex(f->lines[f->at++], &l);
        if (bad)
            error(a, f, line, "%s", bad);
        else if (l.n && tc_same_name(l.tok[0], ".macro"))
            define_macro(a, f, &l);
        else if (l.n)
            statement(a, f, line, &l);
        line_free(&l);
    }
    while (a->nframes)
        pop_frame(a);
}

/* ---- entry points ------------------------------------------------------------------------------ */

static void begin(Asm *a, char *err, size_t errlen)
{
    memset(a, 0, sizeof *a);
    a->err = err;
    a->errlen = errlen;
    if (errlen)
        err[0] = '\0';
    cell(a, "ZERO");
    cell(a, "ONE");
}

static int end(Asm *a, Program *out)
{
    for (int i = 0; i < a->nmacros; i++) {
        Macro *m = &a->macros[i];
        for (int k = 0; k < m->nparams; k++)
            free(m->params[k]);
        for (int k = 0; k < m->nbody; k++)
            free(m->body[k]);
        free(m->name);
        free(m->params);
        free(m->body);
        free(m->body_no);
    }
    free(a->macros);
    free(a->macro_names);
    free(a->macro_table.slot);
    free(a->cells.slot);
    for (size_t i = 0; i < a->nstrings; i++)
        free(a->strings[i]);
    free(a->strings);
    free(a->frames);
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
    if (a->special)
        p.special = a->info;
    else
        free(a->info);
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
    begin(&a, err, errlen);
    const char *file = keep(&a, tc_xstrdup(name));
    const char *dir = keep(&a, tc_xstrdup(base_dir));
    push_text(&a, tc_xstrdup(src), file, dir, NULL, 0);
    drive(&a);
    return end(&a, out);
}

int tc_asm_file(const char *path, Program *out, char *err, size_t errlen)
{
    char *text = read_text(path);
    if (!text) {
        memset(out, 0, sizeof *out);
        snprintf(err, errlen, "%s: cannot open file", path);
        return 0;
    }
    Asm a;
    begin(&a, err, errlen);
    const char *file = keep(&a, tc_xstrdup(path));
    const char *dir = keep(&a, parent_dir(path));
    push_text(&a, text, file, dir, NULL, 0);
    drive(&a);
    return end(&a, out);
}
