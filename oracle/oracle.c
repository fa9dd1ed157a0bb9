/* ORACLE — test infrastructure, not product code.

   A CPU restatement of the reference's semantics for the hot path, used only by tests/, by
   __graft_entry__.smoke() and by bench.py's CPU-baseline leg, always as the checker and never as
   the thing measured or shipped.  Every function cites the reference file and lines it restates
   (paths within the enderPeer/tesseract project).

   Parity pins: the reference machine and the enumeration below are checked against the
   reference's own known-answer tests (tests/test_work.c:244-320, tests/test_ref.c) and against
   golden vectors produced by the reference binary built from its sources (oracle/Makefile,
   tests/golden/make_golden.py).

   Contents
     orc_ref_*        the reference machine, one byte per cell, and the lockstep cube
                      (src/ref.c:49-130)
     orc_spec_value   the specification's right side (src/spec.c:344-377)
     orc_enum_run     verify / equiv / search over every assignment (src/enum.c:90-332), on a
                      bit-sliced CPU engine with the lane engine's semantics
                      (src/lanes.c:176-253, src/enum.c:115-213), on host threads
     orc_enum_ref     the same on the reference machine, one assignment at a time (small cases)
     orc_check_*      the random starting state of check_lanes (src/check.c:52-80)
     orc_life_scalar  plain C Game of Life (src/gen.c:686-700)
     orc_toyhash      plain C toy hash (src/gen.c:107-121) */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../tesseract_gb300/csrc/tc_host.h"

/* ---- the reference machine (src/ref.c) ------------------------------------------------------ */

static int readonly_cell(const Program *p, uint32_t c)
{
    return c < CELL_FIRST_FREE || (p->special && p->special[c].kind != CK_PLAIN);
}

static uint32_t follow(const Program *p, uint32_t c, unsigned *mask)
{
    unsigned m = 0;
    while (p->special && p->special[c].kind == CK_LINK) {
        m ^= 1u << p->special[c].dim;
        c = p->special[c].src;
    }
    *mask = m;
    return c;
}

unsigned orc_dims(const Program *p)
{
    unsigned d = CUBE_DIMS;
    for (uint32_t c = 0; p->special && c < p->ncells; c++)
        if (p->special[c].kind != CK_PLAIN && p->special[c].dim + 1u > d)
            d = p->special[c].dim + 1u;
    return d;
}

/* A cube of 2^dims machines (or one machine: machines = 1, no links allowed).  mem is
   machines x ncells bytes, rr one byte per machine. */
typedef struct {
    const Program *p;
    unsigned       machines;
    uint8_t       *mem, *rr;
    size_t         pc;
    uint64_t       ticks;
} OrcCube;

OrcCube *orc_cube_new(const Program *p, unsigned machines)
{
    OrcCube *c = calloc(1, sizeof *c);
    c->p = p;
    c->machines = machines;
    c->mem = calloc((size_t)machines * p->ncells + 1, 1);
    c->rr = calloc(machines + 1, 1);
    for (unsigned k = 0; k < machines; k++)
        c->mem[(size_t)k * p->ncells + CELL_ONE] = 1;
    return c;
}

void orc_cube_free(OrcCube *c)
{
    if (!c)
        return;
    free(c->mem);
    free(c->rr);
    free(c);
}

/* ref_get (src/ref.c:36-47): links followed, ids read from the machine number */
uint8_t orc_cube_get(const OrcCube *c, unsigned k, uint32_t a)
{
    const Program *p = c->p;
    if (!p->special)
        return c->mem[(size_t)k * p->ncells + a];
    unsigned mask;
    uint32_t cell = follow(p, a, &mask);
    unsigned lane = k ^ mask;
    if (p->special[cell].kind == CK_ID)
        return (uint8_t)((lane >> p->special[cell].dim) & 1);
    return c->mem[(size_t)lane * p->ncells + cell];
}

void orc_cube_set(OrcCube *c, unsigned k, uint32_t a, uint8_t v)
{
    if (!readonly_cell(c->p, a))
        c->mem[(size_t)k * c->p->ncells + a] = v ? 1 : 0;
}

uint8_t orc_cube_rr(const OrcCube *c, unsigned k) { return c->rr[k]; }
void orc_cube_set_rr(OrcCube *c, unsigned k, uint8_t v) { c->rr[k] = v ? 1 : 0; }

/* ref_cube_step (src/ref.c:119-124): one instruction in every machine.  Machine by machine is the
   same as all at once: a NAND only changes RR, a STO only the machine's own cell, and no machine
   reads during a STO. */
void orc_cube_step(OrcCube *c)
{
    const Program *p = c->p;
    if (p->len == 0) {
        c->ticks++;
        return;
    }
    Instr in = p->code[c->pc];
    for (unsigned k = 0; k < c->machines; k++) {
        if (in.op == OP_NAND)
            c->rr[k] = (uint8_t)!(c->rr[k] & orc_cube_get(c, k, in.addr));
        else if (!readonly_cell(p, in.addr))
            c->mem[(size_t)k * p->ncells + in.addr] = c->rr[k];
    }
    if (++c->pc == p->len) {
        c->pc = 0;
        c->ticks++;
    }
}

void orc_cube_tick(OrcCube *c)
{
    uint64_t t = c->ticks;
    while (c->ticks == t)
        orc_cube_step(c);
}

/* ---- the specification (src/spec.c:344-377) ------------------------------------------------- */

uint64_t orc_spec_value(const void *spec, uint64_t x)
{
    const TcSpec *s = spec;
    uint64_t var[TS_MAX_VARS], st[TS_MAX_STACK + 2];
    for (int k = 0; k < s->nvars; k++) {
        uint64_t v = 0;
        for (int b = 0; b < s->var_bits[k]; b++)
            v |= ((x >> s->var_pos[k][b]) & 1) << b;
        var[k] = v;
    }
    int sp = 0;
    for (int i = 0; i < s->nrpn; i++) {
        int op = s->rpn[i].op;
        uint64_t v = s->rpn[i].v;
        if (op == TS_NUM)
            st[sp++] = v;
        else if (op == TS_VAR)
            st[sp++] = var[v];
        else if (op == TS_NOT)
            st[sp - 1] = ~st[sp - 1];
        else if (op == TS_NEG)
            st[sp - 1] = 0 - st[sp - 1];
        else {
            uint64_t b = st[--sp];
            uint64_t a = st[sp - 1];
            switch (op) {
            case TS_ADD: a += b; break;
            case TS_SUB: a -= b; break;
            case TS_MUL: a *= b; break;
            case TS_AND: a &= b; break;
            case TS_OR:  a |= b; break;
            case TS_XOR: a ^= b; break;
            case TS_SHL: a = b < 64 ? a << b : 0; break;
            case TS_SHR: a = b < 64 ? a >> b : 0; break;
            }
            st[sp - 1] = a;
        }
    }
    return s->width == 64 ? st[0] : st[0] & ((1ull << s->width) - 1);
}

/* ---- enumeration ------------------------------------------------------------------------------ */

#define ORC_SHOW 16
#define ORC_CHUNK 64   /* passes of 512 assignments per hand-out (src/enum.c:11) */
#define ORC_PASS 512

/* enum_add_hit (src/enum.c:31-46): keep the 16 smallest */
void orc_add_hit(EnumResult *r, uint64_t x)
{
    int i;
    if (r->nhit < ORC_SHOW) {
        i = r->nhit++;
    } else {
        if (x >= r->hit[ORC_SHOW - 1])
            return;
        i = ORC_SHOW - 1;
    }
    while (i > 0 && r->hit[i - 1] > x) {
        r->hit[i] = r->hit[i - 1];
        i--;
    }
    r->hit[i] = x;
}

static int names_equal(const char *a, const char *b)
{
    for (; *a && *b; a++, b++) {
        int x = *a >= 'A' && *a <= 'Z' ? *a + 32 : *a, y = *b >= 'A' && *b <= 'Z' ? *b + 32 : *b;
        if (x != y)
            return 0;
    }
    return *a == *b;
}

/* enum_match (src/enum.c:48-78): b's index of each of a's inputs/outputs, by name */
static int match(const Program *a, const uint32_t *la, size_t na, const Program *b,
                 const uint32_t *lb, size_t nb, int *map, const char *what, char *err, size_t errlen)
{
    if (na != nb) {
        snprintf(err, errlen, "the programs have %zu and %zu %s", na, nb, what);
        return 0;
    }
    for (size_t i = 0; i < na; i++) {
        map[i] = -1;
        for (size_t j = 0; j < nb; j++)
            if (names_equal(a->cell_names[la[i]], b->cell_names[lb[j]]))
                map[i] = (int)j;
        if (map[i] < 0) {
            snprintf(err, errlen, "the second program has no %s called %s",
                     what[0] == 'i' ? "input" : "output", a->cell_names[la[i]]);
            return 0;
        }
    }
    return 1;
}

static int refusals(const Enum *e, char *err, size_t errlen)
{
    if (e->a->special || (e->mode == EN_EQUIV && e->b->special)) {
        snprintf(err, errlen, "id and link cells connect the lanes, but every input needs a lane "
                              "of its own here");
        return 0;
    }
    if (e->a->ninputs > EN_MAX_IN) {
        snprintf(err, errlen, "%zu inputs is too many to try them all (at most %d)",
                 e->a->ninputs, EN_MAX_IN);
        return 0;
    }
    if (e->parts < 1 || e->part < 0 || e->part > e->part_end || e->part_end >= e->parts ||
        e->ticks < 1) {
        snprintf(err, errlen, "bad --part or --ticks");
        return 0;
    }
    return 1;
}

/* A program decoded for the bit-sliced CPU engine: 64 lanes per uint64, LW words per line. */
enum { LW = 16 };  /* 1024 assignments per line */
typedef struct {
    const Program *p;
    uint32_t      *in;   /* in[k]: cell for input k in program a's order */
} Side;

typedef struct {
    const Enum *e;
    Side        sa, sb;
    const int  *out_map;
    uint64_t    nchunks, passes, space;
    uint64_t    next;
    pthread_mutex_t lock;
    EnumResult  total;
} Job;

typedef struct {
    uint64_t w[LW];
} Line;

/* One program over LW*64 assignments starting at x0 (a multiple of 1024): power-on state,
   inputs from x (input k = bit n-1-k), `ticks` passes (src/enum.c:115-133, src/lanes.c:197-253). */
static void run_lines(const Side *s, unsigned ticks, int n, uint64_t x0, Line *mem, Line *rr)
{
    const Program *p = s->p;
    memset(mem, 0, p->ncells * sizeof *mem);
    memset(rr, 0, sizeof *rr);
    for (int w = 0; w < LW; w++)
        mem[CELL_ONE].w[w] = ~0ull;
    for (int k = 0; k < n; k++) {
        int j = n - 1 - k;
        Line *l = &mem[s->in[k]];
        for (int w = 0; w < LW; w++) {
            uint64_t v;
            if (j < 6) {
                static const uint64_t pat[6] = {0xAAAAAAAAAAAAAAAAull, 0xCCCCCCCCCCCCCCCCull,
                                                0xF0F0F0F0F0F0F0F0ull, 0xFF00FF00FF00FF00ull,
                                                0xFFFF0000FFFF0000ull, 0xFFFFFFFF00000000ull};
                v = pat[j];
            } else {
                uint64_t x = x0 + 64 * (uint64_t)w;
                v = (x >> j) & 1 ? ~0ull : 0;
            }
            l->w[w] = v;
        }
    }
    for (unsigned t = 0; t < ticks; t++)
        for (size_t i = 0; i < p->len; i++) {
            Instr in = p->code[i];
            if (in.op == OP_NAND) {
                const Line *m = &mem[in.addr];
                for (int w = 0; w < LW; w++)
                    rr->w[w] = ~(rr->w[w] & m->w[w]);
            } else if (in.addr >= CELL_FIRST_FREE) {
                mem[in.addr] = *rr;
            }
        }
}

static void lines_for(Job *j, uint64_t x0, EnumResult *r, Line *ma, Line *mb, Line *ra, Line *rb)
{
    const Enum *e = j->e;
    int n = (int)e->a->ninputs;
    uint64_t valid[LW];
    for (int w = 0; w < LW; w++) {
        uint64_t from = x0 + 64 * (uint64_t)w;
        valid[w] = from + 64 <= j->space ? ~0ull
                 : from >= j->space      ? 0
                                         : (1ull << (j->space - from)) - 1;
    }
    run_lines(&j->sa, e->ticks, n, x0, ma, ra);
    uint64_t hit[LW];
    const TcSpec *sp = (const TcSpec *)e->spec;
    if (e->mode == EN_SEARCH) {
        uint64_t target = orc_spec_value(sp, 0);
        for (int w = 0; w < LW; w++)
            hit[w] = valid[w];
        for (int b = 0; b < sp->width; b++) {
            const Line *o = &ma[sp->out[b]];
            for (int w = 0; w < LW; w++)
                hit[w] &= (target >> b) & 1 ? o->w[w] : ~o->w[w];
        }
    } else if (e->mode == EN_EQUIV) {
        run_lines(&j->sb, e->ticks, n, x0, mb, rb);
        memset(hit, 0, sizeof hit);
        for (size_t o = 0; o < e->a->noutputs; o++) {
            const Line *la = &ma[e->a->outputs[o]], *lb = &mb[e->b->outputs[j->out_map[o]]];
            for (int w = 0; w < LW; w++)
                hit[w] |= la->w[w] ^ lb->w[w];
        }
        for (int w = 0; w < LW; w++)
            hit[w] &= valid[w];
    } else {
        memset(hit, 0, sizeof hit);
        for (int w = 0; w < LW; w++)
            for (int l = 0; l < 64; l++) {
                if (!((valid[w] >> l) & 1))
                    continue;
                uint64_t got = 0, x = x0 + 64 * (uint64_t)w + (uint64_t)l;
                for (int b = 0; b < sp->width; b++)
                    got |= ((ma[sp->out[b]].w[w] >> l) & 1) << b;
                if (got != orc_spec_value(sp, x))
                    hit[w] |= 1ull << l;
            }
    }
    for (int w = 0; w < LW; w++) {
        uint64_t v = valid[w];
        r->tried += (uint64_t)__builtin_popcountll(v);
        for (uint64_t h = hit[w]; h; h &= h - 1) {
            r->hits++;
            orc_add_hit(r, x0 + 64 * (uint64_t)w + (uint64_t)__builtin_ctzll(h));
        }
    }
}

static void *worker(void *arg)
{
    Job *j = arg;
    const Enum *e = j->e;
    EnumResult r;
    memset(&r, 0, sizeof r);
    Line *ma = calloc(e->a->ncells + 1, sizeof *ma);
    Line *mb = e->mode == EN_EQUIV ? calloc(e->b->ncells + 1, sizeof *mb) : NULL;
    Line ra, rb;
    for (;;) {
        pthread_mutex_lock(&j->lock);
        uint64_t c = j->next++;
        pthread_mutex_unlock(&j->lock);
        if (c >= j->nchunks)
            break;
        int share = (int)(c % (uint64_t)e->parts);
        if (share < e->part || share > e->part_end)
            continue;
        uint64_t first = c * ORC_CHUNK, end = first + ORC_CHUNK < j->passes ? first + ORC_CHUNK
                                                                            : j->passes;
        /* ops are counted per 512-lane pass, as the reference does (src/enum.c:164,177) */
        r.ops += (end - first) * e->ticks * ORC_PASS *
                 (e->a->len + (e->mode == EN_EQUIV ? e->b->len : 0));
        for (uint64_t x0 = first * ORC_PASS; x0 < end * ORC_PASS && x0 < j->space;
             x0 += 64 * LW)
            lines_for(j, x0, &r, ma, mb, &ra, &rb);
    }
    pthread_mutex_lock(&j->lock);
    j->total.tried += r.tried;
    j->total.hits += r.hits;
    j->total.ops += r.ops;
    for (int h = 0; h < r.nhit; h++)
        orc_add_hit(&j->total, r.hit[h]);
    pthread_mutex_unlock(&j->lock);
    free(ma);
    free(mb);
    return NULL;
}

static double seconds_now(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* enum_run (src/enum.c:244-332).  `limit_chunks` > 0 stops after that many chunks (a bounded
   sample for timing); 0 runs everything. */
int orc_enum_run(const Enum *e, EnumResult *r, int threads, uint64_t limit_chunks, char *err,
                 size_t errlen)
{
    memset(r, 0, sizeof *r);
    if (!refusals(e, err, errlen))
        return 0;
    size_t n = e->a->ninputs;
    int *in_map = calloc(n + 1, sizeof *in_map);
    int *out_map = calloc(e->a->noutputs + 1, sizeof *out_map);
    if (e->mode == EN_EQUIV &&
        !(match(e->a, e->a->inputs, n, e->b, e->b->inputs, e->b->ninputs, in_map, "inputs", err,
                errlen) &&
          match(e->a, e->a->outputs, e->a->noutputs, e->b, e->b->outputs, e->b->noutputs, out_map,
                "outputs", err, errlen))) {
        free(in_map);
        free(out_map);
        return 0;
    }
    Job j;
    memset(&j, 0, sizeof j);
    j.e = e;
    j.sa.p = e->a;
    j.sa.in = e->a->inputs;
    uint32_t *bin = NULL;
    if (e->mode == EN_EQUIV) {
        bin = calloc(n + 1, sizeof *bin);
        for (size_t k = 0; k < n; k++)
            bin[k] = e->b->inputs[in_map[k]];
        j.sb.p = e->b;
        j.sb.in = bin;
    }
    j.out_map = out_map;
    j.space = 1ull << n;
    j.passes = (j.space + ORC_PASS - 1) / ORC_PASS;
    j.nchunks = (j.passes + ORC_CHUNK - 1) / ORC_CHUNK;
    if (limit_chunks && limit_chunks < j.nchunks)
        j.nchunks = limit_chunks;
    pthread_mutex_init(&j.lock, NULL);
    if (threads < 1)
        threads = 1;
    pthread_t *tid = calloc((size_t)threads, sizeof *tid);
    double t0 = seconds_now();
    for (int i = 0; i < threads; i++)
        pthread_create(&tid[i], NULL, worker, &j);
    for (int i = 0; i < threads; i++)
        pthread_join(tid[i], NULL);
    r->seconds = seconds_now() - t0;
    r->space = j.space;
    r->tried = j.total.tried;
    r->hits = j.total.hits;
    r->ops = j.total.ops;
    r->nhit = j.total.nhit;
    memcpy(r->hit, j.total.hit, sizeof r->hit);
    r->threads = threads;
    pthread_mutex_destroy(&j.lock);
    free(tid);
    free(bin);
    free(in_map);
    free(out_map);
    return 1;
}

/* The same result from the reference machine, one assignment at a time: run_one
   (src/work.c:284-297) for every x of the selected shares.  For small input widths. */
int orc_enum_ref(const Enum *e, EnumResult *r, char *err, size_t errlen)
{
    memset(r, 0, sizeof *r);
    if (!refusals(e, err, errlen))
        return 0;
    size_t n = e->a->ninputs;
    int *in_map = calloc(n + 1, sizeof *in_map);
    int *out_map = calloc(e->a->noutputs + 1, sizeof *out_map);
    if (e->mode == EN_EQUIV &&
        !(match(e->a, e->a->inputs, n, e->b, e->b->inputs, e->b->ninputs, in_map, "inputs", err,
                errlen) &&
          match(e->a, e->a->outputs, e->a->noutputs, e->b, e->b->outputs, e->b->noutputs, out_map,
                "outputs", err, errlen))) {
        free(in_map);
        free(out_map);
        return 0;
    }
    const TcSpec *sp = (const TcSpec *)e->spec;
    uint64_t space = 1ull << n, passes = (space + ORC_PASS - 1) / ORC_PASS;
    r->space = space;
    OrcCube *ma = orc_cube_new(e->a, 1), *mb = e->mode == EN_EQUIV ? orc_cube_new(e->b, 1) : NULL;
    for (uint64_t pass = 0; pass < passes; pass++) {
        int share = (int)((pass / ORC_CHUNK) % (uint64_t)e->parts);
        if (share < e->part || share > e->part_end)
            continue;
        r->ops += e->ticks * ORC_PASS * (e->a->len + (mb ? e->b->len : 0));
        for (uint64_t x = pass * ORC_PASS; x < (pass + 1) * ORC_PASS && x < space; x++) {
            memset(ma->mem, 0, e->a->ncells);
            ma->mem[CELL_ONE] = 1;
            ma->rr[0] = 0;
            ma->pc = 0;
            for (size_t k = 0; k < n; k++)
                orc_cube_set(ma, 0, e->a->inputs[k], (uint8_t)((x >> (n - 1 - k)) & 1));
            for (unsigned t = 0; t < e->ticks; t++)
                orc_cube_tick(ma);
            int hit = 0;
            if (e->mode == EN_SEARCH) {
                uint64_t target = orc_spec_value(sp, 0), got = 0;
                for (int b = 0; b < sp->width; b++)
                    got |= (uint64_t)orc_cube_get(ma, 0, sp->out[b]) << b;
                hit = got == target;
            } else if (e->mode == EN_VERIFY) {
                uint64_t got = 0;
                for (int b = 0; b < sp->width; b++)
                    got |= (uint64_t)orc_cube_get(ma, 0, sp->out[b]) << b;
                hit = got != orc_spec_value(sp, x);
            } else {
                memset(mb->mem, 0, e->b->ncells);
                mb->mem[CELL_ONE] = 1;
                mb->rr[0] = 0;
                mb->pc = 0;
                for (size_t k = 0; k < n; k++)
                    orc_cube_set(mb, 0, e->b->inputs[in_map[k]], (uint8_t)((x >> (n - 1 - k)) & 1));
                for (unsigned t = 0; t < e->ticks; t++)
                    orc_cube_tick(mb);
                for (size_t o = 0; o < e->a->noutputs; o++)
                    hit |= orc_cube_get(ma, 0, e->a->outputs[o]) !=
                           orc_cube_get(mb, 0, e->b->outputs[out_map[o]]);
            }
            r->tried++;
            if (hit) {
                r->hits++;
                orc_add_hit(r, x);
            }
        }
    }
    orc_cube_free(ma);
    orc_cube_free(mb);
    free(in_map);
    free(out_map);
    r->threads = 1;
    return 1;
}

/* ---- check_lanes' starting state (src/check.c:60-80) ------------------------------------------ */

static uint64_t smix(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Fills a cube of 2^dims machines with check_lanes' random state: per group of 512, for every
   cell from 2 up, 8 words of splitmix64 (kept for writable cells only), then 8 words for RR;
   machine 512 g + l holds bit l % 64 of word l / 64. */
void orc_check_state(OrcCube *c, uint64_t seed)
{
    const Program *p = c->p;
    unsigned groups = c->machines / ORC_PASS;
    uint64_t s = seed;
    for (unsigned g = 0; g < groups; g++) {
        for (uint32_t a = CELL_FIRST_FREE; a < p->ncells; a++)
            for (int w = 0; w < 8; w++) {
                uint64_t v = smix(&s);
                if (readonly_cell(p, a))
                    continue;
                for (int b = 0; b < 64; b++)
                    c->mem[(size_t)(g * ORC_PASS + (unsigned)w * 64 + (unsigned)b) * p->ncells + a] =
                        (uint8_t)((v >> b) & 1);
            }
        for (int w = 0; w < 8; w++) {
            uint64_t v = smix(&s);
            for (int b = 0; b < 64; b++)
                c->rr[g * ORC_PASS + (unsigned)w * 64 + (unsigned)b] = (uint8_t)((v >> b) & 1);
        }
    }
}

/* ---- plain C workloads -------------------------------------------------------------------------- */

/* life_scalar (src/gen.c:686-700): one generation of B3/S23 on a w x h torus of 0/1 bytes */
void orc_life_scalar(uint8_t *board, int w, int h)
{
    uint8_t *next = malloc((size_t)w * (size_t)h);
    for (int r = 0; r < h; r++)
        for (int c = 0; c < w; c++) {
            int n = 0;
            for (int dr = -1; dr <= 1; dr++)
                for (int dc = -1; dc <= 1; dc++)
                    if (dr || dc)
                        n += board[((r + dr + h) % h) * w + (c + dc + w) % w];
            next[r * w + c] = (uint8_t)(n == 3 || (n == 2 && board[r * w + c]));
        }
    memcpy(board, next, (size_t)w * (size_t)h);
    free(next);
}

/* toyhash (src/gen.c:107-121) */
uint64_t orc_toyhash(uint64_t x, int n, int rounds)
{
    static const int mult[] = {5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61};
    int m = 0;
    for (size_t i = 0; i < sizeof mult / sizeof mult[0] && !m; i++) {
        int a = mult[i], b = n;
        while (b) {
            int t = a % b;
            a = b;
            b = t;
        }
        if (a == 1)
            m = mult[i];
    }
    for (int r = 0; r < rounds; r++) {
        uint64_t y = 0, z = 0;
        for (int i = 0; i < n; i++) {
            uint64_t xi = (x >> i) & 1, x1 = (x >> ((i + 1) % n)) & 1, x2 = (x >> ((i + 2) % n)) & 1;
            y |= (xi ^ (~x1 & x2 & 1)) << i;
        }
        for (int i = 0; i < n; i++)
            z |= ((y >> ((m * i + 3) % n)) & 1) << i;
        uint64_t k = (uint64_t)(r + 1) * 0x9E3779B97F4A7C15ull;
        k = (k ^ (k >> 30)) * 0xBF58476D1CE4E5B9ull;
        k = (k ^ (k >> 27)) * 0x94D049BB133111EBull;
        k ^= k >> 31;
        x = z ^ (n == 64 ? k : k & ((1ull << n) - 1));
    }
    return x;
}

/* ---- plain C Game of Life, 64 cells per word ------------------------------------------------- */

/* The same rule as life_scalar (src/gen.c:686-700): a cell is alive next if it has 3 live
   neighbours, or 2 and is alive now, on a torus.  Rows of w64 words (64 w64 columns, bit j of word
   k = column 64 k + j), `gens` generations, rows split over `threads` host threads.  The eight
   neighbour bitmaps are added with bit-sliced full adders (counts 0..8 in four bit planes). */
typedef struct {
    const uint64_t *cur;
    uint64_t       *next;
    int             w64, h, r0, r1;
} LifeRows;

static inline uint64_t west(const uint64_t *row, int k, int w64)  /* column c-1 */
{
    uint64_t x = row[k], prev = row[(k + w64 - 1) % w64];
    return (x << 1) | (prev >> 63);
}

static inline uint64_t east(const uint64_t *row, int k, int w64)  /* column c+1 */
{
    uint64_t x = row[k], nxt = row[(k + 1) % w64];
    return (x >> 1) | (nxt << 63);
}

static void *life_rows(void *arg)
{
    LifeRows *L = arg;
    int w64 = L->w64, h = L->h;
    for (int r = L->r0; r < L->r1; r++) {
        const uint64_t *up = L->cur + (size_t)((r + h - 1) % h) * w64;
        const uint64_t *me = L->cur + (size_t)r * w64;
        const uint64_t *dn = L->cur + (size_t)((r + 1) % h) * w64;
        uint64_t *out = L->next + (size_t)r * w64;
        for (int k = 0; k < w64; k++) {
            uint64_t n[8] = {west(up, k, w64), up[k], east(up, k, w64), west(me, k, w64),
                             east(me, k, w64), west(dn, k, w64), dn[k], east(dn, k, w64)};
            uint64_t b0 = 0, b1 = 0, b2 = 0, b3 = 0;  /* count bits */
            for (int i = 0; i < 8; i++) {
                uint64_t c0 = b0 & n[i];
                b0 ^= n[i];
                uint64_t c1 = b1 & c0;
                b1 ^= c0;
                uint64_t c2 = b2 & c1;
                b2 ^= c1;
                b3 |= c2;
            }
            uint64_t three = b0 & b1 & ~b2 & ~b3, two = ~b0 & b1 & ~b2 & ~b3;
            out[k] = three | (two & me[k]);
        }
    }
    return NULL;
}

void orc_life_words(uint64_t *board, int w64, int h, int gens, int threads)
{
    if (threads < 1)
        threads = 1;
    if (threads > h)
        threads = h;
    uint64_t *tmp = malloc((size_t)w64 * (size_t)h * sizeof *tmp);
    pthread_t *tid = calloc((size_t)threads, sizeof *tid);
    LifeRows *rows = calloc((size_t)threads, sizeof *rows);
    uint64_t *cur = board, *next = tmp;
    for (int g = 0; g < gens; g++) {
        for (int t = 0; t < threads; t++) {
            rows[t] = (LifeRows){cur, next, w64, h, (int)((long)h * t / threads),
                                 (int)((long)h * (t + 1) / threads)};
            pthread_create(&tid[t], NULL, life_rows, &rows[t]);
        }
        for (int t = 0; t < threads; t++)
            pthread_join(tid[t], NULL);
        uint64_t *s = cur;
        cur = next;
        next = s;
    }
    if (cur != board)
        memcpy(board, cur, (size_t)w64 * (size_t)h * sizeof *board);
    free(tmp);
    free(tid);
    free(rows);
}
