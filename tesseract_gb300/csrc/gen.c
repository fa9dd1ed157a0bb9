/* The gate builder and the workload generators, on the host.

   Gates become short NAND/STO runs that leave their result in a cell; a few scratch cells
   (__t0..__t5, made on first use) are shared by all gates; registers take their new value at the
   end of the pass.  The runs are the reference's shortest forms (src/build.c:150-333: LD, LDC,
   the 7-instruction XOR, the 8-instruction mux, the 11-instruction half adder and the
   19-instruction full adder), and the generators place the same gates in the same order as
   src/gen.c and src/tester.c, so every program here is instruction-for-instruction the
   reference's.  That identity is what makes the GPU engine's workloads the reference's
   workloads; the tests pin it against the reference's own output. */
#include <stdlib.h>
#include <string.h>

#include "tc_host.h"

enum { G_BUF, G_NOT, G_AND, G_NAND, G_OR, G_NOR, G_XOR, G_XNOR };

typedef struct {
    Instr    *code;
    size_t    len, cap;
    char    **names;
    CellInfo *info;
    uint32_t  ncells, capcells;
    uint32_t *slots;
    size_t    nslots;
    uint32_t *in, *out, *rq, *rd;
    size_t    nin, capin, nout, capout, nreg, capreg;
    uint32_t  scratch[6];
    int       special;
} Bld;

static uint64_t fnv(const char *s)
{
    uint64_t h = 0xcbf29ce484222325ull;
    for (; *s; s++) {
        unsigned c = (unsigned char)*s;
        if (c >= 'A' && c <= 'Z')
            c += 32;
        h = (h ^ c) * 0x100000001b3ull;
    }
    return h;
}

static size_t bslot(const Bld *b, const char *name)
{
    size_t i = (size_t)fnv(name) & (b->nslots - 1);
    while (b->slots[i] && !tc_same_name(b->names[b->slots[i] - 1], name))
        i = (i + 1) & (b->nslots - 1);
    return i;
}

static void brehash(Bld *b)
{
    free(b->slots);
    b->nslots = b->nslots ? 2 * b->nslots : 1024;
    b->slots = tc_xcalloc(b->nslots, sizeof *b->slots);
    for (uint32_t c = 0; c < b->ncells; c++)
        b->slots[bslot(b, b->names[c])] = c + 1;
}

static uint32_t bcell(Bld *b, const char *name)
{
    size_t i = bslot(b, name);
    if (b->slots[i])
        return b->slots[i] - 1;
    if (b->ncells == b->capcells) {
        b->capcells = b->capcells ? 2 * b->capcells : 64;
        b->names = tc_xrealloc(b->names, b->capcells * sizeof *b->names);
        b->info = tc_xrealloc(b->info, b->capcells * sizeof *b->info);
    }
    uint32_t c = b->ncells++;
    b->names[c] = tc_xstrdup(name);
    memset(&b->info[c], 0, sizeof b->info[c]);
    int d = tc_program_id_name(name);
    if (d >= 0) {
        b->info[c].kind = CK_ID;
        b->info[c].dim = (uint8_t)d;
        b->special = 1;
    }
    b->slots[i] = c + 1;
    if (2 * (size_t)b->ncells > b->nslots)
        brehash(b);
    return c;
}

static uint32_t bcellf(Bld *b, const char *fmt, int i, int j)
{
    char name[64];
    snprintf(name, sizeof name, fmt, i, j);
    return bcell(b, name);
}

/* A name from a format with one number (in a small ring of buffers, for immediate use). */
static const char *bname(Bld *b, const char *fmt, int i)
{
    static __thread char ring[4][48];
    static __thread int at;
    char *s = ring[at++ & 3];
    snprintf(s, 48, fmt, i);
    (void)b;
    return s;
}

static int bhas(const Bld *b, const char *name)
{
    return b->slots[bslot(b, name)] != 0;
}

static uint32_t blink(Bld *b, const char *name, uint32_t src, int dim)
{
    uint32_t c = bcell(b, name);
    b->info[c].kind = CK_LINK;
    b->info[c].dim = (uint8_t)dim;
    b->info[c].src = src;
    b->special = 1;
    return c;
}

static Bld *bnew(void)
{
    Bld *b = tc_xcalloc(1, sizeof *b);
    brehash(b);
    bcell(b, "ZERO");
    bcell(b, "ONE");
    return b;
}

static uint32_t scratch(Bld *b, int i)
{
    if (!b->scratch[i]) {
        char name[8];
        snprintf(name, sizeof name, "__t%d", i);
        b->scratch[i] = bcell(b, name);
    }
    return b->scratch[i];
}

static void push_list(uint32_t **list, size_t *n, size_t *cap, uint32_t v)
{
    if (*n == *cap) {
        *cap = *cap ? 2 * *cap : 64;
        *list = tc_xrealloc(*list, *cap * sizeof **list);
    }
    (*list)[(*n)++] = v;
}

static void binput(Bld *b, uint32_t c) { push_list(&b->in, &b->nin, &b->capin, c); }
static void boutput(Bld *b, uint32_t c) { push_list(&b->out, &b->nout, &b->capout, c); }

static void breg(Bld *b, uint32_t q, uint32_t d)
{
    if (b->nreg == b->capreg) {
        b->capreg = b->capreg ? 2 * b->capreg : 64;
        b->rq = tc_xrealloc(b->rq, b->capreg * sizeof *b->rq);
        b->rd = tc_xrealloc(b->rd, b->capreg * sizeof *b->rd);
    }
    b->rq[b->nreg] = q;
    b->rd[b->nreg++] = d;
}

static void op(Bld *b, int o, uint32_t c)
{
    if (b->len == b->cap) {
        b->cap = b->cap ? 2 * b->cap : 1024;
        b->code = tc_xrealloc(b->code, b->cap * sizeof *b->code);
    }
    b->code[b->len].op = (uint8_t)o;
    b->code[b->len].addr = c;
    b->len++;
}

static void N(Bld *b, uint32_t c) { op(b, OP_NAND, c); }
static void S(Bld *b, uint32_t c) { op(b, OP_STO, c); }
static void load(Bld *b, uint32_t c) { N(b, CELL_ZERO); N(b, c); N(b, CELL_ONE); }   /* RR = c */
static void loadc(Bld *b, uint32_t c) { N(b, CELL_ZERO); N(b, c); }                /* RR = !c */

/* RR = x ^ y (7 instructions, scratch 0) */
static void rr_xor(Bld *b, uint32_t x, uint32_t y)
{
    uint32_t t = scratch(b, 0);
    N(b, CELL_ZERO);
    N(b, x);
    N(b, y);
    S(b, t);
    N(b, y);
    N(b, x);
    N(b, t);
}

static void gate(Bld *b, int type, uint32_t out, const uint32_t *in, int n)
{
    switch (type) {
    case G_BUF:
        load(b, in[0]);
        break;
    case G_NOT:
        loadc(b, in[0]);
        break;
    case G_AND:
    case G_NAND:
        load(b, in[0]);
        for (int i = 1; i < n; i++) {
            N(b, in[i]);
            if (i < n - 1)
                N(b, CELL_ONE);
        }
        if ((n == 1) == (type == G_NAND))
            N(b, CELL_ONE);
        break;
    case G_OR:
    case G_NOR: {
        uint32_t t = scratch(b, 0);
        loadc(b, in[0]);
        for (int i = 1; i < n; i++) {
            if (i > 1)
                N(b, CELL_ONE);
            S(b, t);
            N(b, in[i]);
            N(b, t);
        }
        if ((n == 1) == (type == G_OR))
            N(b, CELL_ONE);
        break;
    }
    default: /* G_XOR, G_XNOR */
        if (n == 1) {
            load(b, in[0]);
        } else {
            uint32_t acc = scratch(b, 2);  /* made before scratch 0, as the reference does */
            rr_xor(b, in[0], in[1]);
            for (int i = 2; i < n; i++) {
                S(b, acc);
                rr_xor(b, acc, in[i]);
            }
        }
        if (type == G_XNOR)
            N(b, CELL_ONE);
        break;
    }
    S(b, out);
}

static void gate2(Bld *b, int type, uint32_t out, uint32_t x, uint32_t y)
{
    uint32_t in[2] = {x, y};
    gate(b, type, out, in, 2);
}

static void gate1(Bld *b, int type, uint32_t out, uint32_t x)
{
    gate(b, type, out, &x, 1);
}

/* s = x ^ y, k = x & y (11 instructions) */
static void half_add(Bld *b, uint32_t s, uint32_t k, uint32_t x, uint32_t y)
{
    uint32_t t = scratch(b, 0);
    N(b, CELL_ZERO);
    N(b, x);
    N(b, y);
    S(b, t);
    N(b, y);
    N(b, CELL_ONE);
    S(b, k);
    N(b, CELL_ONE);
    N(b, x);
    N(b, t);
    S(b, s);
}

/* s = x ^ y ^ c, k = carry (19 instructions); s may be x or y, k may be c */
static void full_add(Bld *b, uint32_t s, uint32_t k, uint32_t x, uint32_t y, uint32_t c)
{
    uint32_t nx = scratch(b, 0);
    uint32_t n = scratch(b, 1);
    uint32_t o = scratch(b, 2);
    uint32_t q = scratch(b, 3);
    N(b, CELL_ZERO);
    N(b, x);
    S(b, nx);
    N(b, CELL_ONE);
    N(b, y);
    S(b, n);
    N(b, y);
    N(b, nx);
    S(b, o);
    N(b, n);
    N(b, c);
    S(b, q);
    N(b, c);
    N(b, n);
    S(b, k);
    N(b, CELL_ONE);
    N(b, o);
    N(b, q);
    S(b, s);
}

/* Registers take their new values at the end of the pass; one whose input is another register's
   output goes through a staging cell __r<i> first (src/build.c:349-371). */
static void bfinish(Bld *b, Program *p)
{
    unsigned char *is_q = tc_xcalloc(b->ncells + 1, 1);
    for (size_t r = 0; r < b->nreg; r++)
        is_q[b->rq[r]] = 1;
    uint32_t *stage = tc_xcalloc(b->nreg + 1, sizeof *stage);
    for (size_t r = 0; r < b->nreg; r++)
        if (is_q[b->rd[r]]) {
            char name[32];
            snprintf(name, sizeof name, "__r%zu", r);
            stage[r] = bcell(b, name);
            load(b, b->rd[r]);
            S(b, stage[r]);
        }
    for (size_t r = 0; r < b->nreg; r++)
        if (!stage[r]) {
            load(b, b->rd[r]);
            S(b, b->rq[r]);
        }
    for (size_t r = 0; r < b->nreg; r++)
        if (stage[r]) {
            load(b, stage[r]);
            S(b, b->rq[r]);
        }
    free(stage);
    free(is_q);
    memset(p, 0, sizeof *p);
    p->code = b->code;
    p->len = b->len;
    p->ncells = b->ncells;
    p->cell_names = b->names;
    p->inputs = b->in;
    p->ninputs = b->nin;
    p->outputs = b->out;
    p->noutputs = b->nout;
    if (b->special)
        p->special = b->info;
    else
        free(b->info);
    free(b->rq);
    free(b->rd);
    free(b->slots);
    free(b);
}

/* ---- the array multiplier (src/gen.c:39-75) ------------------------------------------------ */

/* pc[0 .. 2n-1] = a * bv over n bits: row 0 is a & b0 with the upper half 0; row j adds
   a & bj into pc[j ..] with a half adder at its low end and full adders above, the carry of the
   row going into pc[j + n]. */
static void multiply(Bld *b, const uint32_t *pc, const uint32_t *a, const uint32_t *bv, int n)
{
    uint32_t pp = bcell(b, "pp");
    uint32_t carry = bcell(b, "carry");
    for (int i = 0; i < n; i++)
        gate2(b, G_AND, pc[i], a[i], bv[0]);
    for (int k = n; k < 2 * n; k++)
        gate1(b, G_BUF, pc[k], CELL_ZERO);
    for (int j = 1; j < n; j++)
        for (int i = 0; i < n; i++) {
            gate2(b, G_AND, pp, a[i], bv[j]);
            if (i == 0)
                half_add(b, pc[j], carry, pc[j], pp);
            else
                full_add(b, pc[i + j], i == n - 1 ? pc[j + n] : carry, pc[i + j], pp, carry);
        }
}

void tc_gen_mul(Program *p, int n)
{
    Bld *b = bnew();
    uint32_t *a = tc_xmalloc((size_t)n * sizeof *a), *bv = tc_xmalloc((size_t)n * sizeof *bv);
    uint32_t *pc = tc_xmalloc(2 * (size_t)n * sizeof *pc);
    for (int i = 0; i < n; i++)
        binput(b, a[i] = bcellf(b, "a%d", i, 0));
    for (int i = 0; i < n; i++)
        binput(b, bv[i] = bcellf(b, "b%d", i, 0));
    for (int k = 0; k < 2 * n; k++)
        pc[k] = bcellf(b, "p%d", k, 0);
    multiply(b, pc, a, bv, n);
    for (int k = 0; k < 2 * n; k++)
        boutput(b, pc[k]);
    bfinish(b, p);
    free(a);
    free(bv);
    free(pc);
}

/* ---- the toy hash (src/gen.c:77-160) -------------------------------------------------------- */

static int coprime_step(int n)
{
    static const int m[] = {5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61};
    for (size_t i = 0; i < sizeof m / sizeof m[0]; i++) {
        int x = m[i], y = n;
        while (y) {
            int t = x % y;
            x = y;
            y = t;
        }
        if (x == 1)
            return m[i];
    }
    return 0;
}

static uint64_t round_key(int r, int bits)
{
    uint64_t s = (uint64_t)r * 0x9E3779B97F4A7C15ull;  /* splitmix64 of state r: output r + 1 */
    uint64_t z = tc_splitmix64(&s);
    return bits == 64 ? z : z & ((1ull << bits) - 1);
}

uint64_t tc_toyhash(uint64_t x, int n, int rounds)
{
    int m = coprime_step(n);
    for (int r = 0; r < rounds; r++) {
        uint64_t y = 0, z = 0;
        for (int i = 0; i < n; i++) {
            uint64_t xi = (x >> i) & 1, x1 = (x >> ((i + 1) % n)) & 1, x2 = (x >> ((i + 2) % n)) & 1;
            y |= (xi ^ (~x1 & x2 & 1)) << i;
        }
        for (int i = 0; i < n; i++)
            z |= ((y >> ((m * i + 3) % n)) & 1) << i;
        x = z ^ round_key(r, n);
    }
    return x;
}

int tc_gen_hash(Program *p, int n, int rounds)
{
    int m = coprime_step(n);
    if (!m)
        return 0;
    Bld *b = bnew();
    uint32_t *cur = tc_xmalloc((size_t)n * sizeof *cur), *nxt = tc_xmalloc((size_t)n * sizeof *nxt);
    for (int i = 0; i < n; i++)
        binput(b, cur[i] = bcellf(b, "x%d", i, 0));
    uint32_t nt = bcell(b, "nt");
    uint32_t tt = bcell(b, "tt");
    for (int r = 0; r < rounds; r++) {
        int bank = r % 2;
        uint64_t rc = round_key(r, n);
        for (int i = 0; i < n; i++) {
            uint32_t y = bcellf(b, "y%d_%d", bank, i);
            gate1(b, G_NOT, nt, cur[(i + 1) % n]);
            gate2(b, G_AND, tt, nt, cur[(i + 2) % n]);
            gate2(b, G_XOR, y, cur[i], tt);
        }
        for (int i = 0; i < n; i++) {
            uint32_t src = bcellf(b, "y%d_%d", bank, (m * i + 3) % n);
            if ((rc >> i) & 1) {
                nxt[i] = bcellf(b, "k%d_%d", bank, i);
                gate1(b, G_NOT, nxt[i], src);
            } else {
                nxt[i] = src;
            }
        }
        memcpy(cur, nxt, (size_t)n * sizeof *cur);
    }
    for (int i = 0; i < n; i++) {
        uint32_t h = bcellf(b, "h%d", i, 0);
        gate1(b, G_BUF, h, cur[i]);
        boutput(b, h);
    }
    bfinish(b, p);
    free(cur);
    free(nxt);
    return 1;
}

/* ---- Game of Life (src/gen.c:163-319) ------------------------------------------------------- */

/* One generation on the w x h board (registers); halo[(r + 1) * (w + 2) + c + 1] is the cell at
   row r, column c for r = -1 .. h, c = -1 .. w.  Neighbour count by full and half adders, then
   alive = c1 & (c0 | self) & !(u | v). */
static void life_generation(Bld *b, const uint32_t *board, const uint32_t *halo, int w, int h)
{
    static const char *const nm[14] = {"s0", "k0", "s1", "k1", "s2", "k2", "c0",
                                       "k3", "t",  "u",  "c1", "v",  "r1", "r2"};
    uint32_t x[14];
    for (int i = 0; i < 14; i++)
        x[i] = bcell(b, nm[i]);
    uint32_t s0 = x[0], k0 = x[1], s1 = x[2], k1 = x[3], s2 = x[4], k2 = x[5], c0 = x[6], k3 = x[7],
             t = x[8], u = x[9], c1 = x[10], v = x[11], r1 = x[12], r2 = x[13];
    for (int r = 0; r < h; r++)
        for (int c = 0; c < w; c++) {
            uint32_t nb[8];
            int k = 0;
            for (int dr = -1; dr <= 1; dr++)
                for (int dc = -1; dc <= 1; dc++)
                    if (dr || dc)
                        nb[k++] = halo[(r + 1 + dr) * (w + 2) + c + 1 + dc];
            full_add(b, s0, k0, nb[0], nb[1], nb[2]);
            full_add(b, s1, k1, nb[3], nb[4], nb[5]);
            half_add(b, s2, k2, nb[6], nb[7]);
            full_add(b, c0, k3, s0, s1, s2);
            full_add(b, t, u, k0, k1, k2);
            half_add(b, c1, v, t, k3);
            uint32_t self = board[r * w + c];
            uint32_t next = bcellf(b, "n%d_%d", r, c);
            uint32_t all[3] = {c1, r1, r2};
            gate2(b, G_OR, r1, c0, self);
            gate2(b, G_NOR, r2, u, v);
            gate(b, G_AND, next, all, 3);
            breg(b, self, next);
        }
}

static uint32_t *board_and_halo(Bld *b, int w, int h, uint32_t *board)
{
    for (int r = 0; r < h; r++)
        for (int c = 0; c < w; c++)
            board[r * w + c] = bcellf(b, "x%d_%d", r, c);
    return tc_xmalloc((size_t)(w + 2) * (size_t)(h + 2) * sizeof(uint32_t));
}

void tc_gen_life(Program *p, int w, int h, uint32_t *board)
{
    Bld *b = bnew();
    uint32_t *halo = board_and_halo(b, w, h, board);
    for (int r = -1; r <= h; r++)
        for (int c = -1; c <= w; c++)
            halo[(r + 1) * (w + 2) + c + 1] = board[((r + h) % h) * w + (c + w) % w];
    life_generation(b, board, halo, w, h);
    free(halo);
    bfinish(b, p);
}

unsigned tc_grid_machine(unsigned row, unsigned col, int cbits)
{
    return (row ^ row >> 1) << cbits | (col ^ col >> 1);
}

/* Masks for a Gray-coded axis over dimensions lo .. lo+k-1: next[j] (prev[j]) is 1 in machines
   whose next (previous) position is across dimension lo + j (src/gen.c:214-253). */
static void axis_masks(Bld *b, int lo, int k, uint32_t *next, uint32_t *prev, const char *tag)
{
    char name[32];
    uint32_t id[CUBE_MAX_DIMS], v[4];
    for (int j = 0; j < k; j++) {
        id[j] = bcellf(b, "ID%d", lo + j, 0);
        snprintf(name, sizeof name, "%s_n%d", tag, j);
        next[j] = bcell(b, name);
        snprintf(name, sizeof name, "%s_v%d", tag, j);
        prev[j] = bcell(b, name);
    }
    for (int i = 0; i < 4; i++) {
        snprintf(name, sizeof name, "%s_%c", tag, "pqol"[i]);
        v[i] = bcell(b, name);
    }
    uint32_t odd = v[0], even = v[1], below = v[2], low = v[3];
    gate(b, G_XOR, odd, id, k);
    gate1(b, G_NOT, even, odd);
    gate1(b, G_BUF, next[0], even);
    gate1(b, G_BUF, prev[0], odd);
    gate1(b, G_BUF, below, CELL_ZERO);
    for (int j = 0; j < k; j++) {
        gate1(b, G_NOT, low, below);
        gate2(b, G_AND, low, low, id[j]);
        if (j + 1 < k) {
            gate2(b, G_AND, next[j + 1], low, odd);
            gate2(b, G_AND, prev[j + 1], low, even);
        } else {
            gate2(b, G_AND, low, low, odd);
            gate2(b, G_OR, next[j], next[j], low);
        }
        gate2(b, G_OR, below, below, id[j]);
    }
    gate1(b, G_NOT, low, below);
    gate2(b, G_OR, prev[k - 1], prev[k - 1], low);
}

/* New cell `name` = src of the machine mask[0..k-1] points to across lo .. lo+k-1. */
static uint32_t axis_gather(Bld *b, const char *name, uint32_t src, int lo, int k,
                            const uint32_t *mask)
{
    uint32_t t[CUBE_MAX_DIMS];
    uint32_t out = bcell(b, name);
    char lname[48];
    for (int j = 0; j < k; j++) {
        snprintf(lname, sizeof lname, "lk%u_%d", (unsigned)src, lo + j);
        uint32_t l = bhas(b, lname) ? bcell(b, lname) : blink(b, lname, src, lo + j);
        t[j] = bcellf(b, "gt%d", j, 0);
        gate2(b, G_NAND, t[j], mask[j], l);
    }
    gate(b, G_NAND, out, t, k);
    return out;
}

void tc_gen_life_cube(Program *p, int w, int h, int rbits, int cbits, uint32_t *board)
{
    Bld *b = bnew();
    int W = w + 2;
    uint32_t *halo = board_and_halo(b, w, h, board);
    uint32_t right[CUBE_MAX_DIMS], left[CUBE_MAX_DIMS], down[CUBE_MAX_DIMS], up[CUBE_MAX_DIMS];
    char name[32];
    if (cbits)
        axis_masks(b, 0, cbits, right, left, "gc");
    if (rbits)
        axis_masks(b, cbits, rbits, down, up, "gr");
    for (int r = 0; r < h; r++)
        for (int c = 0; c < w; c++)
            halo[(r + 1) * W + c + 1] = board[r * w + c];
    for (int r = 0; r < h; r++) {
        uint32_t last = board[r * w + w - 1], first = board[r * w];
        snprintf(name, sizeof name, "hw%d", r);
        halo[(r + 1) * W] = cbits ? axis_gather(b, name, last, 0, cbits, left) : last;
        snprintf(name, sizeof name, "he%d", r);
        halo[(r + 1) * W + w + 1] = cbits ? axis_gather(b, name, first, 0, cbits, right) : first;
    }
    for (int c = 0; c < W; c++) {
        uint32_t last = halo[h * W + c], first = halo[W + c];
        snprintf(name, sizeof name, "hn%d", c);
        halo[c] = rbits ? axis_gather(b, name, last, cbits, rbits, up) : last;
        snprintf(name, sizeof name, "hs%d", c);
        halo[(h + 1) * W + c] = rbits ? axis_gather(b, name, first, cbits, rbits, down) : first;
    }
    life_generation(b, board, halo, w, h);
    free(halo);
    bfinish(b, p);
}

/* ---- cube demos (the big-cube demos of src/cubedemo.c:398-623) ------------------------------

   The reference builds these from its assembly library (lib/cube.inc: OR_DIM, CMPX8, ...) and
   checks them against plain C; here they are built with the same gate builder from the same
   algorithms, and checked against plain C the same way.  Every step reads its neighbours across
   one dimension into cells of its own before it writes anything, because all machines run each
   instruction together (lockstep): a link read sees the neighbour's cell as it is at that
   instruction. */

/* r = OR of x over all 2^dims machines: r = x, then r |= r across each dimension. */
void tc_gen_cube_any(Program *p, int dims)
{
    Bld *b = bnew();
    uint32_t x = bcell(b, "x"), r = bcell(b, "r");
    binput(b, x);
    boutput(b, r);
    gate1(b, G_BUF, r, x);
    for (int d = 0; d < dims; d++) {
        uint32_t l = blink(b, bname(b, "lr%d", d), r, d);
        gate2(b, G_OR, r, r, l);
    }
    bfinish(b, p);
}

/* b-bit ripple add: s += a (cells s[0..n-1], a[0..n-1]); carry is a scratch cell. */
static void add_into(Bld *b, const uint32_t *s, const uint32_t *a, int n, uint32_t carry)
{
    half_add(b, s[0], carry, s[0], a[0]);
    for (int i = 1; i < n; i++)
        full_add(b, s[i], carry, s[i], a[i], carry);
}

/* p = how many machines below k have x = 1, t = how many have it in all (dims + 1 bits each,
   bit 0 first): the hypercube prefix sum.  Each machine keeps t, the count of its subcube so
   far; across dimension d it reads the neighbour's t, adds it to t, and to p when bit d of the
   machine number is 1 (the neighbour holds the lower half). */
static void prefix_count(Bld *b, uint32_t x, const uint32_t *pv, const uint32_t *tv, int dims)
{
    int n = dims + 1;
    uint32_t carry = bcell(b, "cy"), nb[CUBE_MAX_DIMS + 1], ad[CUBE_MAX_DIMS + 1];
    for (int i = 0; i < n; i++) {
        nb[i] = bcell(b, bname(b, "n%d", i));
        ad[i] = bcell(b, bname(b, "m%d", i));
        gate1(b, G_BUF, pv[i], CELL_ZERO);
        gate1(b, G_BUF, tv[i], i == 0 ? x : CELL_ZERO);
    }
    for (int d = 0; d < dims; d++) {
        uint32_t id = bcell(b, bname(b, "ID%d", d));
        int w = d + 1 < n ? d + 1 : n;  /* a subcube of 2^d machines counts to 2^d: d + 1 bits */
        for (int i = 0; i < w; i++) {
            char ln[32];
            snprintf(ln, sizeof ln, "lt%d_%d", i, d);
            gate1(b, G_BUF, nb[i], blink(b, ln, tv[i], d));
        }
        for (int i = w; i < n; i++)
            gate1(b, G_BUF, nb[i], CELL_ZERO);
        for (int i = 0; i < n; i++)
            gate2(b, G_AND, ad[i], nb[i], id);
        add_into(b, pv, ad, n, carry);
        add_into(b, tv, nb, n, carry);
    }
}

void tc_gen_cube_rank(Program *p, int dims)
{
    Bld *b = bnew();
    int n = dims + 1;
    uint32_t x = bcell(b, "x"), pv[CUBE_MAX_DIMS + 1], tv[CUBE_MAX_DIMS + 1];
    binput(b, x);
    for (int i = 0; i < n; i++)
        pv[i] = bcell(b, bname(b, "p%d", i));
    for (int i = 0; i < n; i++)
        tv[i] = bcell(b, bname(b, "t%d", i));
    for (int i = 0; i < n; i++)
        boutput(b, pv[i]);
    for (int i = 0; i < n; i++)
        boutput(b, tv[i]);
    prefix_count(b, x, pv, tv, dims);
    bfinish(b, p);
}

/* x = sel ? y : x, one bit (x ^= (x ^ y) & sel); t is a scratch cell */
static void take_if(Bld *b, uint32_t x, uint32_t y, uint32_t sel, uint32_t t)
{
    gate2(b, G_XOR, t, x, y);
    gate2(b, G_AND, t, t, sel);
    gate2(b, G_XOR, x, x, t);
}

/* The machines with h = 1 hand their bytes v0..v7 to the first machines, in machine order:
   afterwards machine k holds h = 1 and the byte of the k-th such machine when k is below their
   number, h = 0 otherwise.  A byte's destination is its machine's prefix count p.  Bytes move
   across dimension 0, 1, .., dims - 1 in turn, crossing d when bit d of where they are differs
   from bit d of p, and two never meet: after dimension d a byte sits at p's bits 0..d and its
   start's bits above d; two starts that agree above bit d are less than 2^(d+1) apart, so are
   their prefix counts, which then differ in bits 0..d. */
void tc_gen_cube_pack(Program *p, int dims)
{
    Bld *b = bnew();
    int n = dims + 1;
    uint32_t v[8], nv[8], pv[CUBE_MAX_DIMS + 1], tv[CUBE_MAX_DIMS + 1], np[CUBE_MAX_DIMS + 1];
    for (int i = 0; i < 8; i++)
        v[i] = bcell(b, bname(b, "v%d", i));
    uint32_t h = bcell(b, "h");
    for (int i = 0; i < 8; i++)
        binput(b, v[i]);
    binput(b, h);
    for (int i = 0; i < 8; i++)
        boutput(b, v[i]);
    boutput(b, h);
    for (int i = 0; i < n; i++)
        pv[i] = bcell(b, bname(b, "p%d", i));
    for (int i = 0; i < n; i++)
        tv[i] = bcell(b, bname(b, "t%d", i));
    prefix_count(b, h, pv, tv, dims);
    for (int i = 0; i < 8; i++)
        nv[i] = bcell(b, bname(b, "u%d", i));
    for (int i = 0; i < n; i++)
        np[i] = bcell(b, bname(b, "q%d", i));
    uint32_t go = bcell(b, "go"), ngo = bcell(b, "ngo"), stay = bcell(b, "stay"),
             t = bcell(b, "tk");
    for (int d = 0; d < dims; d++) {
        /* this machine's byte leaves across d */
        gate2(b, G_XOR, go, pv[d], bcell(b, bname(b, "ID%d", d)));
        gate2(b, G_AND, go, go, h);
        /* every read of the neighbour before anything it reads is changed */
        gate1(b, G_BUF, ngo, blink(b, bname(b, "lg%d", d), go, d));
        for (int i = 0; i < 8; i++) {
            char ln[32];
            snprintf(ln, sizeof ln, "lv%d_%d", i, d);
            gate1(b, G_BUF, nv[i], blink(b, ln, v[i], d));
        }
        for (int j = d + 1; j < dims; j++) {
            char ln[32];
            snprintf(ln, sizeof ln, "lp%d_%d", j, d);
            gate1(b, G_BUF, np[j], blink(b, ln, pv[j], d));
        }
        /* a byte that stays keeps its place; otherwise the neighbour's, if it crosses, arrives */
        gate2(b, G_XOR, stay, h, go);  /* go implies h: h and not go */
        for (int i = 0; i < 8; i++)
            take_if(b, v[i], nv[i], ngo, t);
        for (int j = d + 1; j < dims; j++)
            take_if(b, pv[j], np[j], ngo, t);
        gate2(b, G_OR, h, stay, ngo);
    }
    bfinish(b, p);
}

/* Bitonic sort of one 8-bit value per machine (v0..v7, bit 0 first): afterwards machine k holds
   the k-th smallest.  Stage st = 1 .. dims sorts blocks of 2^st machines, up or down by bit st
   of the machine number (the last stage up); each step compare-exchanges across dimension j:
   the machine with bit j = 0 keeps the smaller value, unless the direction bit is 1. */
void tc_gen_cube_sort(Program *p, int dims)
{
    Bld *b = bnew();
    uint32_t v[8], o[8], nv[8];
    for (int i = 0; i < 8; i++)
        v[i] = bcell(b, bname(b, "v%d", i));
    for (int i = 0; i < 8; i++)
        binput(b, v[i]);
    for (int i = 0; i < 8; i++)
        boutput(b, v[i]);
    for (int i = 0; i < 8; i++) {
        o[i] = bcell(b, bname(b, "o%d", i));
        nv[i] = bcell(b, bname(b, "w%d", i));
    }
    uint32_t carry = bcell(b, "cy"), sum = bcell(b, "sm"), keep = bcell(b, "km"),
             sel = bcell(b, "se"), dif = bcell(b, "df");
    for (int st = 1; st <= dims; st++)
        for (int j = st - 1; j >= 0; j--) {
            uint32_t idj = bcell(b, bname(b, "ID%d", j));
            uint32_t dir = st < dims ? bcell(b, bname(b, "ID%d", st)) : CELL_ZERO;
            for (int i = 0; i < 8; i++) {
                char ln[32];
                snprintf(ln, sizeof ln, "lv%d_%d", i, j);
                uint32_t l = bhas(b, ln) ? bcell(b, ln) : blink(b, ln, v[i], j);
                gate1(b, G_BUF, o[i], l);
            }
            /* carry out of o + ~v + 1 is (o >= v): o < v is its complement */
            gate1(b, G_BUF, carry, CELL_ONE);
            for (int i = 0; i < 8; i++) {
                gate1(b, G_NOT, nv[i], v[i]);
                full_add(b, sum, carry, o[i], nv[i], carry);
            }
            /* take o when keeping the minimum and o < v, or keeping the maximum and o >= v */
            gate2(b, G_XNOR, keep, idj, dir);
            gate2(b, G_XOR, sel, keep, carry);
            for (int i = 0; i < 8; i++) {
                gate2(b, G_XOR, dif, o[i], v[i]);
                gate2(b, G_AND, dif, dif, sel);
                gate2(b, G_XOR, v[i], v[i], dif);
            }
        }
    bfinish(b, p);
}

/* m = the largest byte v (v0..v7) over all machines: m = v, then m = max(m, m across d) for
   every dimension. */
void tc_gen_cube_max(Program *p, int dims)
{
    Bld *b = bnew();
    uint32_t v[8], m[8], o[8], nm[8];
    for (int i = 0; i < 8; i++)
        binput(b, v[i] = bcell(b, bname(b, "v%d", i)));
    for (int i = 0; i < 8; i++)
        boutput(b, m[i] = bcell(b, bname(b, "m%d", i)));
    for (int i = 0; i < 8; i++) {
        o[i] = bcell(b, bname(b, "o%d", i));
        nm[i] = bcell(b, bname(b, "nm%d", i));
        gate1(b, G_BUF, m[i], v[i]);
    }
    uint32_t carry = bcell(b, "cy"), sum = bcell(b, "sm"), dif = bcell(b, "df");
    for (int d = 0; d < dims; d++) {
        for (int i = 0; i < 8; i++) {
            char ln[32];
            snprintf(ln, sizeof ln, "lm%d_%d", i, d);
            gate1(b, G_BUF, o[i], blink(b, ln, m[i], d));
        }
        /* carry out of o + ~m + 1 is (o >= m): take o then */
        gate1(b, G_BUF, carry, CELL_ONE);
        for (int i = 0; i < 8; i++) {
            gate1(b, G_NOT, nm[i], m[i]);
            full_add(b, sum, carry, o[i], nm[i], carry);
        }
        for (int i = 0; i < 8; i++) {
            gate2(b, G_XOR, dif, o[i], m[i]);
            gate2(b, G_AND, dif, dif, carry);
            gate2(b, G_XOR, m[i], m[i], dif);
        }
    }
    bfinish(b, p);
}

/* f (one bit per machine, machine k holding f(k)) becomes its algebraic normal form, the
   Möbius transform over GF(2): across each dimension d the machines with bit d set XOR in f of
   the machine below. */
void tc_gen_cube_anf(Program *p, int dims)
{
    Bld *b = bnew();
    uint32_t f = bcell(b, "f"), t = bcell(b, "mt");
    binput(b, f);
    boutput(b, f);
    for (int d = 0; d < dims; d++) {
        gate2(b, G_AND, t, blink(b, bname(b, "lf%d", d), f, d), bcell(b, bname(b, "ID%d", d)));
        gate2(b, G_XOR, f, f, t);
    }
    bfinish(b, p);
}

/* The Walsh-Hadamard transform of the n-bit two's complement numbers w (bit 0 first, arithmetic
   mod 2^n) over all dims dimensions: across each dimension the machine below takes a + a', the one
   above a' - a (its own value subtracted from the one below).  Scratch and link cells are named
   after `tag`. */
static void spectrum(Bld *b, const uint32_t *w, int n, int dims, const char *tag)
{
    uint32_t o[2 * CUBE_MAX_DIMS + 4], y[2 * CUBE_MAX_DIMS + 4];
    char fo[16], fy[16], fl[16];
    snprintf(fo, sizeof fo, "%so%%d", tag);
    snprintf(fy, sizeof fy, "%sy%%d", tag);
    snprintf(fl, sizeof fl, "l%s%%d_%%d", tag[0] ? tag : "w");
    for (int i = 0; i < n; i++) {
        o[i] = bcell(b, bname(b, fo, i));
        y[i] = bcell(b, bname(b, fy, i));
    }
    uint32_t carry = bcell(b, "cy");
    for (int d = 0; d < dims; d++) {
        uint32_t id = bcell(b, bname(b, "ID%d", d));
        for (int i = 0; i < n; i++) {
            char ln[32];
            snprintf(ln, sizeof ln, fl, i, d);
            gate1(b, G_BUF, o[i], blink(b, ln, w[i], d));
        }
        /* below (id 0): w + o; above (id 1): o - w = o + ~w + 1 */
        for (int i = 0; i < n; i++)
            gate2(b, G_XOR, y[i], w[i], id);
        gate1(b, G_BUF, carry, id);
        for (int i = 0; i < n; i++)
            full_add(b, w[i], carry, o[i], y[i], carry);
    }
}

/* w = the Walsh-Hadamard spectrum of f: w(k) = sum over j of (-1)^(f(j) + j.k), dims + 3 bits in
   two's complement (bit 0 first), starting from 1 - 2 f(k). */
void tc_gen_cube_walsh(Program *p, int dims)
{
    Bld *b = bnew();
    int n = dims + 3;
    uint32_t f = bcell(b, "f"), w[CUBE_MAX_DIMS + 3];
    binput(b, f);
    for (int i = 0; i < n; i++)
        boutput(b, w[i] = bcell(b, bname(b, "w%d", i)));
    /* 1 - 2f: f = 0 gives 1 (bit 0 set), f = 1 gives -1 (all bits set) */
    gate1(b, G_BUF, w[0], CELL_ONE);
    for (int i = 1; i < n; i++)
        gate1(b, G_BUF, w[i], f);
    spectrum(b, w, n, dims, "");
    bfinish(b, p);
}

/* h(k) = how many j have f(j) = g(j ^ k) = 1, the XOR convolution of f and g, by spectra: the
   transform of the convolution is the product of the transforms F and G, and transforming it
   again gives 2^dims h.  The arithmetic is mod 2^(2 dims + 2), which holds 2^dims h <= 2^(2 dims)
   exactly; h has dims + 1 bits. */
void tc_gen_cube_xorconv(Program *p, int dims)
{
    Bld *b = bnew();
    int n = 2 * dims + 2;
    uint32_t f = bcell(b, "f"), g = bcell(b, "g"), fw[2 * CUBE_MAX_DIMS + 2],
             gw[2 * CUBE_MAX_DIMS + 2], pw[2 * CUBE_MAX_DIMS + 2];
    binput(b, f);
    binput(b, g);
    for (int i = 0; i <= dims; i++)
        boutput(b, bcell(b, bname(b, "h%d", i)));
    for (int i = 0; i < n; i++) {
        gate1(b, G_BUF, fw[i] = bcell(b, bname(b, "F%d", i)), i == 0 ? f : CELL_ZERO);
        gate1(b, G_BUF, gw[i] = bcell(b, bname(b, "G%d", i)), i == 0 ? g : CELL_ZERO);
        pw[i] = bcell(b, bname(b, "P%d", i));
    }
    spectrum(b, fw, n, dims, "F");
    spectrum(b, gw, n, dims, "G");
    /* pw = fw gw mod 2^n: row j of the schoolbook product added into bits j.. */
    uint32_t pp = bcell(b, "pp"), carry = bcell(b, "mc");
    for (int k = 0; k < n; k++)
        gate2(b, G_AND, pw[k], fw[k], gw[0]);
    for (int j = 1; j < n; j++)
        for (int k = j; k < n; k++) {
            gate2(b, G_AND, pp, fw[k - j], gw[j]);
            if (k == j)
                half_add(b, pw[k], carry, pw[k], pp);
            else
                full_add(b, pw[k], carry, pw[k], pp, carry);
        }
    spectrum(b, pw, n, dims, "P");
    for (int i = 0; i <= dims; i++)  /* divided by 2^dims */
        gate1(b, G_BUF, bcell(b, bname(b, "h%d", i)), pw[dims + i]);
    bfinish(b, p);
}

/* Rule 110 on the machines as a ring, position i being machine gray(i): one step,
   x' = (x | right) & ~(left & x & right), the neighbours gathered over the Gray-coded axis as
   the Life board's edges are. */
void tc_gen_cube_ring(Program *p, int dims)
{
    Bld *b = bnew();
    uint32_t x = bcell(b, "x"), next[CUBE_MAX_DIMS], prev[CUBE_MAX_DIMS];
    binput(b, x);
    boutput(b, x);
    axis_masks(b, 0, dims, next, prev, "rg");
    uint32_t left = axis_gather(b, "left", x, 0, dims, prev);
    uint32_t right = axis_gather(b, "right", x, 0, dims, next);
    uint32_t all3 = bcell(b, "all3"), in3[3] = {x, left, right}, t = bcell(b, "or");
    gate(b, G_AND, all3, in3, 3);
    gate2(b, G_OR, t, x, right);
    gate1(b, G_NOT, all3, all3);
    gate2(b, G_AND, x, t, all3);
    bfinish(b, p);
}

/* ---- polynomial product mod x^N + 1 over Z_q by the number-theoretic transform ---------------

   The cube's 2^dims machines hold the coefficients (dims 9..11: q - 1 = 3 * 2^12 allows a
   2N-th root of unity for N up to 2^11).  Numbers mod q take 14 bits.  Products use Montgomery
   reduction with R = 2^14: montmul(x, y) = x y / R mod q, so twiddles given times R come out
   as plain products.  The algorithm is the textbook negacyclic NTT: Cooley-Tukey butterflies
   forward (dimension dims-1 down to 0), the product point by point, Gentleman-Sande butterflies
   back (dimension 0 up), and one last product by R^2 / N. */

enum { NQ = 12289, NQB = 14 };

/* out = x + y + cin over n bits (cin a cell); out may be x or y */
static void add_bits(Bld *b, const uint32_t *out, const uint32_t *x, const uint32_t *y,
                     uint32_t cin, int n, uint32_t carry)
{
    gate1(b, G_BUF, carry, cin);
    for (int i = 0; i < n; i++)
        full_add(b, out[i], carry, x[i], y[i], carry);
}

/* out = sel ? x1 : x0 over n bits; out may be x0 or x1 */
static void mux_bits(Bld *b, const uint32_t *out, uint32_t sel, const uint32_t *x1,
                     const uint32_t *x0, int n, uint32_t t)
{
    for (int i = 0; i < n; i++) {
        gate2(b, G_XOR, t, x0[i], x1[i]);
        gate2(b, G_AND, t, t, sel);
        gate2(b, G_XOR, out[i], x0[i], t);
    }
}

static void const_bits(uint32_t *out, uint64_t v, int n)
{
    for (int i = 0; i < n; i++)
        out[i] = (v >> i) & 1 ? CELL_ONE : CELL_ZERO;
}

/* u = v mod q for v < 2q on 15 bits, into r (14 bits): v - q when it does not borrow */
static void reduce_q(Bld *b, const uint32_t *r, const uint32_t *v, uint32_t carry)
{
    uint32_t k[15], d[15], mt = bcell(b, "nq_t");
    for (int i = 0; i < 15; i++)
        d[i] = bcell(b, bname(b, "nq_d%d", i));
    const_bits(k, 32768 - NQ, 15);
    add_bits(b, d, v, k, CELL_ZERO, 15, carry);  /* carry out: v >= q */
    mux_bits(b, r, carry, d, v, NQB, mt);
}

/* r = x y / R mod q (x, y, r in 0 .. q-1; r may be x or y) */
static void montmul(Bld *b, const uint32_t *r, const uint32_t *x, const uint32_t *y)
{
    uint32_t t[30], sm[NQB], m[NQB], ns[NQB], z[NQB], sh[30], u[15];
    uint32_t carry = bcell(b, "mm_c"), k = bcell(b, "mm_k");
    for (int i = 0; i < 30; i++)
        t[i] = bcell(b, bname(b, "mm_t%d", i));
    for (int i = 0; i < NQB; i++) {
        sm[i] = bcell(b, bname(b, "mm_s%d", i));
        m[i] = bcell(b, bname(b, "mm_m%d", i));
        ns[i] = bcell(b, bname(b, "mm_n%d", i));
    }
    multiply(b, t, x, y, NQB);  /* t = x y < q^2 < 2^28 */
    gate1(b, G_BUF, t[28], CELL_ZERO);
    gate1(b, G_BUF, t[29], CELL_ZERO);
    /* m = -t / q mod R: 1/q = 2^12 + 1 mod 2^14, so m = -(t + (t << 12)) mod 2^14 */
    for (int i = 0; i < 12; i++)
        gate1(b, G_BUF, sm[i], t[i]);
    gate2(b, G_XOR, sm[12], t[12], t[0]);
    gate2(b, G_AND, k, t[12], t[0]);
    gate2(b, G_XOR, sm[13], t[13], t[1]);
    gate2(b, G_XOR, sm[13], sm[13], k);
    for (int i = 0; i < NQB; i++)
        gate1(b, G_NOT, ns[i], sm[i]);
    const_bits(z, 0, NQB);
    add_bits(b, m, ns, z, CELL_ONE, NQB, carry);
    /* t += m q = m + (m << 12) + (m << 13); t is then a multiple of R */
    for (int sft = 0; sft <= 13; sft += sft == 0 ? 12 : 1) {
        for (int i = 0; i < 30; i++)
            sh[i] = i >= sft && i < sft + NQB ? m[i - sft] : CELL_ZERO;
        add_bits(b, t, t, sh, CELL_ZERO, 30, carry);
    }
    for (int i = 0; i < 15; i++)
        u[i] = t[NQB + i];  /* (t + m q) / R < 2q */
    reduce_q(b, r, u, carry);
}

/* out = sel ? x - y : x + y, mod q (all in 0 .. q-1); out may be x or y */
static void addsub_q(Bld *b, const uint32_t *out, uint32_t sel, const uint32_t *x,
                     const uint32_t *y)
{
    uint32_t q[15], ny[15], neg[15], y2[15], x15[15], s[15], carry = bcell(b, "as_c"),
             mt = bcell(b, "as_t");
    for (int i = 0; i < 15; i++) {
        ny[i] = bcell(b, bname(b, "as_n%d", i));
        neg[i] = bcell(b, bname(b, "as_g%d", i));
        y2[i] = bcell(b, bname(b, "as_y%d", i));
        s[i] = bcell(b, bname(b, "as_s%d", i));
        x15[i] = i < NQB ? x[i] : CELL_ZERO;
    }
    const_bits(q, NQ, 15);
    for (int i = 0; i < 15; i++)
        gate1(b, G_NOT, ny[i], i < NQB ? y[i] : CELL_ZERO);
    add_bits(b, neg, q, ny, CELL_ONE, 15, carry);  /* q - y, in 1 .. q */
    for (int i = 0; i < 15; i++)
        gate1(b, G_BUF, y2[i], i < NQB ? y[i] : CELL_ZERO);
    mux_bits(b, y2, sel, neg, y2, 15, mt);
    add_bits(b, s, x15, y2, CELL_ZERO, 15, carry);  /* below 2q */
    reduce_q(b, out, s, carry);
}

/* c = a b mod (x^N + 1, q), N = 2^dims; inputs a, b, and per dimension d the twiddles zf<d>_,
   zi<d>_ (14 bits each, times R mod q) that cuda_cube_demo's polymul computes */
void tc_gen_cube_polymul(Program *p, int dims)
{
    Bld *b = bnew();
    uint32_t a[NQB], bv[NQB], c[NQB], wa[NQB], wb[NQB], f[NQB], x[NQB], y[NQB], t[NQB];
    uint32_t zf[CUBE_MAX_DIMS][NQB], zi[CUBE_MAX_DIMS][NQB], la[NQB], lt[NQB];
    for (int i = 0; i < NQB; i++)
        binput(b, a[i] = bcell(b, bname(b, "a%d", i)));
    for (int i = 0; i < NQB; i++)
        binput(b, bv[i] = bcell(b, bname(b, "b%d", i)));
    char name[48];
    for (int d = 0; d < dims; d++)
        for (int i = 0; i < NQB; i++) {
            snprintf(name, sizeof name, "zf%d_%d", d, i);
            binput(b, zf[d][i] = bcell(b, name));
        }
    for (int d = 0; d < dims; d++)
        for (int i = 0; i < NQB; i++) {
            snprintf(name, sizeof name, "zi%d_%d", d, i);
            binput(b, zi[d][i] = bcell(b, name));
        }
    for (int i = 0; i < NQB; i++) {
        c[i] = bcell(b, bname(b, "c%d", i));
        wa[i] = bcell(b, bname(b, "wa%d", i));
        wb[i] = bcell(b, bname(b, "wb%d", i));
        x[i] = bcell(b, bname(b, "nx%d", i));
        y[i] = bcell(b, bname(b, "ny%d", i));
        t[i] = bcell(b, bname(b, "nt%d", i));
        gate1(b, G_BUF, wa[i], a[i]);
        gate1(b, G_BUF, wb[i], bv[i]);
    }
    uint32_t mt = bcell(b, "nm_t");
    for (int pass = 0; pass < 2; pass++) {  /* forward transforms of a and of b */
        uint32_t *w = pass ? wb : wa;
        for (int d = dims - 1; d >= 0; d--) {
            uint32_t id = bcell(b, bname(b, "ID%d", d));
            montmul(b, t, w, zf[d]);  /* z times this machine's value: used above */
            for (int i = 0; i < NQB; i++) {
                snprintf(name, sizeof name, "f%c_a%d_%d", pass ? 'b' : 'a', d, i);
                la[i] = blink(b, name, w[i], d);
                snprintf(name, sizeof name, "f%c_t%d_%d", pass ? 'b' : 'a', d, i);
                lt[i] = blink(b, name, t[i], d);
            }
            mux_bits(b, x, id, la, w, NQB, mt);  /* x = a_u */
            mux_bits(b, y, id, t, lt, NQB, mt);  /* y = z a_v */
            addsub_q(b, w, id, x, y);
        }
    }
    montmul(b, wa, wa, wb);  /* point by point */
    for (int d = 0; d < dims; d++) {  /* back */
        uint32_t id = bcell(b, bname(b, "ID%d", d));
        for (int i = 0; i < NQB; i++) {
            snprintf(name, sizeof name, "ia_a%d_%d", d, i);
            la[i] = blink(b, name, wa[i], d);
        }
        mux_bits(b, x, id, la, wa, NQB, mt);  /* x = a_u */
        mux_bits(b, y, id, wa, la, NQB, mt);  /* y = a_v */
        addsub_q(b, wa, id, x, y);
        montmul(b, wa, wa, zi[d]);
    }
    /* R^2 / N mod q undoes the two 1/R of the point products and the N of the way back */
    uint64_t r2 = (1ull << NQB) % NQ;
    r2 = r2 * r2 % NQ;
    uint64_t ninv = 1, base = (uint64_t)(1u << dims) % NQ;
    for (uint64_t e = NQ - 2; e; e >>= 1, base = base * base % NQ)
        if (e & 1)
            ninv = ninv * base % NQ;
    const_bits(f, r2 * ninv % NQ, NQB);
    montmul(b, c, wa, f);
    for (int i = 0; i < NQB; i++)
        boutput(b, c[i]);
    bfinish(b, p);
}

/* ---- random programs (src/tester.c:57-81) ---------------------------------------------------- */

static void random_fill(Program *p, uint32_t writable, size_t len, uint64_t seed)
{
    p->len = len;
    p->code = tc_xmalloc((len ? len : 1) * sizeof *p->code);
    uint64_t s = seed;
    for (size_t i = 0; i < len; i++) {
        uint64_t r = tc_splitmix64(&s);
        p->code[i].op = (uint8_t)(r & 1);
        p->code[i].addr = p->code[i].op == OP_NAND ? (uint32_t)((r >> 1) % p->ncells)
                                                   : CELL_FIRST_FREE + (uint32_t)((r >> 1) % writable);
    }
}

/* The program `alpha random --cells N --len L --seed S` prints: cells c0.. all declared .out. */
void tc_random_program(Program *p, uint32_t cells, size_t len, uint64_t seed)
{
    memset(p, 0, sizeof *p);
    p->ncells = cells + CELL_FIRST_FREE;
    p->cell_names = tc_xmalloc(p->ncells * sizeof *p->cell_names);
    p->outputs = tc_xmalloc(cells * sizeof *p->outputs);
    p->noutputs = cells;
    for (uint32_t a = 0; a < p->ncells; a++) {
        char name[16];
        if (a == CELL_ZERO)
            snprintf(name, sizeof name, "ZERO");
        else if (a == CELL_ONE)
            snprintf(name, sizeof name, "ONE");
        else
            snprintf(name, sizeof name, "c%u", a - CELL_FIRST_FREE);
        p->cell_names[a] = tc_xstrdup(name);
        if (a >= CELL_FIRST_FREE)
            p->outputs[a - CELL_FIRST_FREE] = a;
    }
    random_fill(p, cells, len, seed);
}

void tc_random_program_in(Program *p, uint32_t cells, uint32_t width, size_t len, uint64_t seed)
{
    memset(p, 0, sizeof *p);
    p->ncells = cells + width + CELL_FIRST_FREE;
    p->cell_names = tc_xmalloc(p->ncells * sizeof *p->cell_names);
    p->outputs = tc_xmalloc((cells + 1) * sizeof *p->outputs);
    p->inputs = tc_xmalloc((width + 1) * sizeof *p->inputs);
    p->noutputs = cells;
    p->ninputs = width;
    for (uint32_t a = 0; a < p->ncells; a++) {
        char name[16];
        if (a == CELL_ZERO)
            snprintf(name, sizeof name, "ZERO");
        else if (a == CELL_ONE)
            snprintf(name, sizeof name, "ONE");
        else if (a < CELL_FIRST_FREE + cells)
            snprintf(name, sizeof name, "c%u", a - CELL_FIRST_FREE);
        else
            snprintf(name, sizeof name, "w%u", a - CELL_FIRST_FREE - cells);
        p->cell_names[a] = tc_xstrdup(name);
        if (a >= CELL_FIRST_FREE && a < CELL_FIRST_FREE + cells)
            p->outputs[a - CELL_FIRST_FREE] = a;
        else if (a >= CELL_FIRST_FREE + cells)
            p->inputs[a - CELL_FIRST_FREE - cells] = a;
    }
    random_fill(p, cells, len, seed);
}

/* ---- rewriting by local NAND identities ---------------------------------------------------- */

typedef struct {
    Instr *code;
    size_t len, cap;
} Code;

static void put(Code *c, int o, uint32_t a)
{
    if (c->len == c->cap) {
        c->cap = c->cap ? 2 * c->cap : 256;
        c->code = tc_xrealloc(c->code, c->cap * sizeof *c->code);
    }
    c->code[c->len].op = (uint8_t)o;
    c->code[c->len].addr = a;
    c->len++;
}

/* Each NAND a, with RR = r before it, may become (chosen per instruction by splitmix64(seed)):
     double negation   NAND ONE; NAND ONE; NAND a
     commuted operands STO t; NAND ZERO; NAND a; NAND ONE; NAND t          = !(a & r)
     De Morgan         STO t; NAND ZERO; NAND a; STO u; NAND ZERO; NAND t;
                       NAND ONE; STO v; NAND u; NAND v                      = !(!r | a) | ... = !(r & a)
   t, u, v are three new cells (__e0..__e2) that each rewrite writes before it reads, so RR and
   every original cell hold the same values as in p after every original instruction. */
void tc_rewrite_program(const Program *p, Program *out, uint64_t seed, int mutate)
{
    tc_program_copy(p, out);
    uint32_t base = p->ncells;
    out->ncells = p->ncells + 3;
    out->cell_names = tc_xrealloc(out->cell_names, out->ncells * sizeof *out->cell_names);
    for (int i = 0; i < 3; i++) {
        char name[16];
        snprintf(name, sizeof name, "__e%d", i);
        out->cell_names[base + (uint32_t)i] = tc_xstrdup(name);
    }
    if (out->special) {
        out->special = tc_xrealloc(out->special, out->ncells * sizeof *out->special);
        memset(out->special + base, 0, 3 * sizeof *out->special);
    }
    uint32_t t = base, u = base + 1, v = base + 2;
    Code c = {0};
    uint64_t s = seed ^ 0xA5A5F00DCAFEull;
    size_t flip = p->len;  /* the negative control changes the last STO: its cell keeps the
                              value it had, which differs for some input unless that STO was
                              redundant */
    for (size_t i = p->len; i-- > 0;)
        if (p->code[i].op == OP_STO) {
            flip = i;
            break;
        }
    for (size_t i = 0; i < p->len; i++) {
        Instr in = p->code[i];
        if (mutate && i == flip)
            in.op = OP_NAND;
        if (in.op != OP_NAND) {
            put(&c, in.op, in.addr);
            continue;
        }
        uint64_t r = tc_splitmix64(&s) % 8;
        if (r == 0) {
            put(&c, OP_NAND, CELL_ONE);
            put(&c, OP_NAND, CELL_ONE);
            put(&c, OP_NAND, in.addr);
        } else if (r == 1) {
            put(&c, OP_STO, t);
            put(&c, OP_NAND, CELL_ZERO);
            put(&c, OP_NAND, in.addr);
            put(&c, OP_NAND, CELL_ONE);
            put(&c, OP_NAND, t);
        } else if (r == 2) {
            put(&c, OP_STO, t);
            put(&c, OP_NAND, CELL_ZERO);
            put(&c, OP_NAND, in.addr);
            put(&c, OP_STO, u);
            put(&c, OP_NAND, CELL_ZERO);
            put(&c, OP_NAND, t);
            put(&c, OP_NAND, CELL_ONE);
            put(&c, OP_STO, v);
            put(&c, OP_NAND, u);
            put(&c, OP_NAND, v);
        } else {
            put(&c, OP_NAND, in.addr);
        }
    }
    free(out->code);
    out->code = c.code;
    out->len = c.len;
}
