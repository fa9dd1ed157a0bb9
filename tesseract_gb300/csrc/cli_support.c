/* What the command-line tool needs beyond the engine's entry points: running one assignment on
   the reference machine to show a counterexample (src/work.c:284-339 re-runs hits on `ref`), and
   `life --dims D`, which like src/work.c:490-701 runs the board on the engine and checks it
   against plain C Life, and `cube DEMO --dims D` (cuda_cube_demo), which like
   src/cubedemo.c:549-623 runs a demo on the cube and checks every machine against plain C. */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "cli_support.h"
#include "engine.h"
#include "ref_host.h"

int cuda_enum_match(const Program *a, const Program *b, int *in_map, int *out_map, char *err,
                    size_t errlen)
{
    Enum e;
    memset(&e, 0, sizeof e);
    e.mode = EN_EQUIV;
    e.a = a;
    e.b = b;
    e.ticks = 1;
    e.parts = 1;
    return tc_enum_prepare(&e, in_map, out_map, err, errlen);
}

/* p from power-on on assignment x (input k = bit n-1-k), `ticks` passes; the outputs */
int tc_run_one(const Program *p, const uint32_t *in_cells, size_t n, uint64_t x, unsigned ticks,
               uint8_t *outs)
{
    TcRef r;
    if (!tc_ref_init(&r, p, 1))
        return 0;
    for (size_t k = 0; k < n; k++)
        if (!tc_program_readonly(p, in_cells[k]))
            r.mem[in_cells[k]] = (uint8_t)((x >> (n - 1 - k)) & 1);
    for (unsigned t = 0; t < ticks; t++)
        tc_ref_tick(&r);
    for (size_t o = 0; o < p->noutputs; o++)
        outs[o] = tc_ref_get(&r, 0, p->outputs[o]);
    tc_ref_free(&r);
    return 1;
}

/* ---- plain C Life, 64 cells a word, for `life`'s check ----------------------------------------- */

typedef struct {
    const uint64_t *cur;
    uint64_t       *next;
    int             w64, h, r0, r1;
} Rows;

static void *rows_step(void *arg)
{
    Rows *R = arg;
    int w = R->w64, h = R->h;
    for (int r = R->r0; r < R->r1; r++) {
        const uint64_t *rows[3] = {R->cur + (size_t)((r + h - 1) % h) * w,
                                   R->cur + (size_t)r * w, R->cur + (size_t)((r + 1) % h) * w};
        for (int k = 0; k < w; k++) {
            uint64_t nb[8];
            int m = 0;
            for (int i = 0; i < 3; i++) {
                uint64_t x = rows[i][k], prev = rows[i][(k + w - 1) % w], nxt = rows[i][(k + 1) % w];
                nb[m++] = (x << 1) | (prev >> 63);
                if (i != 1)
                    nb[m++] = x;
                nb[m++] = (x >> 1) | (nxt << 63);
            }
            /* count in bit planes c0 (1), c1 (2), c2 (4 or more) */
            uint64_t c0 = 0, c1 = 0, c2 = 0;
            for (int i = 0; i < 8; i++) {
                uint64_t t0 = c0 & nb[i];
                c0 ^= nb[i];
                uint64_t t1 = c1 & t0;
                c1 ^= t0;
                c2 |= t1;
            }
            R->next[(size_t)r * w + k] = c1 & ~c2 & (c0 | rows[1][k]);
        }
    }
    return NULL;
}

static void plain_life(uint64_t *board, int w64, int h, unsigned long long gens)
{
    enum { T = 16 };
    uint64_t *tmp = tc_xmalloc((size_t)w64 * h * 8), *cur = board, *nxt = tmp;
    pthread_t tid[T];
    Rows rows[T];
    for (unsigned long long g = 0; g < gens; g++) {
        for (int t = 0; t < T; t++) {
            rows[t] = (Rows){cur, nxt, w64, h, h * t / T, h * (t + 1) / T};
            pthread_create(&tid[t], NULL, rows_step, &rows[t]);
        }
        for (int t = 0; t < T; t++)
            pthread_join(tid[t], NULL);
        uint64_t *s = cur;
        cur = nxt;
        nxt = s;
    }
    if (cur != board)
        memcpy(board, cur, (size_t)w64 * h * 8);
    free(tmp);
}

/* ---- plain C Life, one byte a cell, for boards whose width is not a multiple of 64 ----------- */

static void life_bytes(uint8_t *b, int w, int h, unsigned long long gens)
{
    uint8_t *next = tc_xmalloc((size_t)w * h);
    for (unsigned long long g = 0; g < gens; g++) {
        for (int r = 0; r < h; r++) {
            const uint8_t *up = b + (size_t)((r + h - 1) % h) * w, *row = b + (size_t)r * w,
                          *dn = b + (size_t)((r + 1) % h) * w;
            for (int c = 0; c < w; c++) {
                int l = (c + w - 1) % w, rt = (c + 1) % w;
                int n = up[l] + up[c] + up[rt] + row[l] + row[rt] + dn[l] + dn[c] + dn[rt];
                next[(size_t)r * w + c] = (uint8_t)(n == 3 || (n == 2 && row[c]));
            }
        }
        memcpy(b, next, (size_t)w * h);
    }
    free(next);
}

typedef struct {
    uint8_t           *boards;  /* boards[k * cells ...]: board k, row-major */
    int                w, h, k0, k1;
    unsigned long long gens;
} BoardRange;

static void *boards_step(void *arg)
{
    BoardRange *R = arg;
    for (int k = R->k0; k < R->k1; k++)
        life_bytes(R->boards + (size_t)k * R->w * R->h, R->w, R->h, R->gens);
    return NULL;
}

/* n independent w x h boards, each `gens` generations, on up to 16 host threads */
static void life_many(uint8_t *boards, int n, int w, int h, unsigned long long gens)
{
    enum { T = 16 };
    pthread_t tid[T];
    BoardRange r[T];
    for (int t = 0; t < T; t++) {
        r[t] = (BoardRange){boards, w, h, n * t / T, n * (t + 1) / T, gens};
        pthread_create(&tid[t], NULL, boards_step, &r[t]);
    }
    for (int t = 0; t < T; t++)
        pthread_join(tid[t], NULL);
}

/* `life` (src/work.c:490-701) on the GPU cube engine: 512 independent boards (gen_life, one lane
   each) or one board over the cube (gen_life_cube), seeded from splitmix64 as the reference
   seeds them, run `gens` generations, and checked against plain C Life: every board, or the whole
   board row by row.  Fills what the command prints. */
int tc_life_run(const TcLifeRun *a, TcLifeResult *r, char *err, size_t errlen)
{
    memset(r, 0, sizeof *r);
    r->bad = -1;
    int w = a->size, h = a->size, cells = w * h;
    int dims = a->cube ? a->dims : CUBE_DIMS, rbits = a->cube ? a->rbits : 0;
    int cbits = dims - rbits;
    uint32_t *board = tc_xmalloc((size_t)cells * sizeof *board);
    Program p;
    if (a->cube)
        tc_gen_life_cube(&p, w, h, rbits, cbits, board);
    else
        tc_gen_life(&p, w, h, board);
    r->len = p.len;
    CudaCube *c;
    if (!cuda_cube_new(&p, &c, err, errlen)) {
        free(board);
        tc_program_free(&p);
        return 0;
    }
    r->segments = cuda_cube_segments(c);
    unsigned machines = 1u << dims, W = machines / 32;
    uint32_t *mem = tc_xcalloc((size_t)W * p.ncells, 4), *rr = tc_xcalloc(W, 4);
    uint64_t s = a->seed;  /* group by group, cell by cell, the line's eight 64-bit words */
    for (unsigned g = 0; g < machines / 512; g++)
        for (int i = 0; i < cells; i++)
            for (int k = 0; k < 8; k++) {
                uint64_t v = tc_splitmix64(&s);
                size_t at = (size_t)board[i] * W + (size_t)g * 16 + 2 * (size_t)k;
                mem[at] = (uint32_t)v;
                mem[at + 1] = (uint32_t)(v >> 32);
            }
#define LANE(cell, m) ((mem[(size_t)(cell) * W + ((m) >> 5)] >> ((m) & 31)) & 1u)
    int gw = w << cbits, gh = h << rbits, w64 = (gw + 63) / 64, packed = gw % 64 == 0;
    uint8_t *start = NULL;
    uint64_t *big = NULL;
    if (!a->cube) {
        start = tc_xmalloc((size_t)machines * cells);
        for (unsigned l = 0; l < machines; l++)
            for (int i = 0; i < cells; i++)
                start[(size_t)l * cells + i] = (uint8_t)LANE(board[i], l);
    } else if (packed) {
        big = tc_xcalloc((size_t)w64 * gh, 8);
    } else {
        start = tc_xcalloc((size_t)gw * gh, 1);
    }
    for (int R = 0; a->cube && R < gh; R++)
        for (int C = 0; C < gw; C++) {
            unsigned m = tc_grid_machine((unsigned)(R / h), (unsigned)(C / w), cbits);
            unsigned v = LANE(board[(R % h) * w + C % w], m);
            if (packed)
                big[(size_t)R * w64 + C / 64] |= (uint64_t)v << (C % 64);
            else
                start[(size_t)R * gw + C] = (uint8_t)v;
        }
    int okay = cuda_cube_write_words(c, mem, rr, err, errlen) &&
               cuda_cube_run(c, a->gens, err, errlen) &&
               cuda_cube_read_words(c, mem, rr, err, errlen);
    CudaLaunchStats st;
    cuda_last_launch(&st);
    r->gpu_ms = st.kernel_ms;
    if (okay && !a->cube) {
        life_many(start, (int)machines, w, h, a->gens);
        for (unsigned l = 0; l < machines && r->bad < 0; l++)
            for (int i = 0; i < cells; i++)
                if (start[(size_t)l * cells + i] != LANE(board[i], l)) {
                    r->bad = (int)l;
                    break;
                }
        r->shown = tc_xmalloc((size_t)cells);  /* board 0 as the engine left it */
        for (int i = 0; i < cells; i++) {
            r->shown[i] = (uint8_t)LANE(board[i], 0);
            r->alive += r->shown[i];
        }
    } else if (okay) {
        if (packed)
            plain_life(big, w64, gh, a->gens);
        else
            life_bytes(start, gw, gh, a->gens);
#define PLAIN(R, C) (packed ? (unsigned)((big[(size_t)(R) * w64 + (C) / 64] >> ((C) % 64)) & 1) \
                            : (unsigned)start[(size_t)(R) * gw + (C)])
        for (int R = 0; R < gh && r->bad < 0; R++)
            for (int C = 0; C < gw; C++) {
                unsigned m = tc_grid_machine((unsigned)(R / h), (unsigned)(C / w), cbits);
                if (PLAIN(R, C) != LANE(board[(R % h) * w + C % w], m)) {
                    r->bad = R;
                    break;
                }
            }
        r->rows = gh < 48 ? gh : 48;  /* the top left corner of the plain C board */
        r->cols = gw < 128 ? gw : 128;
        r->shown = tc_xmalloc((size_t)r->rows * r->cols);
        for (int R = 0; R < r->rows; R++)
            for (int C = 0; C < r->cols; C++)
                r->shown[(size_t)R * r->cols + C] = (uint8_t)PLAIN(R, C);
#undef PLAIN
    }
#undef LANE
    r->board_w = gw;
    r->board_h = gh;
    r->machines = machines;
    free(big);
    free(start);
    free(mem);
    free(rr);
    free(board);
    cuda_cube_free(c);
    tc_program_free(&p);
    return okay;
}

/* ---- cube demos over 2^dims machines (src/cubedemo.c:398-623) ------------------------------- */

static void mset(uint32_t *mem, unsigned W, uint32_t cell, unsigned k, unsigned v)
{
    uint32_t *w = &mem[(size_t)cell * W + (k >> 5)];
    *w = (*w & ~(1u << (k & 31))) | ((v & 1u) << (k & 31));
}

static unsigned mget(const uint32_t *mem, unsigned W, uint32_t cell, unsigned k)
{
    return (mem[(size_t)cell * W + (k >> 5)] >> (k & 31)) & 1u;
}

static void vput(uint32_t *mem, unsigned W, const uint32_t *cells, int n, unsigned k, uint64_t x)
{
    for (int b = 0; b < n; b++)
        mset(mem, W, cells[b], k, (unsigned)((x >> b) & 1));
}

static uint64_t vget(const uint32_t *mem, unsigned W, const uint32_t *cells, int n, unsigned k)
{
    uint64_t x = 0;
    for (int b = 0; b < n; b++)
        x |= (uint64_t)mget(mem, W, cells[b], k) << b;
    return x;
}

static int cmp_u64(const void *a, const void *b)
{
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : x > y;
}

static int find_cells(const Program *p, const char *stem, int n, uint32_t *cells)
{
    for (int i = 0; i < n; i++) {
        char name[32];
        snprintf(name, sizeof name, "%s%d", stem, i);
        if (!tc_program_find_cell(p, name, &cells[i]))
            return 0;
    }
    return 1;
}

/* polymul's numbers mod q = 12289: x^e */
static uint64_t pow_q(uint64_t x, uint64_t e)
{
    uint64_t r = 1;
    for (x %= 12289; e; e >>= 1, x = x * x % 12289)
        if (e & 1)
            r = r * x % 12289;
    return r;
}

/* polymul's inputs: random a and b in 0 .. q-1, and the twiddles of each round in Montgomery
   form (times R = 2^14): round d pairs machines u, u + 2^d with the zeta psi^brv(2^(dims-1-d) +
   u >> (d + 1)) of the usual in-place loop, psi a primitive 2N-th root of unity; the way back
   multiplies the upper machine by 1/zeta.  want gets the product by schoolbook. */
static void polymul_inputs(const Program *p, int dims, uint32_t *mem, unsigned W, uint64_t *s,
                           uint64_t *want)
{
    const uint64_t q = 12289, R = (1u << 14) % q;
    unsigned n = 1u << dims;
    uint64_t g = 2;
    while (pow_q(g, (q - 1) / 2) == 1 || pow_q(g, (q - 1) / 3) == 1)
        g++;
    uint64_t psi = pow_q(g, (q - 1) / (2 * (uint64_t)n));
    uint32_t a[14], b[14], z[14];
    find_cells(p, "a", 14, a);
    find_cells(p, "b", 14, b);
    uint64_t *x = tc_xmalloc((size_t)n * 8), *y = tc_xmalloc((size_t)n * 8);
    for (unsigned k = 0; k < n; k++) {
        vput(mem, W, a, 14, k, x[k] = tc_splitmix64(s) % q);
        vput(mem, W, b, 14, k, y[k] = tc_splitmix64(s) % q);
    }
    for (int d = 0; d < dims; d++)
        for (int inv = 0; inv < 2; inv++) {
            char stem[16];
            snprintf(stem, sizeof stem, "%s%d_", inv ? "zi" : "zf", d);
            find_cells(p, stem, 14, z);
            for (unsigned k = 0; k < n; k++) {
                unsigned idx = (1u << (dims - 1 - d)) + (k >> (d + 1)), rev = 0;
                for (int i = 0; i < dims; i++)
                    rev |= ((idx >> i) & 1) << (dims - 1 - i);
                uint64_t zeta = pow_q(psi, rev), v;
                if (!inv)
                    v = zeta * R % q;
                else
                    v = (k >> d) & 1 ? pow_q(zeta, q - 2) * R % q : R;
                vput(mem, W, z, 14, k, v);
            }
        }
    for (unsigned k = 0; k < n; k++)
        want[k] = 0;
    for (unsigned i = 0; i < n; i++)  /* x^N = -1 */
        for (unsigned j = 0; j < n; j++) {
            uint64_t t = x[i] * y[j] % q;
            unsigned at = (i + j) % n;
            want[at] = (want[at] + (i + j < n ? t : q - t)) % q;
        }
    free(x);
    free(y);
}

/* h(k) = how many j have f(j) = g(j ^ k) = 1, f in bit 0 and g in bit 1 of fg[j]: the sum
   itself up to 2^12 machines, beyond that through the integer Walsh-Hadamard transform
   (exact: the transform of h is the product of those of f and g). */
static uint64_t *xor_convolution(const uint64_t *fg, int dims)
{
    unsigned n = 1u << dims;
    uint64_t *h = tc_xcalloc(n, sizeof *h);
    if (dims <= 12) {
        for (unsigned k = 0; k < n; k++)
            for (unsigned j = 0; j < n; j++)
                h[k] += fg[j] & fg[j ^ k] >> 1 & 1;
        return h;
    }
    int64_t *a = tc_xmalloc((size_t)n * sizeof *a), *b = tc_xmalloc((size_t)n * sizeof *b);
    for (unsigned k = 0; k < n; k++) {
        a[k] = (int64_t)(fg[k] & 1);
        b[k] = (int64_t)(fg[k] >> 1);
    }
    for (int pass = 0; pass < 2; pass++) {
        for (unsigned d = 1; d < n; d <<= 1)
            for (unsigned k = 0; k < n; k++)
                if (!(k & d)) {
                    int64_t u = a[k], v = a[k | d];
                    a[k] = u + v;
                    a[k | d] = u - v;
                    if (!pass) {
                        u = b[k], v = b[k | d];
                        b[k] = u + v;
                        b[k | d] = u - v;
                    }
                }
        if (!pass)
            for (unsigned k = 0; k < n; k++)
                a[k] *= b[k];
    }
    for (unsigned k = 0; k < n; k++)
        h[k] = (uint64_t)(a[k] >> dims);
    free(a);
    free(b);
    return h;
}

int cuda_cube_demo(const char *name, int dims, int checks, double seconds, CudaDemoResult *r,
                   char *err, size_t errlen)
{
    memset(r, 0, sizeof *r);
    if (dims < CUBE_DIMS || dims > CUBE_MAX_DIMS)
        return tc_fail(err, errlen, "--dims must be %d to %d", CUBE_DIMS, CUBE_MAX_DIMS);
    unsigned n = 1u << dims, W = n / 32;
    Program p;
    uint32_t *board = NULL;
    int rbits = dims / 2, cbits = dims - rbits, T = 32;
    if (!strcmp(name, "any")) {
        snprintf(r->what, sizeof r->what, "OR of one bit over all %u machines", n);
        tc_gen_cube_any(&p, dims);
    } else if (!strcmp(name, "rank")) {
        snprintf(r->what, sizeof r->what, "running count of %u bits, %d-bit results", n, dims + 1);
        tc_gen_cube_rank(&p, dims);
    } else if (!strcmp(name, "sort")) {
        snprintf(r->what, sizeof r->what, "sort %u bytes (bitonic, %d rounds)", n,
                 dims * (dims + 1) / 2);
        tc_gen_cube_sort(&p, dims);
    } else if (!strcmp(name, "max")) {
        snprintf(r->what, sizeof r->what, "largest of %u bytes", n);
        tc_gen_cube_max(&p, dims);
    } else if (!strcmp(name, "pack")) {
        snprintf(r->what, sizeof r->what, "gather the bytes of the machines with a hit");
        tc_gen_cube_pack(&p, dims);
    } else if (!strcmp(name, "xorconv")) {
        snprintf(r->what, sizeof r->what, "h(k) = #x: f(x) = g(x^k) = 1, by spectra");
        tc_gen_cube_xorconv(&p, dims);
    } else if (!strcmp(name, "anf")) {
        snprintf(r->what, sizeof r->what, "truth table of %d inputs -> normal form (M\xc3\xb6" "bius)", dims);
        tc_gen_cube_anf(&p, dims);
    } else if (!strcmp(name, "walsh")) {
        snprintf(r->what, sizeof r->what, "Walsh-Hadamard spectrum of f, %d-bit results", dims + 3);
        tc_gen_cube_walsh(&p, dims);
    } else if (!strcmp(name, "ring")) {
        snprintf(r->what, sizeof r->what, "Rule 110 on a ring of %u cells, one step", n);
        tc_gen_cube_ring(&p, dims);
    } else if (!strcmp(name, "polymul")) {
        if (dims > 11)
            return tc_fail(err, errlen, "polymul needs a 2N-th root of unity mod 12289: dims 9..11");
        snprintf(r->what, sizeof r->what, "c = a * b in Z_12289[x]/(x^%u + 1), by NTT", n);
        tc_gen_cube_polymul(&p, dims);
    } else if (!strcmp(name, "life")) {
        snprintf(r->what, sizeof r->what, "Life: one %d x %d board, one generation", T << rbits,
                 T << cbits);
        board = tc_xmalloc((size_t)T * T * sizeof *board);
        tc_gen_life_cube(&p, T, T, rbits, cbits, board);
    } else {
        return tc_fail(err, errlen, "unknown demo '%s' (any, rank, max, sort, pack, anf, walsh, "
                       "xorconv, ring, polymul, life)", name);
    }
    r->instr = p.len;
    CudaCube *c;
    if (!cuda_cube_new(&p, &c, err, errlen)) {
        free(board);
        tc_program_free(&p);
        return 0;
    }
    r->segs = cuda_cube_segments(c);
    r->kernels = cuda_cube_kernels(c);
    uint32_t *mem = tc_xcalloc((size_t)W * p.ncells, 4), *rr = tc_xcalloc(W, 4);
    uint64_t *want = tc_xcalloc((size_t)n + 1, 8), s = 42;
    uint32_t x[CUBE_MAX_DIMS + 2], pv[CUBE_MAX_DIMS + 2], tv[CUBE_MAX_DIMS + 2];
    int okay = 1, ok = 1, rounds = !strcmp(name, "life") && checks > 2 ? 2 : checks;
    int gw = T << cbits, gh = T << rbits, w64 = gw / 64;
    uint64_t *big = board ? tc_xcalloc((size_t)w64 * gh, 8) : NULL;
    for (int round = 0; round < rounds && ok && okay; round++) {
        /* power-on state (src/lanes.c:176-192): cells 0, ONE 1, RR 0; then the inputs */
        memset(mem, 0, (size_t)W * p.ncells * 4);
        memset(rr, 0, (size_t)W * 4);
        for (unsigned w = 0; w < W; w++)
            mem[(size_t)CELL_ONE * W + w] = 0xffffffffu;
        unsigned one = 0;
        uint64_t count = 0;
        if (!strcmp(name, "any")) {
            tc_program_find_cell(&p, "x", &x[0]);
            one = (unsigned)(tc_splitmix64(&s) % (2ull * n));  /* sometimes none */
            for (unsigned k = 0; k < n; k++)
                mset(mem, W, x[0], k, k == one);
        } else if (!strcmp(name, "rank")) {
            tc_program_find_cell(&p, "x", &x[0]);
            for (unsigned k = 0; k < n; k++) {
                unsigned v = tc_splitmix64(&s) % 10 < 3;
                mset(mem, W, x[0], k, v);
                want[k] = count;
                count += v;
            }
        } else if (!strcmp(name, "sort")) {
            find_cells(&p, "v", 8, x);
            for (unsigned k = 0; k < n; k++)
                vput(mem, W, x, 8, k, want[k] = tc_splitmix64(&s) & 255);
            qsort(want, n, sizeof *want, cmp_u64);
        } else if (!strcmp(name, "max")) {
            find_cells(&p, "v", 8, x);
            count = 0;  /* the largest */
            for (unsigned k = 0; k < n; k++) {
                uint64_t v = tc_splitmix64(&s) & 255;
                vput(mem, W, x, 8, k, v);
                count = v > count ? v : count;
            }
        } else if (!strcmp(name, "pack")) {
            find_cells(&p, "v", 8, x);
            tc_program_find_cell(&p, "h", &x[8]);
            for (unsigned k = 0; k < n; k++) {  /* want: the bytes of the hits, in order */
                uint64_t v = tc_splitmix64(&s) & 255, hit = tc_splitmix64(&s) % 10 == 0;
                vput(mem, W, x, 8, k, v);
                mset(mem, W, x[8], k, (unsigned)hit);
                if (hit)
                    want[count++] = v;
            }
        } else if (!strcmp(name, "xorconv")) {
            tc_program_find_cell(&p, "f", &x[0]);
            tc_program_find_cell(&p, "g", &x[1]);
            for (unsigned k = 0; k < n; k++) {  /* want: f in bit 0, g in bit 1 */
                want[k] = tc_splitmix64(&s) & 3;
                mset(mem, W, x[0], k, (unsigned)(want[k] & 1));
                mset(mem, W, x[1], k, (unsigned)(want[k] >> 1));
            }
        } else if (!strcmp(name, "anf") || !strcmp(name, "walsh")) {
            tc_program_find_cell(&p, "f", &x[0]);
            for (unsigned k = 0; k < n; k++)
                mset(mem, W, x[0], k, (unsigned)(want[k] = tc_splitmix64(&s) & 1));
        } else if (!strcmp(name, "ring")) {
            tc_program_find_cell(&p, "x", &x[0]);
            for (unsigned k = 0; k < n; k++)
                mset(mem, W, x[0], k, (unsigned)(want[k] = tc_splitmix64(&s) & 1));
        } else if (!strcmp(name, "polymul")) {
            polymul_inputs(&p, dims, mem, W, &s, want);
        } else {
            memset(big, 0, (size_t)w64 * gh * 8);
            for (int R = 0; R < gh; R++)
                for (int C = 0; C < gw; C++) {
                    unsigned v = tc_splitmix64(&s) % 3 == 0;
                    unsigned m = tc_grid_machine((unsigned)(R / T), (unsigned)(C / T), cbits);
                    mset(mem, W, board[(R % T) * T + C % T], m, v);
                    if (v)
                        big[(size_t)R * w64 + C / 64] |= 1ull << (C % 64);
                }
            plain_life(big, w64, gh, 1);
        }
        okay = cuda_cube_write_words(c, mem, rr, err, errlen) && cuda_cube_run(c, 1, err, errlen) &&
               cuda_cube_read_words(c, mem, rr, err, errlen);
        if (!okay)
            break;
        if (!strcmp(name, "any")) {
            uint32_t rc;
            tc_program_find_cell(&p, "r", &rc);
            for (unsigned k = 0; k < n && ok; k++)
                ok = mget(mem, W, rc, k) == (one < n);
        } else if (!strcmp(name, "rank")) {
            find_cells(&p, "p", dims + 1, pv);
            find_cells(&p, "t", dims + 1, tv);
            for (unsigned k = 0; k < n && ok; k++)
                ok = vget(mem, W, pv, dims + 1, k) == want[k] &&
                     vget(mem, W, tv, dims + 1, k) == count;
        } else if (!strcmp(name, "sort")) {
            for (unsigned k = 0; k < n && ok; k++)
                ok = vget(mem, W, x, 8, k) == want[k];
        } else if (!strcmp(name, "max")) {
            find_cells(&p, "m", 8, pv);
            for (unsigned k = 0; k < n && ok; k++)
                ok = vget(mem, W, pv, 8, k) == count;
        } else if (!strcmp(name, "pack")) {
            for (unsigned k = 0; k < n && ok; k++)
                ok = mget(mem, W, x[8], k) == (k < count) &&
                     (k >= count || vget(mem, W, x, 8, k) == want[k]);
        } else if (!strcmp(name, "xorconv")) {
            uint64_t *h = xor_convolution(want, dims);
            find_cells(&p, "h", dims + 1, pv);
            for (unsigned k = 0; k < n && ok; k++)
                ok = vget(mem, W, pv, dims + 1, k) == h[k];
            free(h);
        } else if (!strcmp(name, "anf")) {
            for (unsigned d = 1; d < n; d <<= 1)  /* the Mobius transform in plain C */
                for (unsigned k = 0; k < n; k++)
                    if (k & d)
                        want[k] ^= want[k ^ d];
            for (unsigned k = 0; k < n && ok; k++)
                ok = mget(mem, W, x[0], k) == want[k];
        } else if (!strcmp(name, "walsh")) {
            /* the spectrum in plain C: the fast transform on integers */
            int64_t *a = tc_xmalloc((size_t)n * sizeof *a);
            for (unsigned k = 0; k < n; k++)
                a[k] = want[k] ? -1 : 1;
            for (unsigned d = 1; d < n; d <<= 1)
                for (unsigned k = 0; k < n; k++)
                    if (!(k & d)) {
                        int64_t u = a[k], v = a[k | d];
                        a[k] = u + v;
                        a[k | d] = u - v;
                    }
            find_cells(&p, "w", dims + 3, pv);
            for (unsigned k = 0; k < n && ok; k++)
                ok = vget(mem, W, pv, dims + 3, k) == ((uint64_t)a[k] & ((1ull << (dims + 3)) - 1));
            free(a);
        } else if (!strcmp(name, "polymul")) {
            find_cells(&p, "c", 14, pv);
            for (unsigned k = 0; k < n && ok; k++)
                ok = vget(mem, W, pv, 14, k) == want[k];
        } else if (!strcmp(name, "ring")) {
            uint64_t *nx = tc_xmalloc((size_t)n * sizeof *nx);
            for (unsigned i = 0; i < n; i++) {  /* Rule 110, position i at machine gray(i) */
                unsigned l = tc_grid_machine(0, (i + n - 1) % n, dims),
                         c = tc_grid_machine(0, i, dims), rt = tc_grid_machine(0, (i + 1) % n, dims);
                nx[c] = (110u >> ((want[l] << 2) | (want[c] << 1) | want[rt])) & 1;
            }
            for (unsigned k = 0; k < n && ok; k++)
                ok = mget(mem, W, x[0], k) == nx[k];
            free(nx);
        } else {
            for (int R = 0; R < gh && ok; R++)
                for (int C = 0; C < gw && ok; C++) {
                    unsigned m = tc_grid_machine((unsigned)(R / T), (unsigned)(C / T), cbits);
                    ok = mget(mem, W, board[(R % T) * T + C % T], m) ==
                         ((big[(size_t)R * w64 + C / 64] >> (C % 64)) & 1);
                }
        }
    }
    r->ok = ok;
    /* timing: double the passes until a run takes a quarter of `seconds` */
    for (uint64_t passes = 1; okay; passes *= 2) {
        double t0 = tc_now();
        okay = cuda_cube_run(c, passes, err, errlen) && cuda_cube_read_words(c, mem, rr, err, errlen);
        double t = tc_now() - t0;
        if (t > seconds / 4 || passes >= (1ull << 30)) {
            CudaLaunchStats st;
            cuda_last_launch(&st);
            r->pass_seconds = st.kernel_ms / 1e3 / (double)passes;
            r->passes_per_second = 1.0 / r->pass_seconds;
            break;
        }
    }
    free(big);
    free(want);
    free(mem);
    free(rr);
    free(board);
    cuda_cube_free(c);
    tc_program_free(&p);
    return okay;
}
