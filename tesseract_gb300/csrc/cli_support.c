/* What the command-line tool needs beyond the engine's entry points: running one assignment on
   the reference machine to show a counterexample (src/work.c:284-339 re-runs hits on `ref`), and
   `life --dims D`, which like src/work.c:490-701 runs the board on the engine and checks it
   against plain C Life. */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

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

int tc_life_cube_run(int dims, int rbits, int size, unsigned long long gens, uint64_t seed,
                     double *gpu_ms, int check, int *ok, char *err, size_t errlen)
{
    int cbits = dims - rbits, w = size, h = size, cells = w * h;
    uint32_t *board = tc_xmalloc((size_t)cells * sizeof *board);
    Program p;
    tc_gen_life_cube(&p, w, h, rbits, cbits, board);
    CudaCube *c;
    if (!cuda_cube_new(&p, &c, err, errlen)) {
        free(board);
        tc_program_free(&p);
        return 0;
    }
    unsigned machines = 1u << dims, W = machines / 32;
    uint32_t *mem = tc_xcalloc((size_t)W * p.ncells, 4), *rr = tc_xcalloc(W, 4);
    uint64_t s = seed;
    for (unsigned g = 0; g < machines / 512; g++)
        for (int i = 0; i < cells; i++)
            for (int k = 0; k < 8; k++) {
                uint64_t v = tc_splitmix64(&s);
                size_t at = (size_t)board[i] * W + (size_t)g * 16 + 2 * (size_t)k;
                mem[at] = (uint32_t)v;
                mem[at + 1] = (uint32_t)(v >> 32);
            }
    int gw = w << cbits, gh = h << rbits, w64 = (gw + 63) / 64;
    uint64_t *big = NULL;
    if (check) {
        big = tc_xcalloc((size_t)w64 * gh, 8);
        for (int R = 0; R < gh; R++)
            for (int C = 0; C < gw; C++) {
                unsigned m = tc_grid_machine((unsigned)(R / h), (unsigned)(C / w), cbits);
                uint32_t cell = board[(R % h) * w + C % w];
                if ((mem[(size_t)cell * W + (m >> 5)] >> (m & 31)) & 1)
                    big[(size_t)R * w64 + C / 64] |= 1ull << (C % 64);
            }
    }
    int okay = cuda_cube_write_words(c, mem, rr, err, errlen) &&
               cuda_cube_run(c, gens, err, errlen) &&
               cuda_cube_read_words(c, mem, rr, err, errlen);
    CudaLaunchStats st;
    cuda_last_launch(&st);
    *gpu_ms = st.kernel_ms;
    *ok = 1;
    if (okay && check && gw % 64 == 0) {
        plain_life(big, w64, gh, gens);
        for (int R = 0; R < gh && *ok; R++)
            for (int C = 0; C < gw; C++) {
                unsigned m = tc_grid_machine((unsigned)(R / h), (unsigned)(C / w), cbits);
                uint32_t cell = board[(R % h) * w + C % w];
                unsigned got = (mem[(size_t)cell * W + (m >> 5)] >> (m & 31)) & 1;
                unsigned want = (big[(size_t)R * w64 + C / 64] >> (C % 64)) & 1;
                if (got != want) {
                    *ok = 0;
                    break;
                }
            }
    }
    free(big);
    free(mem);
    free(rr);
    free(board);
    cuda_cube_free(c);
    tc_program_free(&p);
    return okay;
}
